/*
 * femgpu.h -- C ABI of the GB300 (sm_103a) steady 2D stabilised-FEM solve loop.
 *
 * Drop-in for the hot path of mod-comp-ufes/FEM_CODES: the element build, the
 * EBE/EDE/CSR storage and matvecs, ILU(0)/diagonal preconditioning and the
 * restarted GMRES of 00_CommonFiles.  The reference binds these through
 * function pointers with struct arguments (FemFunctionsType /
 * FemOtherFunctionsType, 01_SS_Transport_Equation/2D/01_CommonFiles/
 * SSTranspEquation.h:97-121); this ABI exposes the same operations with plain
 * pointers and sizes, so a thin shim assigns them to those pointers (the shims
 * for the transport, Euler and Navier-Stokes drivers are in
 * fem_codes_gb300/shims/).  Every
 * entry point returns 0 or a negative FEMGPU_E* code;
 * none aborts the process and none traps the GPU.
 *
 * Host-buffer entry points (no suffix) take arrays in host memory laid out
 * exactly as the reference holds them (length neq+1 vectors, slot neq being the
 * dump for prescribed dofs) and copy across the boundary.  *_dev entry points
 * take device pointers and run on the context's stream without host
 * synchronisation.
 */
#ifndef FEMGPU_H
#define FEMGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------- */
#define FEMGPU_OK                 0
#define FEMGPU_E_ARG             -1   /* bad argument / option                 */
#define FEMGPU_E_CUDA            -2   /* CUDA runtime error                    */
#define FEMGPU_E_NOMEM           -3   /* device allocation failed              */
#define FEMGPU_E_ZERO_PIVOT      -4   /* ILU zero pivot (ILUp_precond_setup.c:154-163) */
#define FEMGPU_E_NOT_CONVERGED   -5   /* GMRES hit its restart limit           */
#define FEMGPU_E_BREAKDOWN       -6   /* GMRES zero/NaN norm (pgmres.c:85,121) */
#define FEMGPU_E_TIMEOUT         -7   /* a device wait exceeded its bound      */
#define FEMGPU_E_MESH            -8   /* mesh/structure unsupported            */
#define FEMGPU_E_NOT_BUILT       -9   /* call order (Build before solve, ...)  */

/* ---- options (the reference's parameter-deck strings, Preprocess.c:44-62) */
enum femgpu_scheme   { FEMGPU_EBE = 0, FEMGPU_EDE = 1, FEMGPU_CSR = 2 };
enum femgpu_reorder  { FEMGPU_REORDER_NOT = 0, FEMGPU_REORDER_SYMRCM = 1 };
enum femgpu_precond  { FEMGPU_PREC_NOT = 0, FEMGPU_PREC_ILU0 = 1, FEMGPU_PREC_DIAG = 2,
                       FEMGPU_PREC_BLOCKDIAG = 3, /* Euler: nodal 4x4 blocks            */
                       FEMGPU_PREC_LEARNED = 4,   /* graph network, ILU(0) fallback    */
                       FEMGPU_PREC_AMG = 5        /* DPA AMG V-cycle (femgpu_amg)      */ };
enum femgpu_shock    { FEMGPU_SHOCK_CAU = 0, FEMGPU_SHOCK_YZBETA = 1,
                       FEMGPU_SHOCK_CAUDD = 2      /* transient DD builds only          */ };
enum femgpu_hshock   { FEMGPU_H_2SQRTAREA = 0, FEMGPU_H_SQRTAREA = 1,
                       FEMGPU_H_OPTION1 = 2, FEMGPU_H_OPTION2 = 3 };
/* Arithmetic of the solve (FGMRES only): FP64 throughout (the reference's);
 * MIXED: preconditioner in FP32, operator and Arnoldi in FP64; MIXED_IR:
 * FP32 operator and preconditioner inside FP64 iterative refinement of the
 * outer residual (CSR storage for both mixed modes). */
enum femgpu_precision { FEMGPU_FP64 = 0, FEMGPU_MIXED = 1, FEMGPU_MIXED_IR = 2 };
/* Krylov solver: the reference's left-preconditioned GMRES, which stops on
 * ||M^-1 r|| <= tol ||M^-1 b|| (pgmres.c:49-53,184), or flexible GMRES with
 * right preconditioning, which stops on the unpreconditioned residual
 * ||b - A x|| <= tol ||b|| and leaves F unpreconditioned. */
enum femgpu_solver { FEMGPU_PGMRES = 0, FEMGPU_FGMRES = 1 };

typedef struct femgpu_transport_opts {
	int scheme;          /* femgpu_scheme        (MatrixVectorProductScheme) */
	int reorder;         /* femgpu_reorder       (reordering)                */
	int precond;         /* femgpu_precond       (Preconditioner)            */
	int shock;           /* femgpu_shock         (ShockCapture)              */
	int hshock;          /* femgpu_hshock        (h_Shock)                   */
	int outflow;         /* OutputFlow == YES                                */
	int kmax;            /* KrylovBasisVectorsQuantity                       */
	int lmax;            /* SolverMaxIter (restart cycles, pgmres.c:15)      */
	double tol;          /* SolverTolerance                                  */
	double nonlin_tol;   /* NonLinearTolerance                               */
	int precision;       /* femgpu_precision                                 */
	int ir_max;          /* mixed precision: max refinement sweeps           */
	int solver;          /* femgpu_solver                                    */
	double inner_tol;    /* mixed precision: relative tolerance of each FP32 */
	                     /* inner solve inside the FP64 refinement           */
	double stall_ratio;  /* learned preconditioner: fall back to ILU(0) when */
	                     /* a restart cycle leaves rho > stall_ratio * rho0  */
	int ilu_blocks;      /* 0: ILU(0) of the whole matrix (the reference's); */
	                     /* P > 1: block ILU(0) over P contiguous row blocks */
	                     /* of the numbering, couplings between blocks       */
	                     /* dropped, one thread block per matrix block       */
	int ilu_level;       /* level of fill p of FEMGPU_PREC_ILU0 -- the deck's */
	                     /* "ILU<p>" (ILUp_precond_setup.c:15): 0 ILU(0),    */
	                     /* p > 0 ILU(p) on LEVEL_OF_FILL_lu's pattern       */
} femgpu_transport_opts;

void femgpu_transport_default_opts(femgpu_transport_opts *o);

/* Opaque device-resident problem: mesh, numbering, storage pattern, matrix,
 * preconditioner and Krylov workspace.  Replaces the storage the reference
 * keeps in MatrixDataType / FemStructsType (SSTranspEquation.h:64-95). */
typedef struct femgpu_transport femgpu_transport;

/* Preprocess (Preprocess.c:160-237): numbering (id = neq++ for Type >= 1),
 * Fill_LM, and the storage pattern -- csr_Initialization (+ SYMRCM
 * reordering), ede_Initialization or EBE allocation -- built on the device.
 *   x, y       [nnodes]   node coordinates
 *   node_type  [nnodes]   reference node Type (>= 1 unknown, 0 prescribed)
 *   vert       [3*nel]    element vertices (0-based)
 *   k, gamma              conductivity and reaction (Condutivity(), Reaction())
 *   beta       [2*nel]    velocity at each element centroid (Velocity(XB,YB))
 *   fsrc       [3*nel]    source at the element's vertices (Font(...))
 *   upresc     [nnodes]   prescribed value at each node (upresc(x,y))
 * beta/fsrc may be NULL when const_beta/fsrc-zero apply: pass beta == NULL with
 * const_beta non-NULL (2 doubles) for a constant velocity, fsrc == NULL for f=0. */
int femgpu_transport_create(femgpu_transport **ctx, const femgpu_transport_opts *opts,
		int nnodes, const double *x, const double *y, const int *node_type,
		int nel, const int *vert, double k, double gamma,
		const double *beta, const double *const_beta, const double *fsrc,
		const double *upresc);
void femgpu_transport_destroy(femgpu_transport *ctx);

/* Bind the context to a CUDA stream (cudaStream_t passed as void*; NULL = the
 * context's own stream). */
int femgpu_transport_set_stream(femgpu_transport *ctx, void *stream);

/* Sizes: info[0]=neq, [1]=nnzero, [2]=nedge, [3]=bandwidth after reordering,
 * [4]=ILU levels (L), [5]=ILU levels (U), [6]=1 (2) when the last learned-
 * preconditioned solve fell back to ILU(0) (to AMG) (7 ints). */
int femgpu_transport_info(const femgpu_transport *ctx, int *info);

/* Block ILU(0) (opts.ilu_blocks = P > 1) drops the couplings between P
 * contiguous row runs of the (reordered) numbering, cut at equal spans of the
 * full factor's dependency levels (FEMGPU_ILU_BLOCK_CUT=depth: the shallowest
 * deepest run; =rows: equal row counts).  Returns the
 * number of runs (1: global ILU(0)) and, when first != NULL, writes the first
 * row of each run and the row count (runs + 1 ints; cap = room in first).
 * FEMGPU_E_NOT_BUILT before the ILU(0) structure exists (CSR + ILU0 only). */
int femgpu_transport_ilu_blocks(const femgpu_transport *ctx, int *first, int cap);

/* 1 when the context's ILU(0) has chain-scan programs -- which its FGMRES
 * (fused-arithmetic) and FP32 sweeps then run: rows chained to their sweep
 * predecessor solved 32 at a time by a warp scan, results equal to the
 * row-by-row sweeps to rounding -- else 0 (too few chained rows; the
 * reference's GMRES always runs the bit-identical row-by-row sweeps).
 * levels [2] (may be NULL) receives their level counts (forward, backward).
 * FEMGPU_E_NOT_BUILT before the ILU(0) structure exists. */
int femgpu_transport_ilu_chain(const femgpu_transport *ctx, int *levels);

/* Bound, in spins, on a sweep warp's wait for the rows its own rows depend
 * on (spins < 0: the default, 2^24); a warp that gives up records
 * FEMGPU_E_TIMEOUT, the other warps of its block stop, the block waits for
 * the copies it has in flight (that wait keeps the default bound) and
 * returns, and the call reports the error.  0 makes every sweep time out at
 * its first dependent row, the way a test reaches the error path.  Also
 * clears the context's device error word, so the context is usable again. */
int femgpu_transport_set_sweep_wait(femgpu_transport *ctx, int spins);

/* The same cut for a CSR pattern on the host, no device needed: returns the
 * number of runs R = max(min(P, n), 1) and writes R + 1 row boundaries to
 * first (cap = room in first; FEMGPU_E_ARG when cap < R + 1).  The pattern
 * must have IA[0] = 0, non-decreasing IA, columns in 0..n-1 and strictly
 * ascending columns in every row; anything else returns FEMGPU_E_ARG. */
int femgpu_ilu_block_cut(int n, const int *IA, const int *JA, int P, int *first, int cap);

/* The chain-scan segmentation of one ILU(0) sweep (lower != 0: forward) of a
 * CSR pattern with the block cut of P, on the host, no device needed: rows
 * of a matrix block in sweep order are grouped into segments of up to 32,
 * each row after a segment's first depending on its predecessor (the
 * recurrence a warp scan solves), segments get dependency levels and each
 * level's segments are packed into 32-slot chunks.  Returns the slot count
 * (padding included) and info[4] = {levels, deepest block's segment levels,
 * deepest block's row levels, most dependencies of a row besides its
 * predecessor}; when the arrays are given (room: cap_slots, cap_levels),
 * slot_row [slots] (-1 padding), slot_pred [slots] (CSR position of the row's
 * coupling to its predecessor, -1 at a segment start) and lstart [levels+1]
 * (first slot of each level).  Same pattern checks as femgpu_ilu_block_cut. */
int femgpu_ilu_chain_segments(int n, const int *IA, const int *JA, int P, int lower, int *info,
		int *slot_row, int *slot_pred, int *lstart, int cap_slots, int cap_levels);

/* Copies of the device-built structure, for parity checks against the
 * reference (IA [neq+1], JA [nnz], CSR_by_Element [9*nel]; EDE: lm2 [2*nedge],
 * EDGE_by_Element [3*nel], order [3*nel]; node ids [nnodes]). NULL skips. */
int femgpu_transport_get_pattern(const femgpu_transport *ctx, int *IA, int *JA, int *sbe,
		int *order, int *node_id);

/* Build (Build_K_F_SUPG.c:5-163 through FemOtherFunctions->Build): element
 * matrices + RHS from the current u.  u_host [neq+1] (NULL = use the device
 * copy, i.e. the last solution), F_host [neq+1] receives F (NULL skips).
 * A_host receives the matrix storage when non-NULL (EBE 9*nel, EDE
 * 4*(nedge+1), CSR nnz+1). */
int femgpu_transport_build(femgpu_transport *ctx, const double *u_host, double *F_host,
		double *A_host);

/* precond_setup (e.g. ILUp_precond_setup.c:8-60): factor, then F := M^-1 F
 * in place on the device copy of F; F_host [neq+1] receives it when non-NULL. */
int femgpu_transport_precond_setup(femgpu_transport *ctx, int tag, double *F_host);

/* precond (ILUp_precond.c, Diag_precond.c): z = M^-1 p; p may equal z. */
int femgpu_transport_precond(femgpu_transport *ctx, const double *p_host, double *z_host);

/* ProductMatrixVector (csrmv.c / ebemv.c / edemv.c): Q = A P, P[neq] and
 * Q[neq] set to 0 as the EBE/EDE products do. */
int femgpu_transport_matvec(femgpu_transport *ctx, const double *P_host, double *Q_host);

/* solver (pgmres.c:4-211, 4-argument steady-transport form): B = the device
 * F (already preconditioned by precond_setup), X = the device u.  X_host
 * [neq+1] receives u when non-NULL; iters receives the inner iterations. */
int femgpu_transport_solve(femgpu_transport *ctx, double *X_host, int *iters);

/* 6-argument pgmres form (Euler/NS solver pointer, EulerEquations.h:168):
 * B_host, X_host [neq+1] in host memory. B is not modified. */
int femgpu_transport_solve_bx(femgpu_transport *ctx, const double *B_host, double *X_host,
		int *iters);

/* Process (Process.c:276-335): Picard iterations Build -> precond_setup ->
 * solver until max|u - u_old| <= NonLinearTolerance or npicard iterations.
 * u_hist [npicard*(neq+1)] and iters [npicard] receive each iterate (NULL
 * skips). Returns the number of Picard iterations run (> 0) or an error. */
int femgpu_transport_process(femgpu_transport *ctx, int npicard, double *u_hist, int *iters);

/* ---- transient scalar transport (02_Transport_Equation/2D) ----------------
 * A transport context switched to the transient driver: its Build is
 * Build_M_K_R_SUPG (Build_M_K_R_SUPG.c:6-183) or Build_M_K_R_DD
 * (Build_M_K_R_DD.c:6-191, with its per-element shock-parameter state) --
 * the storage gets Ae = Me + Alpha*DeltaT*Ke and F the residual
 * R = F - Me a - Ke u -- and its time loop is Predictor_Old
 * (Time_Integration/Predictor_Old.c:3-148) with the stop criteria of
 * Criteria.c.  The context's other options (storage, reordering,
 * preconditioner NOT / Diag / ILU0, solver, shock CAU / YZBETA / CAUDD,
 * h_shock 2sqrtArea / Option1 / Option2) are the deck's as for the steady
 * driver. */
enum femgpu_stab { FEMGPU_STAB_SUPG = 0, FEMGPU_STAB_DD = 1 };
typedef struct femgpu_transient_opts {
	int stab;              /* StabilizationForm                                  */
	double alpha, dt;      /* Alpha, DeltaT                                      */
	double final_time;     /* FinalTime                                          */
	int stop_norm;         /* StopMulticorrection: 0 ITERATION, 1 NORM           */
	int max_corr;          /* NonLinearMaxIter                                   */
	double nonlin_tol;     /* NonLinearTolerance (NORM)                          */
	int steady_stop;       /* StopAtSteadyState: 1 YES, 0 NOT                    */
	double time_tol;       /* TimeIntegrationTolerance (YES)                     */
	int method;            /* TimeIntegration: FEMGPU_TI_*                       */
} femgpu_transient_opts;
/* Predictor1 (Predictor_Old.c), Predictor1_BDF (Predictor_Old_BDF.c:3-176:
 * one implicit step, then BDF2 with u = 4/3 u_n - 1/3 u_(n-1)) and
 * Predictor1_TRBDF2 (Predictor_Old_TRBDF2.c:3-179: a trapezoidal stage of
 * (2 - sqrt 2) dt, then a BDF2 stage), each with the reference's own
 * Alpha / DeltaT bookkeeping for the builds. */
enum femgpu_time_integration { FEMGPU_TI_PREDICTOR1 = 0, FEMGPU_TI_BDF = 1, FEMGPU_TI_TRBDF2 = 2,
                               FEMGPU_TI_PREDICTOR2 = 3, FEMGPU_TI_PREDICTOR2_BDF = 4,
                               FEMGPU_TI_PREDICTOR2_TRBDF2 = 5 };
/* Predictor2 (Predictor_New.c:3-137, DD stabilisation only): the element
 * bubbles are unknowns of the time loop -- uB starts at each element's mean
 * nodal value (uB_InitialSolution.c), the build is Build_M_F_DD
 * (Build_M_F_DD.c:6-218: the bubble row condensed into the element matrix),
 * and after every solve calculate_DaB.c updates the bubbles.
 * Predictor2_BDF (Predictor_New_BDF.c:3-216: uB starts at zero, one implicit
 * step built with Alpha_Build = 1, then BDF2 on u and uB) and
 * Predictor2_TRBDF2 (Predictor_New_TRBDF2.c:3-228: a trapezoidal and a BDF2
 * stage per step on u and uB, DeltaT_Build set per stage) are the same with
 * the two multistep forms (setStabilizationForm.c:54-61). */
int femgpu_transport_set_transient(femgpu_transport *ctx, const femgpu_transient_opts *o);
/* One transient Build on the state (u, a) (host [neq+1]; NULL: the context's):
 * R_host [neq+1] the residual, A_host the storage values (as
 * femgpu_transport_build); each call advances the DD state. */
int femgpu_transport_build_transient(femgpu_transport *ctx, const double *u_host, const double *a_host,
		double *R_host, double *A_host);
/* The bubble state (Predictor2) for the next femgpu_transport_build_transient:
 * uB_host, aB_host [nel] (NULL: leave as is). */
int femgpu_transport_set_bubbles(femgpu_transport *ctx, const double *uB_host, const double *aB_host);
/* The time loop of opts.method from u0_host [neq+1] (the problem's
 * InitialSolution; a = 0, a fresh DD state).  Predictor1: per step
 * u += (1-alpha) dt a, a = 0, then corrections Build -> precond_setup ->
 * solve(R, Da) -> a += Da, u += alpha dt Da until the multicorrection
 * criterion holds; the steps continue until the time criterion holds or
 * max_steps steps.  A stage is one multicorrection loop (two per TRBDF2
 * step, one otherwise): u_hist [S*max_steps*(neq+1)], ncorr [S*max_steps]
 * (corrections of each stage) and iters [S*max_steps*iters_cap] (GMRES
 * iterations of each correction) hold the stages in order, S = 2 for TRBDF2
 * and 1 otherwise; t_hist [max_steps] the time at the end of each step.
 * Arrays are filled when non-NULL.  Returns the number of steps run or an
 * error. */
int femgpu_transport_predictor(femgpu_transport *ctx, const double *u0_host, int max_steps, double *u_hist,
		double *t_hist, int *ncorr, int *iters, int iters_cap);

/* Paraview_Output (Paraview_Output.c:5-85): writes the VTU file the
 * reference writes for a solution -- ASCII UnstructuredGrid with the nodal
 * solution (prescribed value at prescribed nodes) as point data and as the
 * third coordinate, byte for byte -- to path.  u_host [neq+1] (NULL: the
 * context's device u, i.e. the last solution). */
int femgpu_transport_write_vtu(femgpu_transport *ctx, const char *path, const double *u_host);

/* Device-pointer forms (stream-ordered, no synchronisation). */
int femgpu_transport_build_dev(femgpu_transport *ctx);
int femgpu_transport_precond_setup_dev(femgpu_transport *ctx, int tag);
int femgpu_transport_matvec_dev(femgpu_transport *ctx, const double *P, double *Q);
/* Q = A P as the context's Krylov solver applies it (FGMRES with CSR
 * storage: the fused product over the SELL-32 copy, within rounding of
 * csrmv.c; otherwise femgpu_transport_matvec_dev's product), device
 * pointers on the context's stream. */
int femgpu_transport_operator_dev(femgpu_transport *ctx, const double *P, double *Q);
int femgpu_transport_precond_dev(femgpu_transport *ctx, const double *p, double *z);
/* The same preconditioner evaluated in FP32 (the mixed-precision solves'). */
int femgpu_transport_precond32_dev(femgpu_transport *ctx, const double *p, float *z);
int femgpu_transport_solve_dev(femgpu_transport *ctx, int *iters);
/* Device pointers of the context's u and F (length neq+1). */
double *femgpu_transport_u_dev(femgpu_transport *ctx);
double *femgpu_transport_F_dev(femgpu_transport *ctx);

/* True residual ||F_orig - A u|| / ||F_orig|| of the last solve in FP64
 * (F_orig = the RHS before precond_setup). */
int femgpu_transport_true_residual(femgpu_transport *ctx, double *relres);

/* Timing of the last solve's phases in milliseconds (CUDA events):
 * t[0] build, t[1] precond_setup, t[2] solve. */
int femgpu_transport_last_times(const femgpu_transport *ctx, float *t);

/* ---- multi-dof element-by-element operators ------------------------------
 * The Euler (ndof 4: rho, rho u, rho v, rho E; 12x12 element blocks) and
 * steady Navier-Stokes (ndof 3: u, v, p; 9x9) storage of
 * 03_Euler_Equations/2D/01_CommonFiles/EulerEquations.h:87-126 and
 * 04_SS_NavierStokes_Equations/2D/01_CommonFiles/SSNavierStokesEquations.h.
 * node_id [nnodes*ndof]: Node[].id[] of Fill_ID.c (-1 prescribed), so
 * lm[e][ndof*a+k] follows Fill_LM.c (neq for prescribed).  Element matrices
 * A [nel*(3ndof)^2] row-major, the reference's A[e][...] layout. */
typedef struct femgpu_ebe femgpu_ebe;
int femgpu_ebe_create(femgpu_ebe **ctx, int ndof, int nnodes, int nel, const int *vert,
		const int *node_id, int neq);
void femgpu_ebe_destroy(femgpu_ebe *ctx);
int femgpu_ebe_set_stream(femgpu_ebe *ctx, void *stream);
/* Upload element matrices from host memory (the device copy is also
 * reachable through femgpu_ebe_A_dev for matrices built on the device). */
int femgpu_ebe_set_matrix(femgpu_ebe *ctx, const double *A_host);
double *femgpu_ebe_A_dev(femgpu_ebe *ctx);
/* ebemvNDOF4 (EBE/ebemvNDOF4.c:3-112) / ebemvNDOF3 (EBE/ebemvNDOF3.c:3-86):
 * Q = A P; P[neq] read as 0, Q[neq] = 0. */
int femgpu_ebe_matvec(femgpu_ebe *ctx, const double *P_host, double *Q_host);
int femgpu_ebe_matvec_dev(femgpu_ebe *ctx, const double *P, double *Q);
/* Mixed precision (no reference counterpart): Q = A P with the FP32 copy of
 * the element matrices (made by a FEMGPU_MIXED_IR precond_setup) and an FP32
 * P; FP32 element rows, FP64 row totals.  FEMGPU_E_NOT_BUILT without the copy. */
int femgpu_ebe_matvec32_dev(femgpu_ebe *ctx, const float *P, double *Q);
/* ebe2mvNDOF4 (EBE/ebe2mvNDOF4.c:4-79, ndof 4): off-diagonal node blocks of
 * every element, then with_inverse ? Q = P + D^-1 Q (BlockDiag2_precond.c)
 * : Q += D P (NOBlockDiag2_precond.c).  Needs femgpu_ebe_blockdiag_setup. */
int femgpu_ebe_matvec2(femgpu_ebe *ctx, const double *P_host, double *Q_host, int with_inverse);
int femgpu_ebe_matvec2_dev(femgpu_ebe *ctx, const double *P, double *Q, int with_inverse);
/* BlockDiag_precond_EBE_setup.c:6-86 / BlockDiagDOF3_precond_EBE_setup.c:
 * nodal diagonal blocks D, their inverses, then F := D^-1 F (F_host may be
 * NULL).  BD_host / invBD_host [nnodes*ndof^2] receive the blocks (NULL skips). */
int femgpu_ebe_blockdiag_setup(femgpu_ebe *ctx, double *F_host, double *BD_host, double *invBD_host);
/* BlockDiag_precond.c / BlockDiagDOF3_precond.c: z = D^-1 p; p may equal z. */
int femgpu_ebe_blockdiag_apply(femgpu_ebe *ctx, const double *p_host, double *z_host);
int femgpu_ebe_blockdiag_apply_dev(femgpu_ebe *ctx, const double *p, double *z);

/* ---- 2D Euler: SUPG+CAU build and predictor-multicorrector -------------
 * 03_Euler_Equations/2D with StabilizationForm SUPG, ShockCapture CAU,
 * MatrixVectorProductScheme EBE or CSR, TimeIntegration Predictor1
 * (Predictor_Old) and StopMulticorrection ITERATION.  Conservative unknowns
 * per node in the order (rho, rho u, rho v, rho E).  Slip walls (v1Type ==
 * -1, rotation.c) through femgpu_euler_set_slip. */
typedef struct femgpu_euler_opts {
	double gamma;        /* ratio of specific heats (gamma(), constant)     */
	double mach;         /* reference Mach number (dimensionless only)       */
	int dimensionless;   /* Dimensionless: 0 NO, 1 YES (Ax_Ay_calculations.c) */
	double alpha;        /* Alpha of the predictor                           */
	double dt;           /* DeltaT                                           */
	double stab_tol;     /* StabilizationTolerance (CAU switch, Delta_CAU.c:71) */
	int precond;         /* FEMGPU_PREC_NOT, FEMGPU_PREC_BLOCKDIAG (EBE),     */
	                     /* FEMGPU_PREC_ILU0 or FEMGPU_PREC_AMG (CSR)        */
	int solver;          /* femgpu_solver: PGMRES (reference) or FGMRES      */
	int kmax, lmax;      /* KrylovBasisVectorsQuantity, SolverMaxIter        */
	double tol;          /* SolverTolerance                                  */
	int ncorr;           /* NonLinearMaxIter correctors per step (ITERATION) */
	int precision;       /* FEMGPU_FP64 (the reference's), or FEMGPU_MIXED_IR */
	                     /* with FGMRES: FP32 element matrices and           */
	                     /* preconditioner inside the Arnoldi cycles, every  */
	                     /* restart from the FP64 residual, a solve accepted */
	                     /* on the FP64 residual (EBE storage)               */
	int scheme;          /* MatrixVectorProductScheme: FEMGPU_EBE (12x12     */
	                     /* element blocks, NOT / BLOCKDIAG) or FEMGPU_CSR   */
	                     /* (csr_Initialization.c / csr_assembly.c of the    */
	                     /* Euler driver, reordering NOT; NOT / ILU0 / AMG)  */
	int ilu_blocks;      /* CSR + ILU0: 0 the whole matrix (the reference's), */
	                     /* P > 1 block ILU(0) over P row blocks (as         */
	                     /* femgpu_transport_opts.ilu_blocks)                */
	int scaling;         /* Scaling: 0 NOT, 1 BlockScaling (EBE storage):    */
	                     /* after every Build, Block_scaling_EBE              */
	                     /* (Block_scaling.c:7-49): the nodal block diagonal  */
	                     /* set up and R := D^-1 R, the prescribed rows and   */
	                     /* columns of each element matrix made identity, and */
	                     /* each node's row block multiplied by its D^-1      */
	int shock;           /* ShockCapture: FEMGPU_SHOCK_CAU (Delta_CAU.c) or   */
	                     /* FEMGPU_SHOCK_YZBETA (Delta_YZBeta.c:6-108: with   */
	                     /* invY, blended with each element's previous delta, */
	                     /* which starts at 0 when the context is made and    */
	                     /* at every femgpu_euler_predictor call)             */
	double invY[4];      /* the deck's Y^-1 (YZBeta)                          */
	int stab;            /* StabilizationForm: FEMGPU_STAB_SUPG              */
	                     /* (Build_M_K_F_SUPG.c; shock CAU or YZBETA) or      */
	                     /* FEMGPU_STAB_DD (Build_M_K_F_DD_Transiente.c: the  */
	                     /* element bubbles condensed out, updated by every   */
	                     /* build; shock CAUDD (Delta_DD.c) or YZBETA; no     */
	                     /* slip-wall rotation, as the reference's)           */
	int method;          /* TimeIntegration: FEMGPU_TI_PREDICTOR1            */
	                     /* (Predictor_Old.c), FEMGPU_TI_BDF                  */
	                     /* (Predictor_Old_BDF.c: an implicit first step,     */
	                     /* then BDF2) or FEMGPU_TI_TRBDF2                    */
	                     /* (Predictor_Old_TRBDF2.c: a trapezoidal and a BDF2 */
	                     /* stage per step, the build's DeltaT the TR sub-step */
	                     /* for its first build only, the BDF2 one after)     */
} femgpu_euler_opts;

void femgpu_euler_default_opts(femgpu_euler_opts *o);

/* Device-resident Euler problem (replaces MatrixDataType / FemStructsType of
 * EulerEquations.h:84-134 for the EBE and CSR schemes). */
typedef struct femgpu_euler femgpu_euler;

/* Preprocess for the EBE scheme (Preprocess.c, Fill_ID.c, Fill_LM.c):
 *   x, y      [nnodes]     node coordinates
 *   vert      [3*nel]      element vertices (0-based)
 *   node_id   [4*nnodes]   equation of each (node, dof), -1 prescribed
 *   neq                    number of equations
 *   upresc    [4*nnodes]   prescribed values (rhopresc, v1presc, v2presc,
 *                          epresc evaluated at the node; eval_U_dU.c:27-90) */
int femgpu_euler_create(femgpu_euler **ctx, const femgpu_euler_opts *opts, int nnodes, const double *x,
		const double *y, int nel, const int *vert, const int *node_id, int neq, const double *upresc);
void femgpu_euler_destroy(femgpu_euler *ctx);
int femgpu_euler_set_stream(femgpu_euler *ctx, void *stream);

/* Build_M_K_F_SUPG (Build_M_K_F_SUPG.c:6-1072): element matrices
 * Ae = Me + alpha dt Ke and residual R = -(Me dU + Ke U) assembled by lm, from
 * u and du [neq+1] (host; NULL = the context's device u / a).  Ae_host
 * [144*nel] and R_host [neq+1] receive copies (NULL skips). */
int femgpu_euler_build(femgpu_euler *ctx, const double *u, const double *du, double *Ae_host,
		double *R_host);
int femgpu_euler_build_dev(femgpu_euler *ctx);
/* precond_setup (BlockDiag_precond_EBE_setup.c:6-86 with PGMRES: R := D^-1 R;
 * FGMRES leaves R unpreconditioned).  R_host [neq+1] receives R (NULL skips). */
int femgpu_euler_precond_setup(femgpu_euler *ctx, double *R_host);
/* FemFunctions->scaling = Block_scaling_EBE (Block_scaling.c:7-49; Scaling
 * "BlockScaling", EBE storage): after a Build, the block diagonal of the
 * current matrix set up and R := D^-1 R, then the element matrices scaled
 * (opts.scaling makes the predictor call it after every Build). R_host
 * [neq+1] and Ae_host [nel*144] receive the results when non-NULL. */
int femgpu_euler_scale_dev(femgpu_euler *eu);
int femgpu_euler_scale(femgpu_euler *eu, double *R_host, double *Ae_host);
int femgpu_euler_precond_setup_dev(femgpu_euler *ctx);
/* solver (pgmres.c:4-211 with FemFunctions->mv = ebemvNDOF4): Da solves
 * A Da = R.  B_host [neq+1] replaces R when non-NULL; X_host receives Da. */
int femgpu_euler_solve(femgpu_euler *ctx, const double *B_host, double *X_host, int *iters);
/* CSR storage: sizes n_nnz = {neq, nnz} and (arrays may be NULL) the pattern
 * IA [neq+1], JA [nnz], CSR_by_Element sbe [144*nel] (nnz for a prescribed
 * row or column, csr_Initialization.c) and the values of the last build AA
 * [nnz+1]; FEMGPU_E_ARG for EBE storage. */
int femgpu_euler_csr(femgpu_euler *ctx, int *n_nnz, int *IA, int *JA, int *sbe, double *AA);
int femgpu_euler_solve_dev(femgpu_euler *ctx, int *iters);
/* Predictor_Old (Time_Integration/Predictor_Old.c:46-132) for nsteps time
 * steps of ncorr correctors from u (host [neq+1], in/out; NULL = the device
 * state) with a = 0 at the start of every step.  uhist [nsteps*(neq+1)]
 * receives u after each step and iters [nsteps*ncorr] the GMRES iterations
 * of each corrector (NULL skips); with FEMGPU_TI_TRBDF2 a step has two stages
 * and uhist [2*nsteps*(neq+1)], iters [2*nsteps*ncorr] hold them, the TR
 * stage first.  The YZBeta shock parameters start at zero
 * here (Predictor_Old.c:23); femgpu_euler_predictor_dev continues from the
 * device state, theirs included. */
int femgpu_euler_predictor(femgpu_euler *ctx, double *u, int nsteps, double *uhist, int *iters);
/* The Alpha_Build and DeltaT_Build the following builds use
 * (Build_M_K_F_SUPG.c:19-20; the time loops set them: Predictor_Old_TRBDF2.c
 * changes DeltaT_Build between its stages), for a driver that keeps its own
 * time loop; femgpu_euler_predictor sets them itself. */
int femgpu_euler_set_build_params(femgpu_euler *ctx, double alpha_build, double dt_build);
/* DD state: the element bubbles uB [4*nel] for the following builds (NULL:
 * zero), and the current bubbles and delta_old [nel] (either may be NULL). */
int femgpu_euler_set_bubbles(femgpu_euler *ctx, const double *uB);
int femgpu_euler_state(femgpu_euler *ctx, double *uB, double *delta_old);
int femgpu_euler_predictor_dev(femgpu_euler *ctx, int nsteps, int *iters);
/* Device pointers of the state vectors u, a, R, Da [neq+1] and the block
 * EBE operator holding the element matrices. */
double *femgpu_euler_u_dev(femgpu_euler *ctx);
femgpu_ebe *femgpu_euler_ebe(femgpu_euler *ctx);
/* Seconds spent in build, precond_setup and solve by the last
 * femgpu_euler_predictor(_dev) call (t[3]). */
int femgpu_euler_last_times(const femgpu_euler *ctx, double *t);

/* ---- steady incompressible Navier-Stokes: VMS build and damped Newton -----
 * 04_SS_NavierStokes_Equations/2D with StabilizationForm MS (Build_K_F_MS),
 * MatrixVectorProductScheme EBE, BlockDiag preconditioning (3x3 nodal blocks)
 * and Process's damped Newton.  Unknowns per node (u, v, p). */
typedef struct femgpu_ns_opts {
	double re;           /* ReynoldsNumber                                   */
	double velmax;       /* VelMax (reference velocity of the local Re)      */
	int precond;         /* FEMGPU_PREC_NOT, FEMGPU_PREC_BLOCKDIAG (EBE),     */
	                     /* FEMGPU_PREC_ILU0 or FEMGPU_PREC_AMG (CSR)        */
	int solver;          /* femgpu_solver: PGMRES (reference) or FGMRES      */
	int kmax, lmax;      /* KrylovBasisVectorsQuantity, LinearMaxIter        */
	double eta0;         /* SolverTolerance: initial / maximal forcing term  */
	int eta_case;        /* SolverToleranceCase 0..4 (eta_newton.c)          */
	double tol_nl;       /* SolverToleranceNonLin: ||F|| <= tol_nl ||F_0||   */
	int scheme;          /* FEMGPU_EBE (9x9 element blocks) or FEMGPU_CSR    */
	                     /* (csr_Initialization.c / csr_assembly.c, numbering */
	                     /* of the node ids as given: reordering NOT)         */
	int ilu_blocks;      /* CSR + ILU(0): 0 the whole matrix (the            */
	                     /* reference's), P > 1 block ILU(0) over P row      */
	                     /* blocks (as femgpu_transport_opts.ilu_blocks)     */
} femgpu_ns_opts;

void femgpu_ns_default_opts(femgpu_ns_opts *o);
typedef struct femgpu_ns femgpu_ns;

/*   x, y      [nnodes]    node coordinates; vert [3*nel]
 *   node_id   [3*nnodes]  equation of each (node, u|v|p), -1 prescribed
 *   upresc    [3*nnodes]  prescribed values (v1presc, v2presc, ppresc)
 *   f         [2*nnodes]  body force at the nodes (f1ext, f2ext; NULL = 0) */
int femgpu_ns_create(femgpu_ns **ctx, const femgpu_ns_opts *opts, int nnodes, const double *x,
		const double *y, int nel, const int *vert, const int *node_id, int neq, const double *upresc,
		const double *f);
void femgpu_ns_destroy(femgpu_ns *ctx);
int femgpu_ns_set_stream(femgpu_ns *ctx, void *stream);
/* Zero the per-element stabilisation state (delta_old, normres_old) and the
 * build count, as at the start of Process (Process.c:49-56). */
int femgpu_ns_reset(femgpu_ns *ctx);
/* Build_K_F_MS (Build_K_F_MS.c:8-1190) from u [neq+1] (host; NULL = the
 * device state): element matrices Ae_host [81*nel] and F_host [neq+1]
 * (NULL skips); the first build after create/reset takes the reference's
 * first-call branch of the stabilisation update. */
int femgpu_ns_build(femgpu_ns *ctx, const double *u, double *Ae_host, double *F_host);
int femgpu_ns_build_dev(femgpu_ns *ctx);
/* BlockDiagDOF3_precond_EBE_setup: F := D^-1 F (F_host receives it). */
int femgpu_ns_precond_setup(femgpu_ns *ctx, double *F_host);
/* pgmres (6-argument form) on the 3-dof block EBE operator: X solves
 * A X = B (B_host NULL: the context's F) to the current forcing term. */
int femgpu_ns_solve(femgpu_ns *ctx, const double *B_host, double *X_host, int *iters);
/* The relative tolerance of the next femgpu_ns_solve calls: the forcing term
 * that the reference's Process keeps in Parameters->SolverTolerance
 * (eta_newton.c, Process.c:118-140); femgpu_ns_newton sets its own. */
int femgpu_ns_set_tol(femgpu_ns *ctx, double tol);
/* Process.c:62-194 from u = 0: at most maxit damped-Newton iterations (and
 * the reference's 2000 cap), stopping when ||F|| <= tol_nl ||F_0||.  u_host
 * [neq+1] receives the solution; uhist [maxit*(neq+1)], normF, w [maxit],
 * gmres [maxit] the per-iteration history (each may be NULL).  Returns the
 * number of Newton iterations done (>= 0) or an error code. */
int femgpu_ns_newton(femgpu_ns *ctx, int maxit, double *u_host, double *uhist, double *normF, double *w,
		int *gmres);
/* CSR storage: sizes n_nnz = {neq, nnz} and (arrays may be NULL) the pattern
 * IA [neq+1], JA [nnz] and the values of the last build AA [nnz+1];
 * FEMGPU_E_ARG for EBE storage. */
int femgpu_ns_csr(femgpu_ns *ctx, int *n_nnz, int *IA, int *JA, double *AA);
double *femgpu_ns_u_dev(femgpu_ns *ctx);
femgpu_ebe *femgpu_ns_ebe(femgpu_ns *ctx);

/* ---- learned preconditioner ----------------------------------------------
 * No counterpart in the reference.  A mesh graph network (3 message-passing
 * layers of width 32, FP32 weights, bf16 or FP32 activations) on the graph of
 * a CSR matrix maps a residual r to a correction z ~ M^-1 r; it is trained on
 * the GPU on (r, ILU(0) correction) pairs by hand-written forward and
 * backward kernels and Adam, and serves as the right preconditioner of
 * FGMRES (FEMGPU_PREC_LEARNED), with ILU(0) as the fallback when a restart
 * cycle stalls.  Parameters: femgpu_gnn_nparams() floats. */
typedef struct femgpu_gnn femgpu_gnn;
int femgpu_gnn_nparams(void);
/* theta NULL: all parameters zero. */
int femgpu_gnn_create(femgpu_gnn **ctx, int bf16_activations, const float *theta);
void femgpu_gnn_destroy(femgpu_gnn *ctx);
int femgpu_gnn_set_stream(femgpu_gnn *ctx, void *stream);
/* Set the parameters (resets the Adam state) / read parameters, gradient. */
int femgpu_gnn_set_params(femgpu_gnn *ctx, const float *theta);
int femgpu_gnn_get_params(femgpu_gnn *ctx, float *theta);
int femgpu_gnn_get_grad(femgpu_gnn *ctx, float *grad);
/* Attach the graph of an n-row CSR matrix (one diagonal entry per row,
 * structurally symmetric, rows sorted): host arrays, or device arrays with
 * nnz = IA[n]. */
int femgpu_gnn_attach_csr(femgpu_gnn *ctx, int n, const int *IA, const int *JA, const double *AA);
int femgpu_gnn_attach_csr_dev(femgpu_gnn *ctx, int n, int nnz, const int *IA, const int *JA,
		const double *AA);
/* z = N(r) over the attached graph (n entries). */
int femgpu_gnn_apply(femgpu_gnn *ctx, const double *r_host, double *z_host);
int femgpu_gnn_apply_dev(femgpu_gnn *ctx, const double *r, double *z);
/* Forward and backward of L = ||z - t||^2 / ||t||^2 for one pair: z receives
 * N(r), the gradient is stored (accumulate != 0 adds to it); loss (host, may
 * be NULL: no synchronisation) receives L. */
int femgpu_gnn_loss_grad_dev(femgpu_gnn *ctx, const double *r, const double *t, double *z, int accumulate,
		double *loss);
int femgpu_gnn_loss_grad(femgpu_gnn *ctx, const double *r_host, const double *t_host, double *loss,
		float *grad_host, double *z_host);
/* Training loss: 0 supervised ||z - t||^2/||t||^2 against the ILU(0)
 * correction t (default), 1 residual ||A z - r||^2/||r||^2 (t unused), 2 the
 * sum of both. */
int femgpu_gnn_set_loss(femgpu_gnn *ctx, int kind);
/* Adam (beta 0.9, 0.999, eps 1e-8) on the stored gradient scaled by gscale. */
int femgpu_gnn_adam_step(femgpu_gnn *ctx, float lr, float gscale);
/* Use ctx as the FEMGPU_PREC_LEARNED preconditioner of a CSR transport
 * context (re-attached to the matrix at every precond_setup). */
int femgpu_transport_set_learned(femgpu_transport *t, femgpu_gnn *ctx);
/* Device pointers of the context's CSR matrix (IA [neq+1], JA [nnz], AA
 * [nnz+1]); FEMGPU_E_ARG for EBE/EDE storage. */
int femgpu_transport_csr_dev(femgpu_transport *t, const int **IA, const int **JA, const double **AA);
/* Copy up to max (v_i, M^-1 v_i) pairs of the last FGMRES restart cycle
 * (Arnoldi vectors and their preconditioned images, neq entries each) into
 * device arrays V, Z with leading dimension ld; returns the count (>= 0). */
int femgpu_transport_krylov_pairs(femgpu_transport *t, int max, double *V, double *Z, int ld);

/* ---- AMG preconditioner (double pairwise aggregation) ----------------------
 * AMG_precond_setup / AMG_precond with the deck string "AMG 2 NCL beta omega
 * nr" (00_CommonFiles/Solvers_and_Preconditioners/amg_precond.c:26-110):
 * dpa_setup (CSR/AMG/amg_dpa.c:424-463) builds 2*NCL+1 levels by pairwise
 * matching -- matching_c (amg_dpa.c:30-173) for beta >= 0, the
 * half-approximate maximum-product matching bcm_CSRMatrixHMatch
 * (bcm_linmatch.c) for beta == -1 -- and Galerkin products (dpa_galerkin,
 * amg_dpa.c:175-392); the preconditioner is one dpa_Vcycle_precond
 * (amg_dpa.c:485-506) with nr SOR sweeps of weight omega per level.  The
 * set-up runs on the host, the V-cycle on the device; both give the
 * reference's hierarchy and output bit for bit.  The classical Ruge-Stueben
 * variant ("AMG 1 ...") and XDPA ("AMG 3 ...") are not provided. */
typedef struct femgpu_amg femgpu_amg;
int femgpu_amg_create(femgpu_amg **ctx, int ncl, double beta, double omega, int nr);
void femgpu_amg_destroy(femgpu_amg *ctx);
int femgpu_amg_set_stream(femgpu_amg *ctx, void *stream);
/* Hierarchy of an n-row host CSR matrix (sorted rows, symmetric pattern). */
int femgpu_amg_setup(femgpu_amg *ctx, int n, const int *IA, const int *JA, const double *AA);
/* Matrices in the hierarchy (2*NCL+1), and level l's sizes n_nnz = {n, nnz}
 * and (arrays may be NULL) CSR and matching rmatch [n+1] (partner or -1,
 * rmatch[n] = number of pairs; levels below the coarsest). */
int femgpu_amg_levels(const femgpu_amg *ctx);
int femgpu_amg_level(const femgpu_amg *ctx, int l, int *n_nnz, int *IA, int *JA, double *AA, int *rmatch);
/* z = M^-1 q, one V-cycle (q == z allowed). */
int femgpu_amg_apply(femgpu_amg *ctx, const double *q_host, double *z_host);
int femgpu_amg_apply_dev(femgpu_amg *ctx, const double *q, double *z);
/* Use ctx as the FEMGPU_PREC_AMG preconditioner of a CSR transport context
 * (precond_setup rebuilds the hierarchy from the current matrix), or as the
 * fallback of a FEMGPU_PREC_LEARNED context (built when a solve stalls). */
int femgpu_transport_set_amg(femgpu_transport *t, femgpu_amg *ctx);
/* The same for the Navier-Stokes and Euler contexts with CSR storage and
 * precond FEMGPU_PREC_AMG (setPreconditioner.c:63-73 of the Navier-Stokes
 * driver, :130-140 of the Euler driver): precond_setup builds the hierarchy
 * of the current CSR matrix and (left-preconditioned GMRES) applies one
 * V-cycle to the right-hand side; the solves apply one V-cycle per step.
 * In all three ctx runs on the context's stream while set and goes back to
 * its own stream when the context is destroyed, so ctx must outlive it. */
int femgpu_ns_set_amg(femgpu_ns *ns, femgpu_amg *ctx);
int femgpu_euler_set_amg(femgpu_euler *eu, femgpu_amg *ctx);
/* Slip walls of the Euler SUPG build (Build_M_K_F_SUPG.c:1044-1056 with
 * rotation.c:3-43): slip [nnodes] != 0 marks the nodes the reference gives
 * v1Type = -1; their rows and columns of each element matrix and their
 * entries of the element residual are rotated by the wall angle BC_theta(x, y),
 * whose cosine and sine the caller passes (cs, sn [nnodes], evaluated on the
 * host as rotation.c evaluates them).  slip = NULL removes the walls. */
int femgpu_euler_set_slip(femgpu_euler *eu, const int *slip, const double *cs, const double *sn);

/* ---- stateless device kernels (device pointers, stream as void*) -------- */
/* csrmv.c:3-24 in FP64 / FP32 values. */
int femgpu_csrmv_f64(int n, const int *IA, const int *JA, const double *AA,
		const double *P, double *Q, void *stream);
int femgpu_csrmv_f32(int n, const int *IA, const int *JA, const float *AA,
		const float *P, float *Q, void *stream);
/* The FP64 product as the FGMRES contexts apply it: each row's terms in
 * column order as fused multiply-adds (one rounding per entry), so it is
 * within rounding of, not bit-identical to, csrmv.c (femgpu_csrmv_f64 is). */
int femgpu_csrmv_f64_fused(int n, const int *IA, const int *JA, const double *AA,
		const double *P, double *Q, void *stream);

/* Allocation-free residual norm.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc -- a host application that hands the
 * library a fixed device-memory budget, or a driver that must not grow device
 * memory between steps.  Computes, for a CSR system in device memory,
 * out2[0] = ||F - A u||^2 and out2[1] = ||F||^2 (out2: two doubles of device
 * memory), the quantity femgpu_transport_true_residual reports.  Its block
 * partial sums live in a fixed static device array (32 KB, held by every GPU
 * that loads the library until exit), so n <= 4,194,304 rows; larger n returns
 * FEMGPU_E_ARG.  The first call on a device looks up that array's device
 * address with the device current (make that first call before any stream
 * capture); later calls look it up again unless their stream is being
 * captured, so a device reset or another current context is followed.  All
 * calls share the array: calls that overlap on the GPU race, so serialise
 * them. */
int femgpu_csr_resnorm_noalloc(int n, const int *IA, const int *JA, const double *AA,
		const double *u, const double *F, double *out2, void *stream);

/* ---- parameter decks and mesh files (no GPU needed) ------------------------
 * The reading half of each driver's Preprocess (transport Preprocess.c:
 * 44-99, Euler Preprocess.c:45-102, Navier-Stokes Preprocess.c:45-88): the
 * deck's "value<TAB>:label" lines in the driver's order, and the mesh file
 * <dir>/<ProblemTitle>_<nnodes>_<nel>.dat (node count; per node x, y and the
 * driver's node types -- 1 for transport (Type), 4 for Euler (rhoType,
 * v1Type, v2Type, eType), 3 for Navier-Stokes (v1Type, v2Type, pType); the
 * element count; per element three vertices and its type). */
enum femgpu_equation { FEMGPU_EQ_TRANSPORT = 0, FEMGPU_EQ_EULER = 1, FEMGPU_EQ_NS = 2,
                       FEMGPU_EQ_TRANSIENT = 3 };
/* FEMGPU_EQ_TRANSIENT: the transient transport driver's deck
 * (02_Transport_Equation/2D/01_CommonFiles/Preprocess.c:42-66); its mesh
 * file has one node type and no element type column (Preprocess.c:94-97):
 * read it with ntype = 1 | FEMGPU_MESH_NO_ELEM_TYPE. */
#define FEMGPU_MESH_NO_ELEM_TYPE 0x100
typedef struct femgpu_deck {
	int equation;
	char Experiments[200], ProblemTitle[300], Solver[200], Preconditioner[1000], Scaling[200],
	     reordering[200], MatrixVectorProductScheme[200], StabilizationForm[200], ShockCapture[200],
	     h_Shock[200], OutputFlow[200], TimeIntegration[200], StopAtSteadyState[200], Dimensionless[200],
	     StopMulticorrection[200];
	double SolverTolerance, NonLinearTolerance, TimeIntegrationTolerance, StabilizationTolerance, Alpha,
	       DeltaT, FinalTime, Mach, invY[4], ReynoldsNumber, VelMax, SolverToleranceNonLin;
	int SolverMaxIter, KrylovBasisVectorsQuantity, LinearMaxIter, NonLinearMaxIter, SolverToleranceCase,
	    nnodes, nel;
} femgpu_deck;
int femgpu_deck_read(const char *path, int equation, femgpu_deck *deck);
/* The mesh file the driver opens for a deck: <dir>/<ProblemTitle>_<nnodes>_<nel>.dat. */
int femgpu_deck_mesh_file(const femgpu_deck *deck, const char *dir, char *path, int cap);
/* Read a mesh file with ntype node types per node: sizes into nnodes, nel;
 * x, y [nnodes], node_type [ntype*nnodes], vert [3*nel], elem_type [nel]
 * filled when non-NULL (call once with NULL arrays for the sizes).  With
 * FEMGPU_MESH_NO_ELEM_TYPE or-ed into ntype the element lines hold three
 * vertices only and elem_type is set to 0 (the calloc'd Type the transient
 * driver leaves). */
int femgpu_mesh_read(const char *path, int ntype, int *nnodes, int *nel, double *x, double *y, int *node_type,
		int *vert, int *elem_type);
/* The element types the transport drivers' Preprocess sets after reading
 * (01_SS_Transport_Equation/2D/01_CommonFiles/Preprocess.c:107-151): the
 * side of the unit square an element has two vertices on (1 x=0, 2 y=0,
 * 3 x=1, 4 y=1), 5-8 for the corner pairs the reference tests, -1 inside. */
int femgpu_mesh_side_types(int nnodes, const double *x, const double *y, int nel, const int *vert, int *elem_type);
/* The deck's strings as options (each driver's setMatrixVectorProductType.c,
 * setPreconditioner.c, setStabilizationForm.c); FEMGPU_E_ARG for a choice
 * the library does not provide.  femgpu_deck_amg parses "AMG 2 NCL beta
 * omega nr" (amg_precond.c:26-40). */
int femgpu_deck_transport_opts(const femgpu_deck *deck, femgpu_transport_opts *o);
int femgpu_deck_euler_opts(const femgpu_deck *deck, femgpu_euler_opts *o);
int femgpu_deck_ns_opts(const femgpu_deck *deck, femgpu_ns_opts *o);
/* A transient transport deck as a transport context's options and its
 * transient options (02_Transport_Equation/2D/01_CommonFiles:
 * setMatrixVectorProductType.c, setPreconditioner.c (NOT, Diag, ILU<p> with
 * CSR), setStabilizationForm.c (SUPG or DD with the six TimeIntegration
 * strings, the shock capture and h_Shock strings), Criteria.c (ITERATION |
 * NORM, YES | NOT)); Scaling must be NOT. */
int femgpu_deck_transient_opts(const femgpu_deck *deck, femgpu_transport_opts *o, femgpu_transient_opts *tr);
int femgpu_deck_amg(const femgpu_deck *deck, int *ncl, double *beta, double *omega, int *nr);

/* ---- host utilities (no GPU needed) ------------------------------------- */
/* REORDERING_SYMRCM (00_CommonFiles/Reordering/symrcm.c:4-242): reverse
 * Cuthill-McKee permutation perm[new] = old of a structurally symmetric CSR
 * pattern, with the reference's tie-breaking. */
int femgpu_symrcm(int n, const int *IA, const int *JA, int *perm);
/* LEVEL_OF_FILL_lu (Solvers_and_Preconditioners/ilup.c:164-302): the ILU(p)
 * pattern of a CSR pattern (every row with its diagonal) for level of fill p,
 * each row stored as the reference stores it -- lower part ascending, the
 * diagonal, the upper part in the order the symbolic elimination found it.
 * Returns the filled nnz; fIA [n+1] and fJA [cap] receive the pattern when
 * non-NULL (FEMGPU_E_ARG when cap is too small). */
int femgpu_iluk_pattern(int n, const int *IA, const int *JA, int p, int *fIA, int *fJA, int cap);
/* Dependency levels of the ILU(0) forward (lower != 0) or backward sweep:
 * returns the number of levels. */
int femgpu_ilu_levels(int n, const int *IA, const int *JA, int lower);
/* One step of the AMG set-up: the pairwise matching of matching_c
 * (amg_dpa.c:30-173, beta >= 0) or bcm_CSRMatrixHMatch (bcm_linmatch.c,
 * beta == -1), rmatch [n+1] as in femgpu_amg_level; and the Galerkin
 * product dpa_galerkin (amg_dpa.c:175-392): nc_nnz = {rows, nnz} of the
 * coarse matrix, whose CSR goes to IC/JC/AC when they are given (call once
 * with NULL arrays for the sizes). */
int femgpu_dpa_match(int n, const int *IA, const int *JA, const double *AA, double beta, int *rmatch);
int femgpu_dpa_galerkin(int n, const int *IA, const int *JA, const double *AA, const int *rmatch, int *nc_nnz,
		int *IC, int *JC, double *AC);

/* Last CUDA/device error text of this thread (static buffer). */
const char *femgpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
