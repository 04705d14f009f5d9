/*
 * Test infrastructure only -- the CPU oracle.
 *
 * A plain-C restatement of the reference's steady 2D transport solve loop
 * (mod-comp-ufes/FEM_CODES, 01_SS_Transport_Equation/2D + 00_CommonFiles),
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
 * checker.  It is never linked into the product library.  Parity of this
 * restatement is pinned against the reference's own sources run here
 * (oracle/_ref, see tests/golden/make_golden.py): bit-exact on every golden
 * fixture.
 */
#ifndef FEM_ORACLE_H
#define FEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Fill_LM + node numbering (Preprocess.c:73-81, Fill_LM.c:3-19). Returns neq. */
int orc_fill_lm(int nnodes, const int *node_type, int nel, const int *vert,
                int *node_id, int *lm);

/* CSR pattern of csr_Initialization.c:18-123: rows = equations, ascending
 * unique columns; sbe = CSR_by_Element (prescribed entries -> nnzero).
 * Pass IA/JA/sbe == NULL to get the nnz only. Returns nnz. */
int orc_csr_pattern(int neq, int nel, const int *lm, int *IA, int *JA, int *sbe);

/* SYMRCM permutation of symrcm.c:4-236 (perm[new] = old). */
void orc_symrcm(int n, const int *IA, const int *JA, int *perm);

/* Reordering of csr_Initialization.c:144-179 + reordering.c:238-308: permute
 * the CSR in place, remap sbe (nel*9) and node_id (nnodes). Returns the
 * bandwidth after (reordering.c:310-332). */
int orc_reorder_csr(int neq, int nnz, int *IA, int *JA, const int *perm,
                    int nel, int *sbe, int nnodes, int *node_id);
int orc_bandwidth(int n, const int *IA, const int *JA);

/* Edge structure of ede_Initialization.c:16-170. lm2: 2*nedge, ebe: 3*nel,
 * order: 3*nel. Pass NULL outputs to get nedge only. Returns nedge. */
int orc_ede_pattern(int neq, int nel, const int *lm, int *lm2, int *ebe, int *order);

/* Options of the element build */
enum { ORC_EBE = 0, ORC_EDE = 1, ORC_CSR = 2 };
enum { ORC_CAU = 0, ORC_YZBETA = 1 };
enum { ORC_H_2SQRTAREA = 0, ORC_H_SQRTAREA = 1, ORC_H_OPTION1 = 2, ORC_H_OPTION2 = 3 };

typedef struct {
	int nnodes, nel, neq, nnz, nedge;
	const double *x, *y;
	const int *node_type, *node_id, *vert, *etype;
	const double *beta, *fsrc, *upresc;   /* 2*nel, 3*nel, nnodes */
	double k, gamma;
	int scheme, shock, hshock, outflow;
	const int *sbe;                        /* CSR 9*nel / EDE 3*nel */
	const int *order;                      /* EDE 3*nel */
} orc_transport;

/* Build_K_F_SUPG.c:5-163 (+ CAU_ShockCapture.c, YZBeta_ShockCapture.c,
 * h_shock_*.c, F_assembly.c, {ebe,ede,csr}_assembly.c). u: neq+1.
 * A: EBE 9*nel / EDE 4*(nedge+1) / CSR nnz+1. F: neq+1. */
void orc_build_supg(const orc_transport *t, const double *u, double *A, double *F);

/* Matvecs: csrmv.c:3-24, ebemv.c:4-43, edemv.c:4-39. P,Q: neq+1. */
void orc_csrmv(int neq, const int *IA, const int *JA, const double *AA, const double *P, double *Q);
void orc_ebemv(int neq, int nel, const int *lm, const double *A, double *P, double *Q);
void orc_edemv(int neq, int nedge, const int *lm2, const double *A, double *P, double *Q);

/* ILU(0) numeric factorisation in the CSR positions of A (ILUp_precond_setup.c:66-167
 * with p = 0): LU[nnz] holds L (col < row) and U (col > row); Dinv[n] = 1/pivot.
 * Returns 0, or 1 + row of the first zero pivot. */
int orc_ilu0_factor(int n, const int *IA, const int *JA, const double *AA, double *LU, double *Dinv);
int orc_iluk_pattern(int n, const int *IA, const int *JA, int p, int *fIA, int *fJA);
void orc_iluk_scatter(int n, const int *IA, const int *JA, const double *AA, const int *fIA, const int *fJA,
                      double *fA);
/* ILUp_precond.c:26-46: z = (LU)^-1 p; p may alias z. */
void orc_ilu0_apply(int n, const int *IA, const int *JA, const double *LU, const double *Dinv,
                    const double *p, double *z);

/* Reference BLAS order (BLAS_Operations/ddot.c:4-18). */
double orc_ddot(int n, const double *x, const double *y);

/* A complete steady-transport run on in-memory arrays: the same outputs as
 * oracle/ref_harness.c's ref_transport_run. String options as in the deck. */
int orc_transport_run(int nnodes, const double *x, const double *y, const int *ntype,
		int nel, const int *vert, double k, double gamma,
		const double *beta, const double *fsrc, const double *upresc,
		const char *scheme, const char *reord, const char *precond,
		const char *shock, const char *hshock, const char *outflow,
		int kmax, int lmax, double tol, int npicard, double nonlin_tol,
		int *info, int *node_id, int *etype,
		int *IA_out, int *JA_out, int *sbe_out, int *order_out,
		double *Afirst, double *Ffirst, double *Fprec,
		const double *Pin, double *Qmv, double *Zpc,
		double *uhist, int *iters);

/* Phase wall times of the last orc_transport_run in seconds:
 * [set-up, build, precond_setup, solve] (the last three summed over Picard). */
void orc_get_times(double *t);
/* Wall time (seconds) of each of the first n Picard iterations of that run. */
void orc_get_step_times(double *t, int n);
void orc_set_refine(double to, double tol, int maxrounds);
void orc_set_refine_window(int from, double budget_s);
void orc_get_refine(double *res, int *rounds, int n);

/* Operator application out = Op(in) on vectors of neq+1 entries. */
typedef void (*orc_apply_fn)(const void *ctx, double *in, double *out);

/* pgmres.c:4-211 over caller-supplied operator and preconditioner (prec may
 * be NULL for none).  Returns the number of inner iterations. */
int orc_pgmres_cb(int neq, orc_apply_fn mv, orc_apply_fn prec, const void *ctx, int kmax, int lmax,
                  double tol, const double *B, double *X);

/* pgmres.c:4-211 on an assembled CSR system with optional ILU(0):
 * B is overwritten by M^-1 B when precond != 0 (the precond_setup side effect),
 * X receives the solution. Returns the number of inner iterations. */
int orc_csr_gmres(int neq, const int *IA, const int *JA, const double *AA, int use_ilu0,
                  int kmax, int lmax, double tol, double *B, double *X);

/* ---- multi-dof EBE operators (Euler ndof 4, Navier-Stokes ndof 3) ------- */
void orc_fill_lm_blk(int ndof, int nel, const int *vert, const int *node_id, int neq, int *lm);
void orc_ebemv_blk(int ndof, int neq, int nel, const int *lm, const double *A, double *P, double *Q);
void orc_blockdiag_assemble(int ndof, int nnodes, int nel, const int *vert, const double *A, double *BD);
void orc_inverse4(const double *B, double *V);
void orc_inverse3(const double *B, double *V);
void orc_blockdiag_apply(int ndof, int nnodes, int neq, const int *node_id, const double *invBD,
                         const double *p, double *z);
void orc_blockdiag_setup(int ndof, int nnodes, int nel, int neq, const int *vert, const int *node_id,
                         const double *A, double *BD, double *invBD, double *F);
void orc_ebe2mv4(int nnodes, int neq, int nel, const int *lm, const int *node_id, const double *A,
                 const double *BD, const double *invBD, int with_inverse, double *P, double *Q);

/* ---- 2D Euler (03_Euler_Equations/2D) ---------------------------------- */
typedef struct {
	int nnodes, nel, neq;
	const double *x, *y;          /* [nnodes]                                   */
	const int *vert;              /* [3*nel]                                    */
	const int *node_id;           /* [4*nnodes] equation of (node, dof) or -1   */
	const double *upresc;         /* [4*nnodes] prescribed (rho, rho u, rho v, rho E) */
	double gamma, mach;           /* mach used only when dimensionless != 0     */
	int dimensionless;
	double alpha, dt, stab_tol;
} orc_euler;

/* Build_M_K_F_SUPG.c:6-1072 (no slip-wall rotation): element matrices
 * Ae [nel*144] (row-major 12x12) and residual R [neq+1]. */
void orc_euler_build(const orc_euler *p, const double *u, const double *du, double *Ae, double *R);

/* Predictor_Old.c:46-132 with StopByIterations (ncorr correctors per step),
 * BlockDiag_precond_EBE_setup + ebemvNDOF4 + pgmres.  u [neq+1] in/out;
 * uhist [nsteps*(neq+1)] (may be NULL), iters [nsteps*ncorr] (may be NULL).
 * Returns the total GMRES iterations. */
int orc_euler_predictor(const orc_euler *p, int kmax, int lmax, double tol, int nsteps, int ncorr,
                        double *u, double *uhist, int *iters);

/* ---- steady Navier-Stokes (04_SS_NavierStokes_Equations/2D) ------------- */
typedef struct {
	int nnodes, nel, neq;
	const double *x, *y;          /* [nnodes]                                   */
	const int *vert;              /* [3*nel]                                    */
	const int *node_id;           /* [3*nnodes] equation of (node, u|v|p) or -1 */
	const double *upresc;         /* [3*nnodes] prescribed (u, v, p)            */
	const double *f;              /* [2*nnodes] body force at the nodes         */
	double re, velmax;
} orc_ns;

/* Build_K_F_MS.c:8-1190 (the branch it executes): Ae [nel*81], F [neq+1];
 * first != 0 for the first build of a run; dold, nold [nel] are the
 * per-element stabilisation state (delta_old, normres_old), updated. */
void orc_ns_build(const orc_ns *p, const double *u, int first, double *dold, double *nold, double *Ae,
                  double *F);
/* eta_newton.c:5-68 given ||F||, ||Fold||. */
double orc_eta_newton(int ecase, double nF, double nFold, double etaold, int pricek, int it, double talnl,
                      double eta0);
/* Process.c:62-194 from u = 0 with BlockDiagDOF3 + pgmres, at most maxit
 * Newton iterations; returns the iterations done. */
int orc_ns_newton(const orc_ns *p, int kmax, int lmax, double eta0, int ecase, double tolnl, int maxit,
                  double *uhist, double *normF, double *wout, int *gmres);

/* ---- AMG (double pairwise aggregation) ------------------------------------ */
/* One dpa_Vcycle_precond (amg_dpa.c:485-506): z = M^-1 q over nlev levels
 * given as concatenated CSR arrays (n[l] rows each; IA blocks of n[l]+1
 * offsets local to the level, JA/AA blocks of IA_l[n[l]] entries) and the
 * matchings of levels 0..nlev-2 (blocks of n[l]+1). */
int orc_amg_vcycle(int nlev, const int *n, const int *IA, const int *JA, const double *AA, const int *rm,
                   double omega, int nr, const double *q, double *z);
/* pgmres with csrmv (level 0) and that V-cycle, B := M^-1 B first (the
 * AMG_precond_setup side effect); returns the inner iterations. */
int orc_amg_gmres(int nlev, const int *n, const int *IA, const int *JA, const double *AA, const int *rm,
                  double omega, int nr, int kmax, int lmax, double tol, double *B, double *X);

#ifdef __cplusplus
}
#endif
#endif
