/*
 * Internal state and kernel-launch entry points of libfemgpu.
 * Shared by the CUDA translation units (*.cu) and the host C driver
 * (the C files under host/); plain C, no CUDA-only types beyond cuda_runtime_api.h.
 *
 * Device layout (all device memory, allocated once per context):
 *   mesh      x, y [nnodes] f64; node_type, node_id [nnodes] i32;
 *             vert, lm [3*nel] i32 (lm = equation of each vertex, neq = dump)
 *   incidence ri_ptr [neq+1], ri [..] = 3*e + a for every unknown vertex a of
 *             element e, rows sorted by e (drives the deterministic gathers)
 *   CSR       IA [neq+1], JA [nnz], sbe [9*nel] (CSR_by_Element), diag [neq]
 *   EDE       lm2 [2*nedge], sbe [3*nel] (EDGE_by_Element), order [3*nel],
 *             edge contributor lists ec_ptr/ec, row "second endpoint" lists
 *   values    A: EBE 9*nel | EDE 4*(nedge+1) | CSR nnz+1 (f64, plus an f32
 *             copy in mixed precision); ke [9*nel], fe [3*nel] element temps
 *   vectors   u, F, F0 [neq+1]; Krylov basis V [(kmax+1) x ldv]
 */
#ifndef FG_INTERNAL_H
#define FG_INTERNAL_H

#include <cuda_runtime_api.h>
#include "femgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One triangular sweep compiled into level blocks (see ilu.cu). */
typedef struct fg_sweep {
	int nlev, nsb;             /* levels, sub-blocks (<= 512 rows each)      */
	long long bytes, maxblk, nval;
	int npad;                  /* padded length of the level-ordered vector  */
	unsigned char *prog;       /* sub-blocks                                 */
	long long *blk_off;        /* [nsb+1] byte offsets of the sub-blocks     */
	int *sb_in, *sb_inb;       /* [nsb] input slice start (padded), bytes    */
	int *lev_start;            /* [nlev+1] first level-order position        */
	int *rows;                 /* [n] row at each level-order position       */
	int *ppos;                 /* [n] padded position of each position       */
	long long *val_off;        /* [nval] byte offset of each value slot      */
	int *val_src;              /* [nval] CSR position (-1 zero, -2-r pivot)  */
	int nchunk;                /* matrix blocks (block ILU(0); 1: global)    */
	int *chunk_sb, *chunk_lev; /* [nchunk+1] first sub-block / level of each */
	int rw;                    /* record layout width (0: ELL sub-blocks)    */
	int df;                    /* record layout swept without level barriers */
	int skew;                  /* ... levels a warp may run ahead            */
	int bvo, cmax;             /* record layout: input slice offset in a
	                            * stage, most rows of a sub-block            */
	/* chain-scan programs (k_sweep_cs): levels of warp segments, 32 slots a
	 * segment chunk; per slot the byte offset of its five scan multipliers
	 * (-1: padding), the CSR position of its chain coefficient (-1: none)
	 * and its row */
	int cs, nslot;
	long long *cs_voff;
	int *cs_src, *cs_row;
} fg_sweep;

typedef struct fg_ilu_sweeps {
	fg_sweep lo64, up64, lo32, up32;
	/* chain-scan programs of the same factor for the fused (FGMRES) FP64 and
	 * the FP32 sweeps; chain = 0 when the sweeps have too few chained rows */
	fg_sweep lo64c, up64c, lo32c, up32c;
	int chain;
	/* the FP64 chain programs' layout with double-single values (ds = 1:
	 * the fused FP64 sweeps run on the FP32 pipes, 48-bit significands) */
	unsigned char *prog_lo_ds, *prog_up_ds;
	int ds;
	/* bit i: program i of lo64, up64, lo32, up32, lo64c, up64c, lo32c,
	 * up32c still holds an earlier factor's values (refreshed by the first
	 * application that uses it) */
	int stale;
	/* ds: dpos [n] the slot of natural row r in the sweeps' gathered input
	 * (the inverse of the gather of the double-single apply) */
	int *dpos;
	double *bl64, *y64;
	double *o64;                    /* ds: the double-single sweeps' output
	                                   (natural order), apart from their input */
	float *bl32, *y32;
	int *fac_ptr, *fac_prog;   /* precompiled elimination of each row        */
	/* the same elimination for the cluster kernel: per level-order position
	 * {rb, offset, length, len | dpos << 8 | ngroups << 16}, and per row
	 * [nops, operand addresses..., per group (q, cnt, dst...)] */
	int *fac2_hdr, *fac2;
	int fac2_ok;
	int nblocks;               /* matrix blocks (1: global ILU(0))           */
	int *block_first;          /* host [nblocks+1] first row of each block   */
	/* ILU(p), p > 0: the filled pattern the factor and sweeps use (rows as
	 * the reference stores them), each matrix entry's position in it, and
	 * the matrix values scattered onto it before every factorisation */
	int fill, fnnz;
	int *fIA, *fJA, *fmap;
	double *fA;
} fg_ilu_sweeps;

/* CSR storage of a multi-dof element system (csr_Initialization.c of the
 * Navier-Stokes and Euler drivers, reordering NOT): pattern, CSR_by_Element
 * slots [M*M*nel], values [nnz+1]; with ILU(0), the factorisation and
 * sweep engine run on a transport context that holds only this system. */
typedef struct fg_blockcsr {
	int *IA, *JA, *sbe;
	double *AA;
	int nnz;
	struct femgpu_transport *ilu;
	int have_ilu;
	struct femgpu_amg *amg;        /* AMG preconditioner (owned by the caller) */
} fg_blockcsr;

typedef struct fg_ilu {
	int n, nnz;
	double *LU;        /* [nnz] L (col<row) and U (col>row) in A's positions */
	double *Dinv;      /* [n] inverted pivots                                */
} fg_ilu;

/* Device status block (one per context, device memory). */
typedef struct fg_status {
	int err;           /* first device-side error code (FEMGPU_E_*)          */
	int active;        /* GMRES inner loop still running                     */
	int inner;         /* inner iterations done in the current cycle         */
	int total;         /* total inner iterations of the solve                */
	double rho, eps;
	double hdiag;      /* scratch                                            */
	unsigned ticket;   /* last-block reduction ticket                        */
	int pad;
} fg_status;

/* Krylov workspace (device memory unless noted); one per context.  A view
 * of a context's buffers is enough to run the cycles below. */
typedef struct fg_krylov {
	int n, kmax, nblk;              /* unknowns, basis size, reduction blocks */
	size_t ldv;                     /* leading dimension of V / Z (>= n+1)   */
	cudaStream_t stream;
	double *V;                      /* [(kmax+1) x ldv] Arnoldi basis         */
	double *H, *cs, *sn, *ge, *gy;  /* Hessenberg (kmax+1)^2, Givens, rhs, y  */
	double *Z;                      /* [kmax x ldv] FGMRES M^-1 v (FP64)      */
	float *Z32;                     /* [kmax x ldv] FGMRES M^-1 v (FP32)      */
	double *partials;               /* [nblk] reduction partials              */
	fg_status *st;                  /* device status                          */
	fg_status *st_host;             /* pinned host mirror                     */
	int dsv;                        /* FGMRES: Arnoldi basis in double-single */
	/* FGMRES look-ahead (la_s != NULL): the preconditioner of the next step
	 * runs on la_s, on the raw operator output la_w, while the Gram-Schmidt
	 * of this step runs on stream; la_t [ldv] the combination of the stored
	 * directions, la_eta the subdiagonal entry, la_flag [kmax+1] per-step
	 * snapshots of the convergence flag for the la_s work */
	cudaStream_t la_s;
	cudaEvent_t la_ev_w, la_ev_y;
	double *la_w, *la_t, *la_eta;
	int *la_flag;
} fg_krylov;

/* Operator callbacks, stream-ordered, returning cudaError_t (> 0) or a
 * FEMGPU_E* code (< 0).  active (device flag, may be NULL) predicates the
 * work of an inner iteration after convergence.  precond NULL: identity. */
typedef struct fg_linop {
	void *ctx;
	int (*matvec)(void *ctx, const double *p, double *q, const int *active);
	int (*precond)(void *ctx, const double *p, double *z, const int *active);
	/* mixed precision (FGMRES): z = M^-1 p in FP32, and q = A z from an FP32
	 * vector with FP64 (op32 == 0) or FP32 (op32 != 0) matrix values. */
	int (*precond32)(void *ctx, const double *p, float *z, const int *active);
	/* double-single Krylov basis (fg_krylov.dsv): z = M^-1 p from a
	 * double-single p, and q = A p into a double-single q (pairs of floats,
	 * 8 bytes per entry like the FP64 basis) */
	int (*precond_dsin)(void *ctx, const void *p, double *z, const int *active);
	int (*matvec_dsout)(void *ctx, const double *p, void *q, const int *active);
	int (*matvec_xf)(void *ctx, const float *p, double *q, const int *active, int op32);
	/* z = M^-1 p on the given stream (the look-ahead FGMRES step) */
	int (*precond_s)(void *ctx, const double *p, double *z, const int *active, cudaStream_t s);
	/* the look-ahead step with the gather fused into the product (NULL when
	 * the context has no such form): q = A p, also written as the
	 * preconditioner's gathered input; the preconditioner on that input on
	 * the given stream; and its output (double-single, natural order) */
	int (*matvec_g)(void *ctx, const double *p, double *q, const int *active);
	int (*precond_g)(void *ctx, const int *active, cudaStream_t s);
	const void *(*precond_g_out)(void *ctx);
} fg_linop;

struct femgpu_transport {
	femgpu_transport_opts o;
	int nnodes, nel, neq, nnz, nedge, bandwidth;
	cudaStream_t stream, own_stream;
	int built, factored;

	/* mesh / problem */
	double *x, *y, *upresc, *beta, *fsrc;
	int *node_type, *node_id, *vert, *lm;
	double k, gamma, cbx, cby;
	int beta_const, fsrc_zero;
	int *h_node_id;                 /* host copy of the numbering            */

	/* incidence */
	int *ri_ptr, *ri;

	/* storage patterns */
	int *IA, *JA, *sbe, *diag;
	int *lm2, *order, *ec_ptr, *ec, *e2_ptr, *e2;

	/* values */
	double *A, *ke, *fe;
	float *A32;
	double *u, *F, *F0, *invDiag;
	float *invDiag32;
	fg_ilu ilu;
	fg_ilu_sweeps sweeps;
	int sweep_wait1;                /* 1 + dependency-wait bound; 0: default */
	/* the CSR matrix in 32-row slices (SELL-32) for the products: entry j of
	 * row r at sell_base[r/32] + 32 j + r%32; sell_src maps a slot to its CSR
	 * position (-1: padding) for the refresh after each assembly */
	long long *sell_base;
	int *sell_w, *sell_src, *sell_JA;
	double *sell_A;
	int nslice;
	long long nslot;

	/* transient driver (femgpu_transport_set_transient) */
	int transient;
	femgpu_transient_opts tr;
	double *du;                     /* the time derivative a (neq+1)         */
	double *re;                     /* per element: load term + 3 products x3 */
	double *dold;                   /* DD: previous shock parameter per elem */
	double *uold, *Da, *u1, *u2;    /* predictor vectors (neq+1)             */
	double *uB, *aB, *bub;          /* Predictor_New: bubble unknowns, rate, and
	                                   invN2, R2, M2[3] per element          */
	double *uB1, *uB2;              /* Predictor_New_BDF / _TRBDF2: bubble
	                                   history (nel each)                    */

	/* FGMRES look-ahead resources (fg_krylov.la_*), made on first use */
	cudaStream_t la_s;
	cudaEvent_t la_ev[2];
	double *la_buf;                 /* la_w [ldv], la_t [ldv], la_eta [1]    */
	int *la_flag;                   /* [kmax + 1]                            */

	/* Krylov workspace */
	int kmax;
	size_t ldv;
	double *V, *H, *cs, *sn, *ge, *gy, *w2;
	double *Z;                      /* FGMRES preconditioned vectors (FP64)  */
	float *Z32;                     /* ... (FP32, mixed precision)           */
	double *xr, *dr;                /* refinement: residual and correction   */
	double *partials;               /* reduction partials                    */
	int nblk_red;
	fg_status *st;                  /* device status                         */
	fg_status *st_host;             /* pinned mirror                         */

	/* learned preconditioner (FEMGPU_PREC_LEARNED) */
	struct femgpu_gnn *gnn;
	int fell_back;                  /* this solve switched to ILU(0)         */

	/* AMG preconditioner (FEMGPU_PREC_AMG) */
	struct femgpu_amg *amg;

	/* timing */
	cudaEvent_t ev[4];
	float times[3];
};

/* ---- kernels (stream-ordered launchers, return cudaError_t as int) ---- */
/* pattern.cu */
int fg_build_incidence(femgpu_transport *t);                 /* ri_ptr / ri   */
int fg_build_csr(femgpu_transport *t);                       /* IA, JA, sbe   */
int fg_build_ede(femgpu_transport *t);                       /* lm2, sbe, ... */
int fg_compute_lm(femgpu_transport *t);                      /* lm from ids   */

/* build.cu */
int fg_build_elements(femgpu_transport *t);                  /* ke / A, fe    */
int fg_assemble(femgpu_transport *t);                        /* A (CSR/EDE), F */
int fg_build_transient(femgpu_transport *t, int dd, double adt);   /* Ae, re   */
int fg_assemble_transient(femgpu_transport *t);              /* A, R -> F     */
int fg_tr_predict(femgpu_transport *t, double c);            /* uold, u, a    */
int fg_tr_correct(femgpu_transport *t, double c);            /* a, u += Da    */
int fg_tr_diff(femgpu_transport *t);                         /* Da = u - uold */
int fg_build_mfdd(femgpu_transport *t, double adt);          /* Me, re, bub   */
int fg_bubble_correct(femgpu_transport *t, double c);        /* DaB, aB, uB   */
int fg_bubble_predict(femgpu_transport *t, double c);
int fg_bubble_init(femgpu_transport *t);
int fg_bubble_lin(femgpu_transport *t, const double *p, const double *q, double cp, double cq);
int fg_tr_axpy_zero(femgpu_transport *t, double c);          /* u += c a, a=0 */
int fg_tr_lin(femgpu_transport *t, const double *p, const double *q, double cp, double cq); /* u=cp p-cq q */

/* linalg.cu */
int fg_matvec(femgpu_transport *t, const double *P, double *Q, const int *active);
int fg_csrmv64(int n, const int *IA, const int *JA, const double *AA, const double *P,
               double *Q, const int *active, cudaStream_t s);
int fg_csrmv32(int n, const int *IA, const int *JA, const float *AA, const float *P,
               float *Q, const int *active, cudaStream_t s);
int fg_csrmv64_fused(int n, const int *IA, const int *JA, const double *AA, const double *P,
                     double *Q, const int *active, cudaStream_t s);
int fg_csrmv64_fused_ds(int n, const int *IA, const int *JA, const double *AA, const double *P,
                        void *Q, const int *active, cudaStream_t s);
int fg_sell_refresh(femgpu_transport *t);                    /* sell_A from A */
int fg_sellmv(femgpu_transport *t, const double *P, void *Q, int fused, int ds_out, const int *active);
int fg_diag_setup(femgpu_transport *t);
int fg_precond(femgpu_transport *t, const double *p, double *z, const int *active);
/* One restart cycle of the reference's left-preconditioned GMRES
 * (pgmres.c:58-184) / of flexible right-preconditioned GMRES (mixed 0: FP64,
 * 1: FP32 preconditioner, 2: FP32 preconditioner and operator). */
int fg_kry_pgmres_cycle(const fg_krylov *k, const fg_linop *op, const double *B, double *X);
/* cycle: index of this restart cycle within the solve (picks the
 * orthogonalisation, see gs_mode in linalg.cu) */
int fg_kry_fgmres_cycle(const fg_krylov *k, const fg_linop *op, const double *B, double *X, int mixed,
                        int cycle);
/* CSR storage for M equations per element (M = 9: Navier-Stokes): pattern,
 * CSR_by_Element slots [M*M*nel], and the per-row assembly from element
 * matrices Ae [nel][M][M] (device arrays; pattern arrays allocated here). */
int fg_build_csr_m(int M, int nel, int neq, const int *ri_ptr, const int *ri, const int *lm, cudaStream_t s,
                   int *err, int **IA, int **JA, int **sbe, int *nnz);
int fg_assemble_csr_m(int M, int neq, int nnz, const int *IA, const int *sbe, const int *ri_ptr, const int *ri,
                      const double *Ae, double *AA, cudaStream_t s);
/* st->rho = ||B - A X|| (A X is formed in V[kmax]). */
int fg_kry_true_rho(const fg_krylov *k, const fg_linop *op, const double *B, double *X);
int fg_kry_dot(const fg_krylov *k, const double *a, const double *b, int n, double *out_dev);
/* The transport context's Krylov buffers and operator as a view. */
void fg_transport_krylov(femgpu_transport *t, fg_krylov *k, fg_linop *op);
int fg_gmres_cycle(femgpu_transport *t, const double *B, double *X, int first);
/* Flexible GMRES cycle, right preconditioned; mixed != 0: FP32 operator and
 * preconditioner (A32, FP32 ILU/diagonal), FP64 Arnoldi. */
int fg_fgmres_cycle(femgpu_transport *t, const double *B, double *X, int mixed);
int fg_to_f32(const double *a, float *b, long long n, cudaStream_t s);
int fg_axpy_resid(femgpu_transport *t, const double *B, double *r);     /* r = B - A u */
int fg_add(double *x, const double *d, int n, cudaStream_t s);          /* x += d */

/* ilu.cu */
int fg_ilu_prepare(femgpu_transport *t, const int *hIA, const int *hJA);
int fg_ilu0_factor(femgpu_transport *t);
int fg_ilu0_apply64(femgpu_transport *t, const double *p, double *z, const int *active);
int fg_ilu0_sweeps_gathered(femgpu_transport *t, const int *active);
int fg_ilu0_apply32(femgpu_transport *t, const double *p, float *z, const int *active);
void fg_ilu_free(femgpu_transport *t);
int fg_dot(femgpu_transport *t, const double *a, const double *b, int n, double *out_dev);
int fg_residual_norm(femgpu_transport *t, const double *B, const double *X, double *out_dev);

#ifdef __cplusplus
}
#endif
#endif
