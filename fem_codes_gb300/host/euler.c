/*
 * Host driver of the 2D Euler path: the control flow of Predictor_Old
 * (00_CommonFiles/Time_Integration/Predictor_Old.c:46-132, multicorrector
 * stopped after NonLinearMaxIter correctors as StopByIterations does,
 * Criteria.c:25-31) around device kernels for the build
 * (Build_M_K_F_SUPG), the nodal block-diagonal preconditioner, the block-EBE
 * matvec and GMRES, or -- CSR storage -- the element matrices assembled into
 * the driver's CSR pattern (csr_assembly.c), csrmv and ILU(0).  Plain C.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_euler.h"
#include "../csrc/fg_amg.h"

#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)

void femgpu_euler_default_opts(femgpu_euler_opts *o)
{
	memset(o, 0, sizeof *o);
	o->gamma = 1.4;
	o->mach = 1.0;
	o->alpha = 0.5;
	o->dt = 1e-3;
	o->stab_tol = 1e-6;
	o->precond = FEMGPU_PREC_BLOCKDIAG;
	o->solver = FEMGPU_PGMRES;
	o->kmax = 30;
	o->lmax = 100;
	o->tol = 1e-8;
	o->ncorr = 2;
	o->scheme = FEMGPU_EBE;
	o->shock = FEMGPU_SHOCK_CAU;
	o->invY[0] = o->invY[1] = o->invY[2] = o->invY[3] = 1.0;
}

/* ---- operator callbacks of the Krylov solver ---------------------------- */
static int op_matvec(void *ctx, const double *p, double *q, const int *active)
{
	(void)active;
	return fg_ebe_matvec(((femgpu_euler *)ctx)->ebe, p, q, 0);
}

static int op_precond(void *ctx, const double *p, double *z, const int *active)
{
	(void)active;
	return fg_ebe_blockdiag_apply(((femgpu_euler *)ctx)->ebe, p, z, 0);
}

/* mixed precision: z = D^-1 p in FP32, q = A32 z */
static int op_precond32(void *ctx, const double *p, float *z, const int *active)
{
	femgpu_euler *c = (femgpu_euler *)ctx;
	(void)active;
	if (c->o.precond == FEMGPU_PREC_BLOCKDIAG) return fg_ebe_blockdiag_apply32(c->ebe, p, z);
	return fg_to_f32(p, z, (long long)c->neq + 1, c->stream);
}

static int op_matvec_xf(void *ctx, const float *p, double *q, const int *active, int op32)
{
	(void)active;
	if (!op32) return FEMGPU_E_ARG;                   /* only the FP32 operator is provided */
	return fg_ebe_matvec32(((femgpu_euler *)ctx)->ebe, p, q);
}

/* CSR storage: csrmv and ILUp_precond */
static int op_matvec_csr(void *ctx, const double *p, double *q, const int *active)
{
	femgpu_euler *c = (femgpu_euler *)ctx;
	return fg_csrmv64(c->neq, c->csr.IA, c->csr.JA, c->csr.AA, p, q, active, c->stream);
}

static int op_precond_ilu(void *ctx, const double *p, double *z, const int *active)
{
	return fg_ilu0_apply64(((femgpu_euler *)ctx)->csr.ilu, p, z, active);
}

static int op_precond_amg(void *ctx, const double *p, double *z, const int *active)
{
	return fg_amg_vcycle(((femgpu_euler *)ctx)->csr.amg, p, z, active);
}

static void linop(femgpu_euler *c, fg_linop *op)
{
	memset(op, 0, sizeof *op);
	op->ctx = c;
	if (c->o.scheme == FEMGPU_CSR) {
		op->matvec = op_matvec_csr;
		op->precond = c->o.precond == FEMGPU_PREC_ILU0 ? op_precond_ilu
		            : c->o.precond == FEMGPU_PREC_AMG ? op_precond_amg : NULL;
		return;
	}
	op->matvec = op_matvec;
	op->precond = c->o.precond == FEMGPU_PREC_BLOCKDIAG ? op_precond : NULL;
	op->precond32 = op_precond32;
	op->matvec_xf = op_matvec_xf;
}

static int uploadd(double **dst, const double *src, size_t n)
{
	int rc = fgh_dmalloc((void **)dst, sizeof(double) * n);
	if (rc) return rc;
	CK(cudaMemcpy(*dst, src, sizeof(double) * n, cudaMemcpyHostToDevice));
	return 0;
}

static int create(femgpu_euler *c, const femgpu_euler_opts *o, int nnodes, const double *x, const double *y,
                  int nel, const int *vert, const int *node_id, int neq, const double *upresc)
{
	size_t n1 = (size_t)neq + 1;
	int i, rc;
	c->o = *o;
	c->nnodes = nnodes; c->nel = nel; c->neq = neq;
	rc = femgpu_ebe_create(&c->ebe, 4, nnodes, nel, vert, node_id, neq);
	if (rc) return rc;
	CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
	c->stream = c->own_stream;
	KR(femgpu_ebe_set_stream(c->ebe, c->stream));
	rc = uploadd(&c->x, x, (size_t)nnodes);
	if (!rc) rc = uploadd(&c->y, y, (size_t)nnodes);
	if (!rc) rc = uploadd(&c->upresc, upresc, 4 * (size_t)nnodes);
	if (rc) return rc;
	DM(c->u, sizeof(double) * n1);
	DM(c->a, sizeof(double) * n1);
	DM(c->R, sizeof(double) * n1);
	DM(c->Da, sizeof(double) * n1);
	DM(c->Re, sizeof(double) * 12 * (size_t)nel);
	DM(c->dold, sizeof(double) * (size_t)nel);
	DM(c->uB, sizeof(double) * 4 * (size_t)nel);
	CK(cudaMemsetAsync(c->uB, 0, sizeof(double) * 4 * (size_t)nel, c->stream));
	c->alpha_build = o->alpha;
	c->dt_build = o->dt;
	CK(cudaMemsetAsync(c->dold, 0, sizeof(double) * (size_t)nel, c->stream));
	CK(cudaMemsetAsync(c->u, 0, sizeof(double) * n1, c->stream));
	CK(cudaMemsetAsync(c->a, 0, sizeof(double) * n1, c->stream));
	CK(cudaMemsetAsync(c->R, 0, sizeof(double) * n1, c->stream));
	CK(cudaMemsetAsync(c->Da, 0, sizeof(double) * n1, c->stream));
	rc = fgh_kry_alloc(&c->kry, neq, o->kmax,
	                   o->solver != FEMGPU_FGMRES ? 0 : o->precision == FEMGPU_MIXED_IR ? 2 : 1, c->stream);
	if (rc) return rc;
	if (o->scheme == FEMGPU_CSR &&
	    (rc = fgh_blockcsr_create(&c->csr, 12, c->ebe, nel, neq, c->stream, o->precond == FEMGPU_PREC_ILU0,
	                              o->solver, o->ilu_blocks))) return rc;
	for (i = 0; i < 4; i++) CK(cudaEventCreate(&c->ev[i]));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_euler_create(femgpu_euler **out, const femgpu_euler_opts *opts, int nnodes, const double *x,
                        const double *y, int nel, const int *vert, const int *node_id, int neq,
                        const double *upresc)
{
	femgpu_euler_opts o;
	femgpu_euler *c;
	int rc;
	if (!out) return FEMGPU_E_ARG;
	*out = NULL;
	if (opts) o = *opts; else femgpu_euler_default_opts(&o);
	if (nnodes <= 0 || nel <= 0 || neq <= 0 || !x || !y || !vert || !node_id || !upresc ||
	    o.kmax < 1 || o.lmax < 1 || o.ncorr < 1 || !(o.dt > 0.0) || !(o.tol > 0.0) ||
	    (o.scheme != FEMGPU_EBE && o.scheme != FEMGPU_CSR) || o.ilu_blocks < 0 ||
	    (o.scheme == FEMGPU_EBE && o.precond != FEMGPU_PREC_NOT && o.precond != FEMGPU_PREC_BLOCKDIAG) ||
	    (o.scheme == FEMGPU_CSR && o.precond != FEMGPU_PREC_NOT && o.precond != FEMGPU_PREC_ILU0 &&
	     o.precond != FEMGPU_PREC_AMG) ||
	    (o.scheme == FEMGPU_CSR && o.precision != FEMGPU_FP64) ||
	    (o.solver != FEMGPU_PGMRES && o.solver != FEMGPU_FGMRES) ||
	    (o.precision != FEMGPU_FP64 && o.precision != FEMGPU_MIXED_IR) ||
	    (o.precision == FEMGPU_MIXED_IR && o.solver != FEMGPU_FGMRES) ||
	    (o.scaling != 0 && (o.scaling != 1 || o.scheme != FEMGPU_EBE)) ||
	    (o.stab != FEMGPU_STAB_SUPG && o.stab != FEMGPU_STAB_DD) ||
	    (o.stab == FEMGPU_STAB_SUPG && o.shock != FEMGPU_SHOCK_CAU && o.shock != FEMGPU_SHOCK_YZBETA) ||
	    (o.stab == FEMGPU_STAB_DD && o.shock != FEMGPU_SHOCK_CAUDD && o.shock != FEMGPU_SHOCK_YZBETA) ||
	    (o.method != FEMGPU_TI_PREDICTOR1 && o.method != FEMGPU_TI_BDF && o.method != FEMGPU_TI_TRBDF2)) {
		fgh_set_error("femgpu_euler_create: bad argument or option");
		return FEMGPU_E_ARG;
	}
	c = calloc(1, sizeof *c);
	if (!c) return FEMGPU_E_NOMEM;
	rc = create(c, &o, nnodes, x, y, nel, vert, node_id, neq, upresc);
	if (rc) { femgpu_euler_destroy(c); return rc; }
	*out = c;
	return 0;
}

void femgpu_euler_destroy(femgpu_euler *c)
{
	int i;
	if (!c) return;
	if (c->stream) cudaStreamSynchronize(c->stream);
	fgh_blockcsr_destroy(&c->csr);
	if (c->ebe) femgpu_ebe_destroy(c->ebe);
	{
		void *p[] = { c->x, c->y, c->upresc, c->u, c->a, c->R, c->Da, c->Re, c->slip_flag, c->slip_el, c->slip_cs,
		              c->slip_sn, c->dold, c->uB, c->u1, c->u2, c->uold };
		for (i = 0; i < (int)(sizeof p / sizeof p[0]); i++) if (p[i]) cudaFree(p[i]);
	}
	fgh_kry_free(&c->kry);
	for (i = 0; i < 4; i++) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
	if (c->own_stream) cudaStreamDestroy(c->own_stream);
	free(c);
}

int femgpu_euler_set_stream(femgpu_euler *c, void *stream)
{
	if (!c) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(c->stream));
	c->stream = stream ? (cudaStream_t)stream : c->own_stream;
	c->kry.stream = c->stream;
	KR(femgpu_ebe_set_stream(c->ebe, c->stream));
	fgh_blockcsr_set_stream(&c->csr, c->stream);
	return 0;
}

int femgpu_euler_set_slip(femgpu_euler *c, const int *slip, const double *cs, const double *sn)
{
	int *vert = NULL, *el = NULL, n = 0, e, k, rc = 0;
	if (!c) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(c->stream));
	if (c->slip_flag) { cudaFree(c->slip_flag); cudaFree(c->slip_el); cudaFree(c->slip_cs); cudaFree(c->slip_sn); }
	c->slip_flag = c->slip_el = NULL;
	c->slip_cs = c->slip_sn = NULL;
	c->nslip_el = 0;
	if (!slip) return 0;
	if (!cs || !sn) return FEMGPU_E_ARG;
	vert = malloc(sizeof(int) * 3 * (size_t)c->nel);
	el = malloc(sizeof(int) * (size_t)c->nel + sizeof(int));
	if (!vert || !el) { free(vert); free(el); return FEMGPU_E_NOMEM; }
	if (cudaMemcpy(vert, c->ebe->vert, sizeof(int) * 3 * (size_t)c->nel, cudaMemcpyDeviceToHost) != cudaSuccess) {
		free(vert); free(el); return FEMGPU_E_CUDA;
	}
	for (e = 0; e < c->nel; e++) {
		for (k = 0; k < 3; k++) if (slip[vert[3 * e + k]]) break;
		if (k < 3) el[n++] = e;
	}
	free(vert);
	if (fgh_dmalloc((void **)&c->slip_flag, sizeof(int) * (size_t)c->nnodes) ||
	    fgh_dmalloc((void **)&c->slip_el, sizeof(int) * ((size_t)n + 1)) ||
	    fgh_dmalloc((void **)&c->slip_cs, sizeof(double) * (size_t)c->nnodes) ||
	    fgh_dmalloc((void **)&c->slip_sn, sizeof(double) * (size_t)c->nnodes))
		rc = FEMGPU_E_NOMEM;
	if (!rc && (cudaMemcpy(c->slip_flag, slip, sizeof(int) * (size_t)c->nnodes, cudaMemcpyHostToDevice) ||
	            cudaMemcpy(c->slip_el, el, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice) ||
	            cudaMemcpy(c->slip_cs, cs, sizeof(double) * (size_t)c->nnodes, cudaMemcpyHostToDevice) ||
	            cudaMemcpy(c->slip_sn, sn, sizeof(double) * (size_t)c->nnodes, cudaMemcpyHostToDevice)))
		rc = FEMGPU_E_CUDA;
	free(el);
	if (!rc) c->nslip_el = n;
	c->built = 0;
	c->have_bd = 0;
	return rc;
}

int femgpu_euler_set_amg(femgpu_euler *c, femgpu_amg *g)
{
	if (!c || !g || c->o.precond != FEMGPU_PREC_AMG) return FEMGPU_E_ARG;
	KR(femgpu_amg_set_stream(g, c->stream));
	c->csr.amg = g;
	c->have_bd = 0;
	return 0;
}

int femgpu_euler_csr(femgpu_euler *c, int *n_nnz, int *IA, int *JA, int *sbe, double *AA)
{
	if (!c || !n_nnz || c->o.scheme != FEMGPU_CSR) return FEMGPU_E_ARG;
	n_nnz[0] = c->neq; n_nnz[1] = c->csr.nnz;
	if (IA) CK(cudaMemcpyAsync(IA, c->csr.IA, sizeof(int) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost,
	                           c->stream));
	if (JA) CK(cudaMemcpyAsync(JA, c->csr.JA, sizeof(int) * (size_t)c->csr.nnz, cudaMemcpyDeviceToHost, c->stream));
	if (sbe) CK(cudaMemcpyAsync(sbe, c->csr.sbe, sizeof(int) * 144 * (size_t)c->nel, cudaMemcpyDeviceToHost,
	                            c->stream));
	if (AA) CK(cudaMemcpyAsync(AA, c->csr.AA, sizeof(double) * ((size_t)c->csr.nnz + 1), cudaMemcpyDeviceToHost,
	                           c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

double *femgpu_euler_u_dev(femgpu_euler *c) { return c ? c->u : NULL; }
femgpu_ebe *femgpu_euler_ebe(femgpu_euler *c) { return c ? c->ebe : NULL; }

int femgpu_euler_last_times(const femgpu_euler *c, double *t)
{
	if (!c || !t) return FEMGPU_E_ARG;
	memcpy(t, c->times, sizeof c->times);
	return 0;
}

/* ---- Build / precond_setup / solver ------------------------------------- */
int femgpu_euler_build_dev(femgpu_euler *c)
{
	if (!c) return FEMGPU_E_ARG;
	KR(fg_euler_build(c, c->u, c->a));
	if (c->o.scheme == FEMGPU_CSR) KR(fgh_blockcsr_assemble(&c->csr, 12, c->ebe, c->neq, c->stream));
	c->built = 1;
	c->have_bd = 0;
	return 0;
}

int femgpu_euler_build(femgpu_euler *c, const double *u, const double *du, double *Ae_host, double *R_host)
{
	size_t n1;
	if (!c) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	if (u) CK(cudaMemcpyAsync(c->u, u, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	if (du) CK(cudaMemcpyAsync(c->a, du, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	KR(femgpu_euler_build_dev(c));
	if (Ae_host)
		CK(cudaMemcpyAsync(Ae_host, c->ebe->A, sizeof(double) * 144 * (size_t)c->nel, cudaMemcpyDeviceToHost,
		                   c->stream));
	if (R_host) CK(cudaMemcpyAsync(R_host, c->R, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

/* FemFunctions->scaling = Block_scaling_EBE (Block_scaling.c:7-49): the
 * block diagonal of the current matrix set up and R := D^-1 R
 * (BlockDiag_precond_EBE_setup), then the element matrices scaled. */
int femgpu_euler_scale_dev(femgpu_euler *c)
{
	if (!c) return FEMGPU_E_ARG;
	if (!c->built) { fgh_set_error("scaling before build"); return FEMGPU_E_NOT_BUILT; }
	if (c->o.scheme != FEMGPU_EBE) { fgh_set_error("BlockScaling needs EBE storage (setScaling.c)"); return FEMGPU_E_ARG; }
	KR(fg_ebe_blockdiag_setup(c->ebe));
	KR(fg_ebe_blockdiag_apply(c->ebe, c->R, c->R, 0));
	KR(fg_ebe_block_scale(c->ebe));
	c->ebe->have_bd = 0;
	c->have_bd = 0;
	return 0;
}

int femgpu_euler_scale(femgpu_euler *c, double *R_host, double *Ae_host)
{
	if (!c) return FEMGPU_E_ARG;
	KR(femgpu_euler_scale_dev(c));
	if (R_host)
		CK(cudaMemcpyAsync(R_host, c->R, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost, c->stream));
	if (Ae_host)
		CK(cudaMemcpyAsync(Ae_host, c->ebe->A, sizeof(double) * 144 * (size_t)c->nel, cudaMemcpyDeviceToHost,
		                   c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_euler_precond_setup_dev(femgpu_euler *c)
{
	if (!c) return FEMGPU_E_ARG;
	if (!c->built) { fgh_set_error("precond_setup before build"); return FEMGPU_E_NOT_BUILT; }
	if (c->o.precision == FEMGPU_MIXED_IR) KR(fg_ebe_to_f32(c->ebe));
	if (c->o.precond == FEMGPU_PREC_ILU0) {
		/* ILUp_precond_setup.c:8-167 at fill level 0, then R := M^-1 R */
		KR(fgh_blockcsr_factor(&c->csr, c->stream));
		c->have_bd = 1;
		if (c->o.solver == FEMGPU_PGMRES) KR(fg_ilu0_apply64(c->csr.ilu, c->R, c->R, NULL));
		return 0;
	}
	if (c->o.precond == FEMGPU_PREC_AMG) {
		/* AMG_precond_setup (amg_precond.c:26-100) on the CSR matrix, R := M^-1 R */
		KR(fgh_blockcsr_amg_setup(&c->csr, c->neq, c->stream));
		c->have_bd = 1;
		if (c->o.solver == FEMGPU_PGMRES) KR(fg_amg_vcycle(c->csr.amg, c->R, c->R, NULL));
		return 0;
	}
	if (c->o.precond != FEMGPU_PREC_BLOCKDIAG) return 0;     /* NO_precond_setup */
	KR(fg_ebe_blockdiag_setup(c->ebe));
	c->ebe->have_bd = 1;
	c->have_bd = 1;
	if (c->o.solver == FEMGPU_PGMRES) KR(fg_ebe_blockdiag_apply(c->ebe, c->R, c->R, 0));
	return 0;
}

int femgpu_euler_precond_setup(femgpu_euler *c, double *R_host)
{
	if (!c) return FEMGPU_E_ARG;
	KR(femgpu_euler_precond_setup_dev(c));
	if (R_host)
		CK(cudaMemcpyAsync(R_host, c->R, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost,
		                   c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

static int solve(femgpu_euler *c, const double *B, double *X, int *iters)
{
	fg_linop op;
	double normb2;
	int it = 0, rc;
	if (c->o.precond != FEMGPU_PREC_NOT && !c->have_bd) {
		fgh_set_error("solve before precond_setup");
		return FEMGPU_E_NOT_BUILT;
	}
	if (iters) *iters = 0;
	CK(cudaMemsetAsync(X, 0, sizeof(double) * ((size_t)c->neq + 1), c->stream));      /* pgmres.c:46 */
	rc = fgh_kry_dot_host(&c->kry, B, B, c->neq, &normb2);
	if (rc) return rc;
	if (!(normb2 > 0.0)) return normb2 == 0.0 ? 0 : FEMGPU_E_BREAKDOWN;
	linop(c, &op);
	rc = fgh_kry_cycles(&c->kry, &op, B, X,
	                    c->o.solver == FEMGPU_PGMRES ? -1 : c->o.precision == FEMGPU_MIXED_IR ? 2 : 0,
	                    c->o.tol * sqrt(normb2), c->o.lmax, &it);
	if (iters) *iters = it;
	return rc;
}

int femgpu_euler_solve_dev(femgpu_euler *c, int *iters)
{
	if (!c) return FEMGPU_E_ARG;
	return solve(c, c->R, c->Da, iters);
}

int femgpu_euler_solve(femgpu_euler *c, const double *B_host, double *X_host, int *iters)
{
	int rc;
	if (!c) return FEMGPU_E_ARG;
	if (B_host)
		CK(cudaMemcpyAsync(c->R, B_host, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyHostToDevice,
		                   c->stream));
	rc = femgpu_euler_solve_dev(c, iters);
	if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;
	if (X_host)
		CK(cudaMemcpyAsync(X_host, c->Da, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost,
		                   c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return rc;
}

/* ---- Predictor_Old ------------------------------------------------------- */
static double elapsed(cudaEvent_t a, cudaEvent_t b)
{
	float ms = 0.0f;
	cudaEventElapsedTime(&ms, a, b);
	return 1e-3 * ms;
}

/* One multicorrection stage (Predictor_Old.c:68-126): ncorr correctors of
 * build, scaling, preconditioner set-up, solve and a += Da, u += coef Da;
 * then u to uhist[stage] and the iterations to iters[stage*ncorr...]. */
static int stage(femgpu_euler *c, double coef, int st, double *uhist, int *iters)
{
	size_t n1 = (size_t)c->neq + 1;
	int i, rc;
	for (i = 0; i < c->o.ncorr; i++) {
		int it = 0;
		CK(cudaEventRecord(c->ev[0], c->stream));
		KR(femgpu_euler_build_dev(c));                                      /* :71      */
		if (c->o.scaling) KR(femgpu_euler_scale_dev(c));                    /* :73      */
		CK(cudaEventRecord(c->ev[1], c->stream));
		KR(femgpu_euler_precond_setup_dev(c));                              /* :75      */
		CK(cudaEventRecord(c->ev[2], c->stream));
		rc = solve(c, c->R, c->Da, &it);                                    /* :111     */
		if (rc) return rc;
		CK(cudaEventRecord(c->ev[3], c->stream));
		KR(fg_euler_correct(c, coef));                                      /* :115-116 */
		CK(cudaEventSynchronize(c->ev[3]));
		c->times[0] += elapsed(c->ev[0], c->ev[1]);
		c->times[1] += elapsed(c->ev[1], c->ev[2]);
		c->times[2] += elapsed(c->ev[2], c->ev[3]);
		if (iters) iters[st * c->o.ncorr + i] = it;
	}
	if (uhist)
		CK(cudaMemcpyAsync(uhist + (size_t)st * n1, c->u, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	return 0;
}

static int predictor(femgpu_euler *c, int nsteps, double *uhist, int *iters)
{
	const double alpha = c->o.alpha, dt = c->o.dt;
	const size_t n1 = (size_t)c->neq + 1, nb = sizeof(double) * (size_t)c->neq;
	int step;
	memset(c->times, 0, sizeof c->times);
	c->alpha_build = alpha;                                  /* Alpha_Build = Alpha   */
	c->dt_build = dt;                                        /* DeltaT_Build = DeltaT */
	if (c->o.method != FEMGPU_TI_PREDICTOR1 && !c->u1) {
		DM(c->u1, sizeof(double) * n1);
		DM(c->u2, sizeof(double) * n1);
		DM(c->uold, sizeof(double) * n1);
	}
	if (c->o.method == FEMGPU_TI_BDF && nsteps > 0) {
		/* Predictor_Old_BDF.c:50-160: an implicit first step whose update
		 * keeps the deck's alpha, then BDF2 u = 4/3 u_n - 1/3 u_(n-1) with
		 * updates of 2/3 dt; the builds keep Alpha_Build and DeltaT_Build */
		const double four_thirds = 4.0/3.0, two_thirds = 2.0/3.0, one_third = 1.0/3.0;
		CK(cudaMemcpyAsync(c->u1, c->u, nb, cudaMemcpyDeviceToDevice, c->stream));
		CK(cudaMemsetAsync(c->a, 0, nb, c->stream));
		KR(stage(c, alpha*dt, 0, uhist, iters));
		CK(cudaMemcpyAsync(c->u2, c->u, nb, cudaMemcpyDeviceToDevice, c->stream));
		for (step = 1; step < nsteps; step++) {
			KR(fg_euler_lin(c, c->u2, c->u1, four_thirds, one_third));
			KR(stage(c, two_thirds*dt, step, uhist, iters));
			CK(cudaMemcpyAsync(c->u1, c->u2, nb, cudaMemcpyDeviceToDevice, c->stream));
			CK(cudaMemcpyAsync(c->u2, c->u, nb, cudaMemcpyDeviceToDevice, c->stream));
		}
	} else if (c->o.method == FEMGPU_TI_TRBDF2) {
		/* Predictor_Old_TRBDF2.c:34-165: per step a trapezoidal stage of
		 * lambda dt (alpha 1/2) and a BDF2 stage u = A u - B u_old (alpha
		 * 1/(2 - lambda)) over the rest; DeltaT_Build is the TR sub-step
		 * before the loop and the BDF2 sub-step from the first BDF2 stage on */
		const double lambda = 2.0 - sqrt(2.0);
		const double A = 1.0/(lambda*(2.0 - lambda));
		const double B = (1.0 - lambda)*(1.0 - lambda)/(lambda*(2.0 - lambda));
		const double dtTR = lambda*dt, dtBDF2 = (1.0 - lambda)*dt;
		const double a_tr = 0.5, a_bdf = 1.0/(2.0 - lambda);
		CK(cudaMemcpyAsync(c->uold, c->u, nb, cudaMemcpyDeviceToDevice, c->stream));
		c->dt_build = dtTR;
		for (step = 0; step < nsteps; step++) {
			KR(fg_euler_predict(c, a_tr*dtTR));                    /* u += alpha dtTR a, a = 0 */
			KR(stage(c, a_tr*dtTR, 2 * step, uhist, iters));
			c->dt_build = dtBDF2;
			KR(fg_euler_lin(c, c->u, c->uold, A, B));              /* u = A u - B u_old, a = 0 */
			KR(stage(c, a_bdf*dtBDF2, 2 * step + 1, uhist, iters));
			CK(cudaMemcpyAsync(c->uold, c->u, nb, cudaMemcpyDeviceToDevice, c->stream));
		}
	} else {
		const double c_pred = (1.0 - alpha) * dt, c_corr = alpha * dt;
		for (step = 0; step < nsteps; step++) {
			KR(fg_euler_predict(c, c_pred));                       /* :57-62   */
			KR(stage(c, c_corr, step, uhist, iters));
		}
	}
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_euler_set_build_params(femgpu_euler *c, double alpha_build, double dt_build)
{
	if (!c || !(dt_build > 0.0)) return FEMGPU_E_ARG;
	c->alpha_build = alpha_build;
	c->dt_build = dt_build;
	return 0;
}

int femgpu_euler_set_bubbles(femgpu_euler *c, const double *uB)
{
	const size_t nb = sizeof(double) * 4 * (size_t)(c ? c->nel : 0);
	if (!c) return FEMGPU_E_ARG;
	if (uB) CK(cudaMemcpyAsync(c->uB, uB, nb, cudaMemcpyHostToDevice, c->stream));
	else CK(cudaMemsetAsync(c->uB, 0, nb, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_euler_state(femgpu_euler *c, double *uB, double *delta_old)
{
	if (!c) return FEMGPU_E_ARG;
	if (uB) CK(cudaMemcpyAsync(uB, c->uB, sizeof(double) * 4 * (size_t)c->nel, cudaMemcpyDeviceToHost, c->stream));
	if (delta_old)
		CK(cudaMemcpyAsync(delta_old, c->dold, sizeof(double) * (size_t)c->nel, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_euler_predictor_dev(femgpu_euler *c, int nsteps, int *iters)
{
	if (!c || nsteps < 0) return FEMGPU_E_ARG;
	return predictor(c, nsteps, NULL, iters);
}

int femgpu_euler_predictor(femgpu_euler *c, double *u, int nsteps, double *uhist, int *iters)
{
	size_t n1;
	int rc;
	if (!c || nsteps < 0) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	if (u) CK(cudaMemcpyAsync(c->u, u, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	CK(cudaMemsetAsync(c->a, 0, sizeof(double) * n1, c->stream));          /* a = 0 (mycalloc, :18) */
	CK(cudaMemsetAsync(c->dold, 0, sizeof(double) * (size_t)c->nel, c->stream));   /* delta_old = 0 (:23) */
	CK(cudaMemsetAsync(c->uB, 0, sizeof(double) * 4 * (size_t)c->nel, c->stream));  /* uB_old = 0 (:22)   */
	rc = predictor(c, nsteps, uhist, iters);
	if (rc) return rc;
	if (u) CK(cudaMemcpyAsync(u, c->u, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}
