/*
 * Host driver of the steady Navier-Stokes path: the control flow of the
 * reference's Process (04_SS_NavierStokes_Equations/2D/01_CommonFiles/
 * Process.c:62-194: damped Newton with backtracking on ||F||, F the
 * preconditioned residual) and its forcing terms (eta_newton.c:5-68)
 * around device kernels for the VMS build, the 3-dof block-EBE operator with
 * the nodal block-diagonal preconditioner or the CSR operator with ILU(0)
 * (the drivers' two configurations), and GMRES.  Plain C.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_ns.h"
#include "../csrc/fg_amg.h"

#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)

void femgpu_ns_default_opts(femgpu_ns_opts *o)
{
	memset(o, 0, sizeof *o);
	o->re = 1000.0;
	o->velmax = 1.0;
	o->precond = FEMGPU_PREC_BLOCKDIAG;
	o->solver = FEMGPU_PGMRES;
	o->kmax = 50;
	o->lmax = 100;
	o->eta0 = 0.1;
	o->eta_case = 2;
	o->tol_nl = 1e-8;
}

static int op_matvec(void *ctx, const double *p, double *q, const int *active)
{
	(void)active;
	return fg_ebe_matvec(((femgpu_ns *)ctx)->ebe, p, q, 0);
}

static int op_precond(void *ctx, const double *p, double *z, const int *active)
{
	(void)active;
	return fg_ebe_blockdiag_apply(((femgpu_ns *)ctx)->ebe, p, z, 0);
}

/* CSR storage: csrmv and ILUp_precond */
static int op_matvec_csr(void *ctx, const double *p, double *q, const int *active)
{
	femgpu_ns *c = (femgpu_ns *)ctx;
	return fg_csrmv64(c->neq, c->csr.IA, c->csr.JA, c->csr.AA, p, q, active, c->stream);
}

static int op_precond_ilu(void *ctx, const double *p, double *z, const int *active)
{
	return fg_ilu0_apply64(((femgpu_ns *)ctx)->csr.ilu, p, z, active);
}

/* CSR storage: AMG_precond, one V-cycle */
static int op_precond_amg(void *ctx, const double *p, double *z, const int *active)
{
	return fg_amg_vcycle(((femgpu_ns *)ctx)->csr.amg, p, z, active);
}

static int up(double **dst, const double *src, size_t n)
{
	int rc = fgh_dmalloc((void **)dst, sizeof(double) * n);
	if (rc) return rc;
	if (src) CK(cudaMemcpy(*dst, src, sizeof(double) * n, cudaMemcpyHostToDevice));
	else CK(cudaMemset(*dst, 0, sizeof(double) * n));
	return 0;
}

static int create(femgpu_ns *c, const femgpu_ns_opts *o, int nnodes, const double *x, const double *y, int nel,
                  const int *vert, const int *node_id, int neq, const double *upresc, const double *f)
{
	size_t n1 = (size_t)neq + 1;
	int rc;
	c->o = *o;
	c->nnodes = nnodes; c->nel = nel; c->neq = neq;
	c->tol = o->eta0;
	rc = femgpu_ebe_create(&c->ebe, 3, nnodes, nel, vert, node_id, neq);
	if (rc) return rc;
	CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
	c->stream = c->own_stream;
	KR(femgpu_ebe_set_stream(c->ebe, c->stream));
	if ((rc = up(&c->x, x, (size_t)nnodes)) || (rc = up(&c->y, y, (size_t)nnodes)) ||
	    (rc = up(&c->upresc, upresc, 3 * (size_t)nnodes)) || (rc = up(&c->f, f, 2 * (size_t)nnodes)))
		return rc;
	if ((rc = up(&c->u, NULL, n1)) || (rc = up(&c->F, NULL, n1)) || (rc = up(&c->s, NULL, n1)) ||
	    (rc = up(&c->Fold, NULL, n1)) || (rc = up(&c->Re, NULL, 9 * (size_t)nel)) ||
	    (rc = up(&c->dold, NULL, (size_t)nel)) || (rc = up(&c->nold, NULL, (size_t)nel)))
		return rc;
	rc = fgh_kry_alloc(&c->kry, neq, o->kmax, o->solver == FEMGPU_FGMRES ? 1 : 0, c->stream);
	if (rc) return rc;
	if (o->scheme == FEMGPU_CSR &&
	    (rc = fgh_blockcsr_create(&c->csr, 9, c->ebe, c->nel, c->neq, c->stream, o->precond == FEMGPU_PREC_ILU0,
	                              o->solver, o->ilu_blocks))) return rc;
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_ns_create(femgpu_ns **out, const femgpu_ns_opts *opts, int nnodes, const double *x, const double *y,
                     int nel, const int *vert, const int *node_id, int neq, const double *upresc, const double *f)
{
	femgpu_ns_opts o;
	femgpu_ns *c;
	int rc;
	if (!out) return FEMGPU_E_ARG;
	*out = NULL;
	if (opts) o = *opts; else femgpu_ns_default_opts(&o);
	if (nnodes <= 0 || nel <= 0 || neq <= 0 || !x || !y || !vert || !node_id || !upresc || !(o.re > 0.0) ||
	    o.kmax < 1 || o.lmax < 1 || o.eta_case < 0 || o.eta_case > 4 || !(o.eta0 > 0.0) ||
	    (o.scheme != FEMGPU_EBE && o.scheme != FEMGPU_CSR) || o.ilu_blocks < 0 ||
	    (o.precond != FEMGPU_PREC_NOT && o.precond != FEMGPU_PREC_BLOCKDIAG && o.precond != FEMGPU_PREC_ILU0 &&
	     o.precond != FEMGPU_PREC_AMG) ||
	    (o.precond == FEMGPU_PREC_AMG && o.scheme != FEMGPU_CSR) ||
	    (o.precond == FEMGPU_PREC_BLOCKDIAG && o.scheme != FEMGPU_EBE) ||     /* setPreconditioner.c:54-73 */
	    (o.precond == FEMGPU_PREC_ILU0 && o.scheme != FEMGPU_CSR) ||
	    (o.solver != FEMGPU_PGMRES && o.solver != FEMGPU_FGMRES)) {
		fgh_set_error("femgpu_ns_create: bad argument or option");
		return FEMGPU_E_ARG;
	}
	c = calloc(1, sizeof *c);
	if (!c) return FEMGPU_E_NOMEM;
	rc = create(c, &o, nnodes, x, y, nel, vert, node_id, neq, upresc, f);
	if (rc) { femgpu_ns_destroy(c); return rc; }
	*out = c;
	return 0;
}

void femgpu_ns_destroy(femgpu_ns *c)
{
	int i;
	if (!c) return;
	if (c->stream) cudaStreamSynchronize(c->stream);
	fgh_blockcsr_destroy(&c->csr);
	if (c->ebe) femgpu_ebe_destroy(c->ebe);
	{
		void *p[] = { c->x, c->y, c->upresc, c->f, c->u, c->F, c->s, c->Fold, c->Re, c->dold, c->nold };
		for (i = 0; i < (int)(sizeof p / sizeof p[0]); i++) if (p[i]) cudaFree(p[i]);
	}
	fgh_kry_free(&c->kry);
	if (c->own_stream) cudaStreamDestroy(c->own_stream);
	free(c);
}

int femgpu_ns_set_stream(femgpu_ns *c, void *stream)
{
	if (!c) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(c->stream));
	c->stream = stream ? (cudaStream_t)stream : c->own_stream;
	c->kry.stream = c->stream;
	fgh_blockcsr_set_stream(&c->csr, c->stream);
	KR(femgpu_ebe_set_stream(c->ebe, c->stream));
	return 0;
}

double *femgpu_ns_u_dev(femgpu_ns *c) { return c ? c->u : NULL; }
femgpu_ebe *femgpu_ns_ebe(femgpu_ns *c) { return c ? c->ebe : NULL; }

int femgpu_ns_reset(femgpu_ns *c)
{
	if (!c) return FEMGPU_E_ARG;
	CK(cudaMemsetAsync(c->dold, 0, sizeof(double) * (size_t)c->nel, c->stream));
	CK(cudaMemsetAsync(c->nold, 0, sizeof(double) * (size_t)c->nel, c->stream));
	c->nbuild = 0;
	c->setup_tag = 0;
	c->tol = c->o.eta0;
	return 0;
}

int femgpu_ns_build_dev(femgpu_ns *c)
{
	if (!c) return FEMGPU_E_ARG;
	KR(fg_ns_build(c, c->nbuild == 0));
	if (c->o.scheme == FEMGPU_CSR)                              /* csr_assembly, element by element */
		KR(fgh_blockcsr_assemble(&c->csr, 9, c->ebe, c->neq, c->stream));
	c->nbuild++;
	c->have_bd = 0;
	return 0;
}

int femgpu_ns_csr(femgpu_ns *c, int *n_nnz, int *IA, int *JA, double *AA)
{
	if (!c || !n_nnz || c->o.scheme != FEMGPU_CSR) return FEMGPU_E_ARG;
	n_nnz[0] = c->neq; n_nnz[1] = c->csr.nnz;
	if (IA) CK(cudaMemcpyAsync(IA, c->csr.IA, sizeof(int) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost,
	                           c->stream));
	if (JA) CK(cudaMemcpyAsync(JA, c->csr.JA, sizeof(int) * (size_t)c->csr.nnz, cudaMemcpyDeviceToHost, c->stream));
	if (AA) CK(cudaMemcpyAsync(AA, c->csr.AA, sizeof(double) * ((size_t)c->csr.nnz + 1), cudaMemcpyDeviceToHost,
	                           c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_ns_build(femgpu_ns *c, const double *u, double *Ae_host, double *F_host)
{
	size_t n1;
	if (!c) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	if (u) CK(cudaMemcpyAsync(c->u, u, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	KR(femgpu_ns_build_dev(c));
	if (Ae_host)
		CK(cudaMemcpyAsync(Ae_host, c->ebe->A, sizeof(double) * 81 * (size_t)c->nel, cudaMemcpyDeviceToHost,
		                   c->stream));
	if (F_host) CK(cudaMemcpyAsync(F_host, c->F, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

static int setup_dev(femgpu_ns *c)
{
	if (!c->nbuild) { fgh_set_error("precond_setup before build"); return FEMGPU_E_NOT_BUILT; }
	c->setup_tag++;
	if (c->o.precond == FEMGPU_PREC_ILU0) {
		/* ILUp_precond_setup.c:8-167 at fill level 0, then F := M^-1 F */
		KR(fgh_blockcsr_factor(&c->csr, c->stream));
		c->have_bd = 1;
		if (c->o.solver == FEMGPU_PGMRES) KR(fg_ilu0_apply64(c->csr.ilu, c->F, c->F, NULL));
		return 0;
	}
	if (c->o.precond == FEMGPU_PREC_AMG) {
		/* AMG_precond_setup (amg_precond.c:26-100): the hierarchy of the
		 * current CSR matrix on the host, then F := M^-1 F */
		KR(fgh_blockcsr_amg_setup(&c->csr, c->neq, c->stream));
		c->have_bd = 1;
		if (c->o.solver == FEMGPU_PGMRES) KR(fg_amg_vcycle(c->csr.amg, c->F, c->F, NULL));
		return 0;
	}
	if (c->o.precond != FEMGPU_PREC_BLOCKDIAG) return 0;
	KR(fg_ebe_blockdiag_setup(c->ebe));
	c->ebe->have_bd = 1;
	c->have_bd = 1;
	if (c->o.solver == FEMGPU_PGMRES) KR(fg_ebe_blockdiag_apply(c->ebe, c->F, c->F, 0));
	return 0;
}

int femgpu_ns_precond_setup(femgpu_ns *c, double *F_host)
{
	if (!c) return FEMGPU_E_ARG;
	KR(setup_dev(c));
	if (F_host)
		CK(cudaMemcpyAsync(F_host, c->F, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost,
		                   c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

static int solve(femgpu_ns *c, const double *B, double *X, int *iters)
{
	fg_linop op;
	double nb2;
	int it = 0, rc;
	if (c->o.precond != FEMGPU_PREC_NOT && !c->have_bd) {
		fgh_set_error("solve before precond_setup");
		return FEMGPU_E_NOT_BUILT;
	}
	*iters = 0;
	CK(cudaMemsetAsync(X, 0, sizeof(double) * ((size_t)c->neq + 1), c->stream));       /* pgmres.c:46 */
	if ((rc = fgh_kry_dot_host(&c->kry, B, B, c->neq, &nb2))) return rc;
	if (!(nb2 > 0.0)) return nb2 == 0.0 ? 0 : FEMGPU_E_BREAKDOWN;
	memset(&op, 0, sizeof op);
	op.ctx = c;
	op.matvec = c->o.scheme == FEMGPU_CSR ? op_matvec_csr : op_matvec;
	op.precond = c->o.precond == FEMGPU_PREC_BLOCKDIAG ? op_precond
	           : c->o.precond == FEMGPU_PREC_ILU0 ? op_precond_ilu
	           : c->o.precond == FEMGPU_PREC_AMG ? op_precond_amg : NULL;
	rc = fgh_kry_cycles(&c->kry, &op, B, X, c->o.solver == FEMGPU_PGMRES ? -1 : 0, c->tol * sqrt(nb2), c->o.lmax,
	                    &it);
	*iters = it;
	return rc;
}

int femgpu_ns_set_amg(femgpu_ns *c, femgpu_amg *g)
{
	if (!c || !g || c->o.precond != FEMGPU_PREC_AMG) return FEMGPU_E_ARG;
	KR(femgpu_amg_set_stream(g, c->stream));
	c->csr.amg = g;
	c->have_bd = 0;
	return 0;
}

int femgpu_ns_set_tol(femgpu_ns *c, double tol)
{
	if (!c || !(tol > 0.0)) return FEMGPU_E_ARG;
	c->tol = tol;
	return 0;
}

int femgpu_ns_solve(femgpu_ns *c, const double *B_host, double *X_host, int *iters)
{
	int it = 0, rc;
	if (!c) return FEMGPU_E_ARG;
	if (B_host)
		CK(cudaMemcpyAsync(c->F, B_host, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyHostToDevice,
		                   c->stream));
	rc = solve(c, c->F, c->s, &it);
	if (iters) *iters = it;
	if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;
	if (X_host)
		CK(cudaMemcpyAsync(X_host, c->s, sizeof(double) * ((size_t)c->neq + 1), cudaMemcpyDeviceToHost,
		                   c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return rc;
}

/* eta_newton.c:5-68 (forcing term of the inexact Newton step) from ||F||
 * and ||Fold||. */
static double eta_newton(int ecase, double nF, double nFold, double etaold, int pricek, int it, double talnl,
                         double eta0)
{
	double ratio = nF / nFold, eta = 0.0, lim, cand;
	if (ecase == 1) {
		eta = eta0 < ratio ? eta0 : ratio * ratio;
	} else if (ecase == 2 || ecase == 3) {
		double alpha = ecase == 2 ? 2. : (1. + sqrt(5)) * 0.5, gamma = ecase == 2 ? 0.9 : 1.0;
		double beta = ecase == 2 ? 0.1 : 0.;
		double etaa = gamma * pow(ratio, alpha), prev = gamma * pow(etaold, alpha);
		if (prev < beta) {
			eta = eta0 < etaa ? eta0 : etaa;
		} else {
			cand = etaa > prev ? etaa : prev;
			eta = eta0 < cand ? eta0 : cand;
		}
	} else if (ecase == 4) {
		double ak = log10(nF) - log10(nFold), bk = log10(pricek);
		double theta = bk / sqrt(ak * ak + bk * bk);
		double gamma = pow(1. / (it + 1), 1.1) * cos(theta) * cos(theta);
		double etaa = gamma * ratio;
		eta = eta0 < etaa ? eta0 : etaa;
	}
	lim = 0.5 * talnl / nF;
	cand = eta > lim ? eta : lim;
	eta = eta0 < cand ? eta0 : cand;
	if (ecase == 0) eta = eta0;
	return eta;
}

static int norm_dev(femgpu_ns *c, const double *v, double *out)
{
	double s2;
	int rc = fgh_kry_dot_host(&c->kry, v, v, c->neq, &s2);
	*out = sqrt(s2);
	return rc;
}

int femgpu_ns_newton(femgpu_ns *c, int maxit, double *u_host, double *uhist, double *normF, double *wout,
                     int *gmres)
{
	const double w_min = 0.05, c1 = 1.001, c2 = 1.1, c3 = 1.001, c4 = 0.9, c5 = 0.5;
	double w_max = 1.00, w = w_max, w_old = 0.0, norm_F, norm_Fold, epsilon;
	size_t n1;
	int it, iter = 0, iterold, pricek, fd, cont, nit = 0, rc;
	if (!c || maxit < 0) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	KR(femgpu_ns_reset(c));
	CK(cudaMemsetAsync(c->u, 0, sizeof(double) * n1, c->stream));                      /* Process.c:42-47 */
	CK(cudaMemsetAsync(c->s, 0, sizeof(double) * n1, c->stream));
	KR(femgpu_ns_build_dev(c));                                                         /* :62 */
	it = 1;
	KR(setup_dev(c));                                                                   /* :68 */
	if ((rc = norm_dev(c, c->F, &norm_F))) return rc;
	epsilon = c->o.tol_nl * norm_F;
	pricek = 1;
	CK(cudaMemcpyAsync(c->Fold, c->F, sizeof(double) * n1, cudaMemcpyDeviceToDevice, c->stream));
	while (norm_F > epsilon && it < 2000 && nit < maxit) {                              /* :92 */
		int its = 0;
		it++;
		iterold = iter;
		if ((rc = norm_dev(c, c->Fold, &norm_Fold))) return rc;
		rc = solve(c, c->F, c->s, &its);                                                /* :111 */
		if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;
		iter += its;
		pricek = iter - iterold + 1;
		fd = 1;
		cont = 1;
		do {                                                                            /* :127-176 */
			double etaold = c->tol;
			w_old = w;
			KR(fg_ns_axpy(c, w, c->s, c->u));
			KR(femgpu_ns_build_dev(c));
			KR(setup_dev(c));
			if ((rc = norm_dev(c, c->F, &norm_F))) return rc;
			c->tol = eta_newton(c->o.eta_case, norm_F, norm_Fold, etaold, pricek, it, epsilon, c->o.eta0);
			if (norm_F < norm_Fold || w < c1 * w_min) {
				if (norm_F < norm_Fold && fd == 1) {
					w_max = (1.0 < c3 * w_max) ? 1.0 : c3 * w_max;
					w = (w_max < c2 * w) ? w_max : c2 * w;
				}
				cont = 0;
			} else {
				w = (w_min > c5 * w) ? w_min : c5 * w;
				if (fd == 1) {
					w_max = (w_min > c4 * w_max) ? w_min : c4 * w_max;
					fd = 0;
				}
				KR(fg_ns_axpy(c, -1. * w_old, c->s, c->u));
			}
		} while (cont == 1);
		CK(cudaMemcpyAsync(c->Fold, c->F, sizeof(double) * n1, cudaMemcpyDeviceToDevice, c->stream));
		if (uhist)
			CK(cudaMemcpyAsync(uhist + (size_t)nit * n1, c->u, sizeof(double) * n1, cudaMemcpyDeviceToHost,
			                   c->stream));
		if (normF) normF[nit] = norm_F;
		if (wout) wout[nit] = w_old;
		if (gmres) gmres[nit] = pricek - 1;
		nit++;
	}
	if (u_host) CK(cudaMemcpyAsync(u_host, c->u, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return nit;
}
