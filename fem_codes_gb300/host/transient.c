/*
 * The transient scalar transport driver (02_Transport_Equation/2D) on a
 * transport context: Build_M_K_R_SUPG / Build_M_K_R_DD on the device
 * (csrc/build.cu) and the predictor-multicorrector of
 * 00_CommonFiles/Time_Integration/Predictor_Old.c:3-148 with the stop
 * criteria of Criteria.c:22-79, every vector operation on the device and the
 * criteria's norms read back once per correction.  Plain C.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_internal.h"

int fg_dot(femgpu_transport *t, const double *a, const double *b, int n, double *out_dev);

static int dnorm(femgpu_transport *t, const double *a, double *out)
{
	KR(fg_dot(t, a, a, t->neq, &t->st->hdiag));
	CK(cudaMemcpyAsync(&t->st_host->hdiag, &t->st->hdiag, sizeof(double), cudaMemcpyDeviceToHost, t->stream));
	CK(cudaStreamSynchronize(t->stream));
	*out = sqrt(t->st_host->hdiag);
	return 0;
}

int femgpu_transport_set_transient(femgpu_transport *t, const femgpu_transient_opts *o)
{
	size_t n1;
	if (!t || !o) return FEMGPU_E_ARG;
	if ((o->stab != FEMGPU_STAB_SUPG && o->stab != FEMGPU_STAB_DD) || !(o->dt > 0.0) || o->max_corr < 1 ||
	    t->o.hshock == FEMGPU_H_SQRTAREA) {
		fgh_set_error("transient options: stab %d, dt %g, max_corr %d, h_shock %d", o->stab, o->dt, o->max_corr,
		              t->o.hshock);
		return FEMGPU_E_ARG;
	}
	if (t->o.shock == FEMGPU_SHOCK_CAUDD && o->stab != FEMGPU_STAB_DD) {
		fgh_set_error("CAUDD shock capturing belongs to the DD build (setStabilizationForm.c:67)");
		return FEMGPU_E_ARG;
	}
	n1 = (size_t)t->neq + 1;
	if (!t->du) {
		if (fgh_dmalloc((void **)&t->du, sizeof(double) * n1) ||
		    fgh_dmalloc((void **)&t->uold, sizeof(double) * n1) ||
		    fgh_dmalloc((void **)&t->Da, sizeof(double) * n1) ||
		    fgh_dmalloc((void **)&t->re, sizeof(double) * 12 * (size_t)t->nel) ||
		    fgh_dmalloc((void **)&t->dold, sizeof(double) * (size_t)t->nel))
			return FEMGPU_E_NOMEM;
		if (t->o.scheme != FEMGPU_EBE && !t->ke && fgh_dmalloc((void **)&t->ke, sizeof(double) * 9 * (size_t)t->nel))
			return FEMGPU_E_NOMEM;
	}
	CK(cudaMemsetAsync(t->du, 0, sizeof(double) * n1, t->stream));
	CK(cudaMemsetAsync(t->Da, 0, sizeof(double) * n1, t->stream));
	CK(cudaMemsetAsync(t->dold, 0, sizeof(double) * (size_t)t->nel, t->stream));
	t->tr = *o;
	t->transient = 1;
	t->built = 0;
	t->factored = 0;
	CK(cudaStreamSynchronize(t->stream));
	return 0;
}

static int build_transient_dev(femgpu_transport *t)
{
	KR(fg_build_transient(t, t->tr.stab == FEMGPU_STAB_DD, t->tr.alpha * t->tr.dt));
	KR(fg_assemble_transient(t));
	t->built = 1;
	t->factored = 0;
	return 0;
}

int femgpu_transport_build_transient(femgpu_transport *t, const double *u_host, const double *a_host,
		double *R_host, double *A_host)
{
	size_t n1;
	if (!t) return FEMGPU_E_ARG;
	if (!t->transient) { fgh_set_error("build_transient before set_transient"); return FEMGPU_E_NOT_BUILT; }
	n1 = (size_t)t->neq + 1;
	if (u_host) CK(cudaMemcpyAsync(t->u, u_host, sizeof(double) * n1, cudaMemcpyHostToDevice, t->stream));
	if (a_host) CK(cudaMemcpyAsync(t->du, a_host, sizeof(double) * n1, cudaMemcpyHostToDevice, t->stream));
	KR(build_transient_dev(t));
	if (R_host) CK(cudaMemcpyAsync(R_host, t->F, sizeof(double) * n1, cudaMemcpyDeviceToHost, t->stream));
	if (A_host) {
		size_t nA = t->o.scheme == FEMGPU_CSR ? (size_t)t->nnz + 1
		          : t->o.scheme == FEMGPU_EDE ? 4 * ((size_t)t->nedge + 1) : 9 * (size_t)t->nel;
		CK(cudaMemcpyAsync(A_host, t->A, sizeof(double) * nA, cudaMemcpyDeviceToHost, t->stream));
	}
	CK(cudaStreamSynchronize(t->stream));
	CK(cudaMemcpy(t->st_host, t->st, sizeof(fg_status), cudaMemcpyDeviceToHost));
	if (t->st_host->err) {
		fgh_set_error("device reported error %d", t->st_host->err);
		return t->st_host->err;
	}
	return 0;
}

/* Criteria.c:22-38 */
static int stop_corr(const femgpu_transient_opts *o, double norm_a, double norm_Da, int i)
{
	if (o->stop_norm) return norm_Da < o->nonlin_tol * norm_a || i >= o->max_corr;
	return i >= o->max_corr;
}

int femgpu_transport_predictor(femgpu_transport *t, const double *u0_host, int max_steps, double *u_hist,
		double *t_hist, int *ncorr, int *iters, int iters_cap)
{
	const femgpu_transient_opts *o;
	size_t n1;
	int step = 0, tag = 1, rc, done;
	double time = 0.0, c1, c2;
	if (!t || !u0_host || max_steps < 1 || (iters && iters_cap < 1)) return FEMGPU_E_ARG;
	if (!t->transient) { fgh_set_error("predictor before set_transient"); return FEMGPU_E_NOT_BUILT; }
	o = &t->tr;
	n1 = (size_t)t->neq + 1;
	/* Predictor_Old.c:16-45: a, delta_old zeroed, u = InitialSolution */
	CK(cudaMemcpyAsync(t->u, u0_host, sizeof(double) * n1, cudaMemcpyHostToDevice, t->stream));
	CK(cudaMemsetAsync(t->du, 0, sizeof(double) * n1, t->stream));
	CK(cudaMemsetAsync(t->dold, 0, sizeof(double) * (size_t)t->nel, t->stream));
	c1 = (1.0 - o->alpha) * o->dt;
	c2 = o->alpha * o->dt;
	do {
		double norm_a, norm_Da;
		int i = 0;
		step++;
		time += o->dt;
		KR(fg_tr_predict(t, c1));
		KR(dnorm(t, t->du, &norm_a));
		norm_Da = norm_a + 1.0;
		do {
			int it = 0;
			i++;
			KR(build_transient_dev(t));
			KR(femgpu_transport_precond_setup_dev(t, tag++));
			rc = fgh_transport_gmres(t, t->F, t->Da, &it);
			if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;    /* gmres stops at lmax cycles, as pgmres */
			if (iters && i <= iters_cap) iters[(size_t)(step - 1) * iters_cap + (i - 1)] = it;
			KR(fg_tr_correct(t, c2));
			KR(dnorm(t, t->du, &norm_a));
			KR(dnorm(t, t->Da, &norm_Da));
		} while (!stop_corr(o, norm_a, norm_Da, i));
		if (u_hist) CK(cudaMemcpyAsync(u_hist + (size_t)(step - 1) * n1, t->u, sizeof(double) * n1,
		                               cudaMemcpyDeviceToHost, t->stream));
		if (t_hist) t_hist[step - 1] = time;
		if (ncorr) ncorr[step - 1] = i;
		/* Criteria.c:41-79 */
		if (o->steady_stop) {
			double norm_u, norm_diff;
			KR(fg_tr_diff(t));                                    /* Da := u - u_old */
			KR(dnorm(t, t->Da, &norm_diff));
			KR(dnorm(t, t->u, &norm_u));
			done = o->time_tol * norm_u > norm_diff || fabs(o->final_time - time) < o->dt;
		} else {
			done = fabs(o->final_time - time) < 1e-15;
		}
		CK(cudaStreamSynchronize(t->stream));
	} while (!done && step < max_steps);
	return step;
}
