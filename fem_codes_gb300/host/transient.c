/*
 * The transient scalar transport driver (02_Transport_Equation/2D) on a
 * transport context: Build_M_K_R_SUPG / Build_M_K_R_DD / Build_M_F_DD on the
 * device (csrc/build.cu) and the predictor-multicorrectors of
 * 00_CommonFiles/Time_Integration (Predictor_Old.c:3-148 and its BDF /
 * TRBDF2 forms, Predictor_New.c and its BDF / TRBDF2 forms) with the stop
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
	if (o->method < FEMGPU_TI_PREDICTOR1 || o->method > FEMGPU_TI_PREDICTOR2_TRBDF2 ||
	    (o->method >= FEMGPU_TI_PREDICTOR2 && o->stab != FEMGPU_STAB_DD)) {
		fgh_set_error("time integration %d with stabilisation %d (setStabilizationForm.c:7-61)", o->method, o->stab);
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
	if (o->method >= FEMGPU_TI_PREDICTOR2 && !t->uB) {
		if (fgh_dmalloc((void **)&t->uB, sizeof(double) * (size_t)t->nel) ||
		    fgh_dmalloc((void **)&t->aB, sizeof(double) * (size_t)t->nel) ||
		    fgh_dmalloc((void **)&t->bub, sizeof(double) * 5 * (size_t)t->nel))
			return FEMGPU_E_NOMEM;
	}
	if (o->method > FEMGPU_TI_PREDICTOR2 && !t->uB1) {
		if (fgh_dmalloc((void **)&t->uB1, sizeof(double) * (size_t)t->nel) ||
		    fgh_dmalloc((void **)&t->uB2, sizeof(double) * (size_t)t->nel))
			return FEMGPU_E_NOMEM;
	}
	if (t->uB) {
		CK(cudaMemsetAsync(t->uB, 0, sizeof(double) * (size_t)t->nel, t->stream));
		CK(cudaMemsetAsync(t->aB, 0, sizeof(double) * (size_t)t->nel, t->stream));
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

int femgpu_transport_set_bubbles(femgpu_transport *t, const double *uB_host, const double *aB_host)
{
	if (!t) return FEMGPU_E_ARG;
	if (!t->transient || !t->uB) { fgh_set_error("set_bubbles: not a Predictor2 context"); return FEMGPU_E_NOT_BUILT; }
	if (uB_host) CK(cudaMemcpyAsync(t->uB, uB_host, sizeof(double) * (size_t)t->nel, cudaMemcpyHostToDevice, t->stream));
	if (aB_host) CK(cudaMemcpyAsync(t->aB, aB_host, sizeof(double) * (size_t)t->nel, cudaMemcpyHostToDevice, t->stream));
	CK(cudaStreamSynchronize(t->stream));
	return 0;
}

static int build_transient_dev(femgpu_transport *t)
{
	if (t->tr.method >= FEMGPU_TI_PREDICTOR2) KR(fg_build_mfdd(t, t->tr.alpha * t->tr.dt));
	else KR(fg_build_transient(t, t->tr.stab == FEMGPU_STAB_DD, t->tr.alpha * t->tr.dt));
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

/* The loop's bookkeeping: the reference's Parameters->Alpha / DeltaT (the
 * SUPG build's Alpha*DeltaT) and Alpha_Build / DeltaT_Build (the DD build's),
 * the stage counter and the history arrays. */
typedef struct {
	femgpu_transport *t;
	double Alpha, DeltaT, AlphaB, DeltaTB;
	int tag, stage, bubble;
	double *u_hist;
	int *ncorr, *iters, iters_cap;
} tr_loop;

/* One multicorrection loop (Predictor_Old.c:87-134 and its BDF / TRBDF2
 * forms): corrections until the criterion holds; u += c Da each time. */
static int multicorrect(tr_loop *L, double c)
{
	femgpu_transport *t = L->t;
	const femgpu_transient_opts *o = &t->tr;
	const int dd = o->stab == FEMGPU_STAB_DD;
	double norm_a, norm_Da;
	int i = 0, rc;
	do {
		int it = 0;
		i++;
		if (L->bubble) KR(fg_build_mfdd(t, L->AlphaB * L->DeltaTB));
		else KR(fg_build_transient(t, dd, dd ? L->AlphaB * L->DeltaTB : L->Alpha * L->DeltaT));
		KR(fg_assemble_transient(t));
		t->built = 1;
		t->factored = 0;
		KR(femgpu_transport_precond_setup_dev(t, L->tag++));
		rc = fgh_transport_gmres(t, t->F, t->Da, &it);
		if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;    /* gmres stops at lmax cycles, as pgmres */
		if (L->iters && i <= L->iters_cap) L->iters[(size_t)L->stage * L->iters_cap + (i - 1)] = it;
		if (L->bubble) KR(fg_bubble_correct(t, c));          /* calculate_DaB, aB, uB */
		KR(fg_tr_correct(t, c));
		KR(dnorm(t, t->du, &norm_a));
		KR(dnorm(t, t->Da, &norm_Da));
	} while (!stop_corr(o, norm_a, norm_Da, i));
	if (L->u_hist)
		CK(cudaMemcpyAsync(L->u_hist + (size_t)L->stage * ((size_t)t->neq + 1), t->u,
		                   sizeof(double) * ((size_t)t->neq + 1), cudaMemcpyDeviceToHost, t->stream));
	if (L->ncorr) L->ncorr[L->stage] = i;
	L->stage++;
	return 0;
}

/* Criteria.c:41-79 on u and the method's u_old. */
static int stop_time(tr_loop *L, const double *uold, double time, int *done)
{
	femgpu_transport *t = L->t;
	const femgpu_transient_opts *o = &t->tr;
	if (o->steady_stop) {
		double norm_u, norm_diff;
		if (uold != t->uold)
			CK(cudaMemcpyAsync(t->uold, uold, sizeof(double) * (size_t)t->neq, cudaMemcpyDeviceToDevice, t->stream));
		KR(fg_tr_diff(t));                                    /* Da := u - u_old */
		KR(dnorm(t, t->Da, &norm_diff));
		KR(dnorm(t, t->u, &norm_u));
		*done = o->time_tol * norm_u > norm_diff || fabs(o->final_time - time) < L->DeltaT;
	} else {
		*done = fabs(o->final_time - time) < 1e-15;
	}
	return 0;
}

int femgpu_transport_predictor(femgpu_transport *t, const double *u0_host, int max_steps, double *u_hist,
		double *t_hist, int *ncorr, int *iters, int iters_cap)
{
	const femgpu_transient_opts *o;
	size_t n1, nb;
	int step = 0, done = 0;
	double time = 0.0, alpha, dt;
	tr_loop L;
	if (!t || !u0_host || max_steps < 1 || (iters && iters_cap < 1)) return FEMGPU_E_ARG;
	if (!t->transient) { fgh_set_error("predictor before set_transient"); return FEMGPU_E_NOT_BUILT; }
	o = &t->tr;
	n1 = (size_t)t->neq + 1;
	nb = sizeof(double) * (size_t)t->neq;
	if (o->method != FEMGPU_TI_PREDICTOR1 && !t->u1 &&
	    (fgh_dmalloc((void **)&t->u1, sizeof(double) * n1) || fgh_dmalloc((void **)&t->u2, sizeof(double) * n1)))
		return FEMGPU_E_NOMEM;
	/* a, delta_old zeroed, u = InitialSolution (Predictor_Old.c:16-45) */
	CK(cudaMemcpyAsync(t->u, u0_host, sizeof(double) * n1, cudaMemcpyHostToDevice, t->stream));
	CK(cudaMemsetAsync(t->du, 0, sizeof(double) * n1, t->stream));
	CK(cudaMemsetAsync(t->dold, 0, sizeof(double) * (size_t)t->nel, t->stream));
	alpha = o->alpha;
	dt = o->dt;
	memset(&L, 0, sizeof L);
	L.t = t; L.tag = 1; L.u_hist = u_hist; L.ncorr = ncorr; L.iters = iters; L.iters_cap = iters_cap;
	L.Alpha = alpha; L.DeltaT = dt; L.AlphaB = alpha; L.DeltaTB = dt;

	if (o->method == FEMGPU_TI_PREDICTOR2) {
		/* Predictor_New.c:52-123 */
		const double c1 = (1.0 - alpha) * dt, c2 = alpha * dt;
		KR(fg_bubble_init(t));                                /* uB_InitialSolution, aB = 0 */
		L.bubble = 1;
		do {
			step++;
			time += dt;
			KR(fg_tr_predict(t, c1));                         /* u_old = u, u += c1 a, a = 0 */
			KR(fg_bubble_predict(t, c1));                     /* uB += c1 aB, aB = 0 */
			KR(multicorrect(&L, c2));
			if (t_hist) t_hist[step - 1] = time;
			KR(stop_time(&L, t->uold, time, &done));
		} while (!done && step < max_steps);
	} else if (o->method == FEMGPU_TI_PREDICTOR2_BDF) {
		/* Predictor_New_BDF.c:56-198: uB starts at zero (the file's
		 * uB_InitialSolution call is commented out); one implicit step
		 * built with Alpha_Build = 1, then BDF2 on u and uB with
		 * Alpha_Build = 2/3; u_old is u before each BDF2 prediction */
		const double four_thirds = 4.0/3.0, two_thirds = 2.0/3.0, one_third = 1.0/3.0;
		const size_t nbB = sizeof(double) * (size_t)t->nel;
		L.bubble = 1;
		CK(cudaMemsetAsync(t->uB, 0, nbB, t->stream));
		CK(cudaMemsetAsync(t->aB, 0, nbB, t->stream));
		step = 1;
		time += dt;
		L.Alpha = 1.0;
		L.AlphaB = 1.0;
		CK(cudaMemcpyAsync(t->u1, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		CK(cudaMemcpyAsync(t->uB1, t->uB, nbB, cudaMemcpyDeviceToDevice, t->stream));
		KR(multicorrect(&L, dt));
		CK(cudaMemcpyAsync(t->u2, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		CK(cudaMemcpyAsync(t->uB2, t->uB, nbB, cudaMemcpyDeviceToDevice, t->stream));
		if (t_hist) t_hist[0] = time;
		L.Alpha = two_thirds;
		L.AlphaB = two_thirds;
		while (step < max_steps) {
			step++;
			time += dt;
			CK(cudaMemcpyAsync(t->uold, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
			KR(fg_tr_lin(t, t->u2, t->u1, four_thirds, one_third));    /* u = 4/3 u2 - 1/3 u1, a = 0 */
			KR(fg_bubble_lin(t, t->uB2, t->uB1, four_thirds, one_third));
			KR(multicorrect(&L, two_thirds * dt));
			CK(cudaMemcpyAsync(t->u1, t->u2, nb, cudaMemcpyDeviceToDevice, t->stream));
			CK(cudaMemcpyAsync(t->u2, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
			CK(cudaMemcpyAsync(t->uB1, t->uB2, nbB, cudaMemcpyDeviceToDevice, t->stream));
			CK(cudaMemcpyAsync(t->uB2, t->uB, nbB, cudaMemcpyDeviceToDevice, t->stream));
			if (t_hist) t_hist[step - 1] = time;
			KR(stop_time(&L, t->uold, time, &done));
			if (done) break;
		}
	} else if (o->method == FEMGPU_TI_PREDICTOR2_TRBDF2) {
		/* Predictor_New_TRBDF2.c:52-199: TR then BDF2 stages on u and uB,
		 * DeltaT_Build and Alpha_Build set per stage; uB_old starts at zero
		 * and u_old at the initial solution, both copied after each BDF2
		 * stage */
		const double lambda = 2.0 - sqrt(2.0);
		const double A = 1.0/(lambda*(2.0 - lambda));
		const double B = (1.0 - lambda)*(1.0 - lambda)/(lambda*(2.0 - lambda));
		const double dtTR = lambda*dt, dtBDF2 = (1.0 - lambda)*dt;
		const size_t nbB = sizeof(double) * (size_t)t->nel;
		double *u_old = t->u1, *uB_old = t->uB1;
		L.bubble = 1;
		KR(fg_bubble_init(t));                                /* uB_InitialSolution, aB = 0 */
		CK(cudaMemsetAsync(uB_old, 0, nbB, t->stream));
		CK(cudaMemcpyAsync(u_old, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		do {
			const double a_tr = 0.5, a_bdf = 1.0/(2.0 - lambda);
			L.DeltaT = dtTR;
			L.DeltaTB = dtTR;
			L.Alpha = a_tr;
			L.AlphaB = a_tr;
			step++;
			time += dtTR;
			KR(fg_tr_axpy_zero(t, a_tr*dtTR));                  /* u += alpha dtTR a, a = 0 */
			KR(fg_bubble_predict(t, a_tr*dtTR));                /* uB += alpha dtTR aB, aB = 0 */
			KR(multicorrect(&L, a_tr*dtTR));
			L.Alpha = a_bdf;
			L.AlphaB = a_bdf;
			L.DeltaT = dtBDF2;
			L.DeltaTB = dtBDF2;
			time += dtBDF2;
			KR(fg_tr_lin(t, t->u, u_old, A, B));                 /* u = A u - B u_old, a = 0 */
			KR(fg_bubble_lin(t, t->uB, uB_old, A, B));           /* uB = A uB - B uB_old, aB = 0 */
			KR(multicorrect(&L, a_bdf*dtBDF2));
			CK(cudaMemcpyAsync(u_old, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
			CK(cudaMemcpyAsync(uB_old, t->uB, nbB, cudaMemcpyDeviceToDevice, t->stream));
			if (t_hist) t_hist[step - 1] = time;
			KR(stop_time(&L, u_old, time, &done));
		} while (!done && step < max_steps);
	} else if (o->method == FEMGPU_TI_PREDICTOR1) {
		/* Predictor_Old.c:62-136 */
		const double c1 = (1.0 - alpha) * dt, c2 = alpha * dt;
		do {
			step++;
			time += dt;
			KR(fg_tr_predict(t, c1));                         /* u_old = u, u += c1 a, a = 0 */
			KR(multicorrect(&L, c2));
			if (t_hist) t_hist[step - 1] = time;
			KR(stop_time(&L, t->uold, time, &done));
		} while (!done && step < max_steps);
	} else if (o->method == FEMGPU_TI_BDF) {
		/* Predictor_Old_BDF.c:50-160: an implicit first step built with
		 * Alpha = 1 (the updates keep the deck's alpha), then BDF2 with
		 * Alpha = 2/3; u_old stays the initial solution */
		const double four_thirds = 4.0/3.0, two_thirds = 2.0/3.0, one_third = 1.0/3.0;
		double *u_old = t->uold;
		step = 1;
		time += dt;
		L.Alpha = 1.0;
		CK(cudaMemcpyAsync(u_old, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		CK(cudaMemcpyAsync(t->u1, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		CK(cudaMemsetAsync(t->du, 0, nb, t->stream));
		KR(multicorrect(&L, alpha * dt));
		CK(cudaMemcpyAsync(t->u2, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		if (t_hist) t_hist[0] = time;
		L.Alpha = two_thirds;
		while (step < max_steps) {
			step++;
			time += dt;
			KR(fg_tr_lin(t, t->u2, t->u1, four_thirds, one_third));    /* u = 4/3 u2 - 1/3 u1, a = 0 */
			KR(multicorrect(&L, two_thirds * dt));
			CK(cudaMemcpyAsync(t->u1, t->u2, nb, cudaMemcpyDeviceToDevice, t->stream));
			CK(cudaMemcpyAsync(t->u2, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
			if (t_hist) t_hist[step - 1] = time;
			KR(stop_time(&L, u_old, time, &done));
			if (done) break;
		}
	} else {
		/* Predictor_Old_TRBDF2.c:34-165; DeltaT_Build is set to the TR
		 * sub-step once, then stays at the BDF2 sub-step */
		const double lambda = 2.0 - sqrt(2.0);
		const double A = 1.0/(lambda*(2.0 - lambda));
		const double B = (1.0 - lambda)*(1.0 - lambda)/(lambda*(2.0 - lambda));
		const double dtTR = lambda*dt, dtBDF2 = (1.0 - lambda)*dt;
		double *u_old = t->u1;
		CK(cudaMemcpyAsync(u_old, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
		L.DeltaTB = dtTR;
		do {
			double a_tr = 0.5, a_bdf = 1.0/(2.0 - lambda);
			step++;
			time += dtTR;
			L.Alpha = a_tr;
			L.DeltaT = dtTR;
			KR(fg_tr_axpy_zero(t, a_tr*dtTR));                  /* u += alpha dtTR a, a = 0 */
			KR(multicorrect(&L, a_tr*dtTR));
			L.Alpha = a_bdf;
			L.DeltaT = dtBDF2;
			L.DeltaTB = dtBDF2;
			time += dtBDF2;
			KR(fg_tr_lin(t, t->u, u_old, A, B));                 /* u = A u - B u_old, a = 0 */
			KR(multicorrect(&L, a_bdf*dtBDF2));
			CK(cudaMemcpyAsync(u_old, t->u, nb, cudaMemcpyDeviceToDevice, t->stream));
			if (t_hist) t_hist[step - 1] = time;
			KR(stop_time(&L, u_old, time, &done));
		} while (!done && step < max_steps);
	}
	CK(cudaStreamSynchronize(t->stream));
	return step;
}
