/*
 * Host side of the device Krylov solvers: workspace allocation and the
 * restart loop of pgmres.c:55-184 (one host synchronisation per restart
 * cycle; the inner iterations run stream-ordered on the device, predicated on
 * the device status block).  Shared by the transport and Euler contexts.
 * Plain C.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_internal.h"

#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)

int fgh_kry_alloc(fg_krylov *k, int n, int kmax, int zmode, void *stream)
{
	size_t m1 = (size_t)kmax + 1;
	memset(k, 0, sizeof *k);
	k->n = n;
	k->kmax = kmax;
	k->nblk = 2 * 152;
	k->ldv = (((size_t)n + 1) + 31) & ~(size_t)31;
	k->stream = (cudaStream_t)stream;
	DM(k->V, sizeof(double) * k->ldv * m1);
	DM(k->H, sizeof(double) * m1 * m1);
	DM(k->cs, sizeof(double) * m1);
	DM(k->sn, sizeof(double) * m1);
	DM(k->ge, sizeof(double) * (m1 + 1));
	DM(k->gy, sizeof(double) * m1);
	if (zmode == 1) DM(k->Z, sizeof(double) * k->ldv * (size_t)kmax);
	if (zmode == 2) DM(k->Z32, sizeof(float) * k->ldv * (size_t)kmax);
	DM(k->partials, sizeof(double) * ((size_t)k->nblk * (m1 + 1) + m1 + 1));
	DM(k->st, sizeof(fg_status));
	CK(cudaMemsetAsync(k->V, 0, sizeof(double) * k->ldv * m1, k->stream));
	CK(cudaMemsetAsync(k->st, 0, sizeof(fg_status), k->stream));
	CK(cudaMallocHost((void **)&k->st_host, sizeof(fg_status)));
	memset(k->st_host, 0, sizeof(fg_status));
	return 0;
}

void fgh_kry_free(fg_krylov *k)
{
	void *p[] = { k->V, k->H, k->cs, k->sn, k->ge, k->gy, k->Z, k->Z32, k->partials, k->st };
	int i;
	for (i = 0; i < (int)(sizeof p / sizeof p[0]); i++) if (p[i]) cudaFree(p[i]);
	if (k->st_host) cudaFreeHost(k->st_host);
	memset(k, 0, sizeof *k);
}

static int sync_status(const fg_krylov *k)
{
	CK(cudaMemcpyAsync(k->st_host, k->st, sizeof(fg_status), cudaMemcpyDeviceToHost, k->stream));
	CK(cudaStreamSynchronize(k->stream));
	if (k->st_host->err) {
		fgh_set_error("device reported error %d", k->st_host->err);
		return k->st_host->err;
	}
	return 0;
}

int fgh_kry_begin(const fg_krylov *k, double eps)
{
	k->st_host->eps = eps;
	k->st_host->total = 0;
	k->st_host->err = 0;
	k->st_host->ticket = 0;
	k->st_host->active = 0;
	CK(cudaMemcpyAsync(k->st, k->st_host, sizeof(fg_status), cudaMemcpyHostToDevice, k->stream));
	return 0;
}

int fgh_kry_cycle(const fg_krylov *k, const fg_linop *op, const double *B, double *X, int kind, int cycle)
{
	if (kind < 0) KR(fg_kry_pgmres_cycle(k, op, B, X));
	else KR(fg_kry_fgmres_cycle(k, op, B, X, kind, cycle));
	return sync_status(k);
}

int fgh_kry_cycles(const fg_krylov *k, const fg_linop *op, const double *B, double *X, int kind, double eps,
                   int lmax, int *iters)
{
	int l = 0, rc;
	if ((rc = fgh_kry_begin(k, eps))) return rc;
	for (;;) {
		do {
			if ((rc = fgh_kry_cycle(k, op, B, X, kind, l))) return rc;
			l++;
		} while (k->st_host->rho > eps && l < lmax);
		/* FGMRES stops on the unpreconditioned residual: confirm the
		 * recurrence's estimate with ||B - A X|| before accepting it */
		if (kind < 0 || k->st_host->rho > eps) break;
		KR(fg_kry_true_rho(k, op, B, X));
		if ((rc = sync_status(k))) return rc;
		if (k->st_host->rho <= eps || l >= lmax) break;
	}
	*iters += k->st_host->total;
	if (k->st_host->rho > eps) {
		fgh_set_error("GMRES: %d restarts, rho %.3e > eps %.3e", l, k->st_host->rho, eps);
		return FEMGPU_E_NOT_CONVERGED;
	}
	return 0;
}

int fgh_kry_dot_host(const fg_krylov *k, const double *a, const double *b, int n, double *out)
{
	KR(fg_kry_dot(k, a, b, n, &k->st->hdiag));
	CK(cudaMemcpyAsync(&k->st_host->hdiag, &k->st->hdiag, sizeof(double), cudaMemcpyDeviceToHost, k->stream));
	CK(cudaStreamSynchronize(k->stream));
	*out = k->st_host->hdiag;
	return 0;
}
