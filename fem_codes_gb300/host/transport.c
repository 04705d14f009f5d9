/*
 * Host driver of the steady-transport solve loop: the control flow of the
 * reference's Preprocess (storage set-up, Preprocess.c:160-237), Process
 * (Picard loop, Process.c:276-335) and pgmres (restart loop, pgmres.c:55-184),
 * calling device kernels for every data-parallel step.  Plain C.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_internal.h"

int fg_maxabsdiff(femgpu_transport *t, const double *a, const double *b, int n, double *out_dev);

static __thread char g_err[512];

void fgh_set_error(const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof g_err, fmt, ap);
	va_end(ap);
}

const char *femgpu_last_error(void) { return g_err; }


void femgpu_transport_default_opts(femgpu_transport_opts *o)
{
	memset(o, 0, sizeof *o);
	o->scheme = FEMGPU_CSR;
	o->reorder = FEMGPU_REORDER_NOT;
	o->precond = FEMGPU_PREC_ILU0;
	o->shock = FEMGPU_SHOCK_CAU;
	o->hshock = FEMGPU_H_2SQRTAREA;
	o->kmax = 30;
	o->lmax = 1000;
	o->tol = 1e-8;
	o->nonlin_tol = 0.0;
	o->precision = FEMGPU_FP64;
	o->ir_max = 30;
	o->stall_ratio = 0.9;
}

int fgh_dmalloc(void **p, size_t bytes)
{
	cudaError_t e = cudaMalloc(p, bytes ? bytes : 8);
	if (e != cudaSuccess) {
		fgh_set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
		return FEMGPU_E_NOMEM;
	}
	return 0;
}

#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)

static int upload(void **dst, const void *src, size_t bytes)
{
	int rc = fgh_dmalloc(dst, bytes);
	if (rc) return rc;
	CK(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
	return 0;
}

#define UP(ptr, src, bytes) do { int r_ = upload((void **)&(ptr), (src), (bytes)); if (r_) return r_; } while (0)

static int sync_err(femgpu_transport *t)
{
	CK(cudaMemcpyAsync(t->st_host, t->st, sizeof(fg_status), cudaMemcpyDeviceToHost, t->stream));
	CK(cudaStreamSynchronize(t->stream));
	if (t->st_host->err) {
		fgh_set_error("device reported error %d", t->st_host->err);
		return t->st_host->err;
	}
	return 0;
}

/* The SELL-32 layout of the CSR pattern (rows in slices of 32, each slice
 * padded to its longest row and stored entry index by entry index): the
 * slots' columns, their CSR positions and the slice offsets. */
static int build_sell(femgpu_transport *t, const int *IA, const int *JA)
{
	const int n = t->neq, ns = (n + 31) / 32;
	long long *base = malloc(sizeof(long long) * ((size_t)ns + 1)), nslot = 0;
	int *w = malloc(sizeof(int) * (size_t)ns), *src = NULL, *col = NULL, s, r, j, rc = 0;
	if (!base || !w) { free(base); free(w); return FEMGPU_E_NOMEM; }
	for (s = 0; s < ns; s++) {
		int wm = 0;
		for (r = 32 * s; r < n && r < 32 * s + 32; r++) if (IA[r + 1] - IA[r] > wm) wm = IA[r + 1] - IA[r];
		base[s] = nslot;
		w[s] = wm;
		nslot += 32LL * wm;
	}
	base[ns] = nslot;
	src = malloc(sizeof(int) * ((size_t)nslot + 1));
	col = malloc(sizeof(int) * ((size_t)nslot + 1));
	if (!src || !col) rc = FEMGPU_E_NOMEM;
	if (!rc) {
		long long k;
		for (k = 0; k < nslot; k++) { src[k] = -1; col[k] = 0; }
		for (r = 0; r < n; r++)
			for (j = 0; j < IA[r + 1] - IA[r]; j++) {
				long long at = base[r / 32] + 32LL * j + (r & 31);
				src[at] = IA[r] + j;
				col[at] = JA[IA[r] + j];
			}
		t->nslice = ns;
		t->nslot = nslot;
		if (upload((void **)&t->sell_base, base, sizeof(long long) * ((size_t)ns + 1)) ||
		    upload((void **)&t->sell_w, w, sizeof(int) * (size_t)ns) ||
		    upload((void **)&t->sell_src, src, sizeof(int) * ((size_t)nslot + 1)) ||
		    upload((void **)&t->sell_JA, col, sizeof(int) * ((size_t)nslot + 1)) ||
		    fgh_dmalloc((void **)&t->sell_A, sizeof(double) * ((size_t)nslot + 1)))
			rc = FEMGPU_E_NOMEM;
	}
	free(base); free(w); free(src); free(col);
	return rc;
}

/* Download the CSR pattern and rebuild the device structures under a new
 * equation numbering (reverse Cuthill-McKee, csr_Initialization.c:144-179). */
static int reorder_symrcm(femgpu_transport *t, int *hIA, int *hJA)
{
	int n = t->neq, i, rc;
	int *perm = malloc(sizeof(int) * (size_t)n), *inv = malloc(sizeof(int) * (size_t)n);
	if (!perm || !inv) return FEMGPU_E_NOMEM;
	rc = fgh_symrcm(n, hIA, hJA, perm);
	if (rc) return rc;
	for (i = 0; i < n; i++) inv[perm[i]] = i;
	for (i = 0; i < t->nnodes; i++)
		if (t->h_node_id[i] != -1) t->h_node_id[i] = inv[t->h_node_id[i]];
	free(perm);
	free(inv);
	CK(cudaMemcpy(t->node_id, t->h_node_id, sizeof(int) * (size_t)t->nnodes, cudaMemcpyHostToDevice));
	KR(fg_compute_lm(t));
	KR(fg_build_incidence(t));
	KR(fg_build_csr(t));
	return 0;
}

int femgpu_transport_create(femgpu_transport **out, const femgpu_transport_opts *opts,
		int nnodes, const double *x, const double *y, const int *node_type,
		int nel, const int *vert, double k, double gamma,
		const double *beta, const double *const_beta, const double *fsrc,
		const double *upresc)
{
	femgpu_transport *t;
	int i, neq = 0, rc;
	size_t nA = 0;
	int *hIA = NULL, *hJA = NULL;

	if (!out || nnodes <= 0 || nel <= 0 || !x || !y || !node_type || !vert || !upresc ||
	    (!beta && !const_beta)) {
		fgh_set_error("femgpu_transport_create: missing argument");
		return FEMGPU_E_ARG;
	}
	for (i = 0; i < 3 * nel; i++)
		if (vert[i] < 0 || vert[i] >= nnodes) {
			fgh_set_error("element vertex %d out of range", vert[i]);
			return FEMGPU_E_MESH;
		}
	t = calloc(1, sizeof *t);
	if (!t) return FEMGPU_E_NOMEM;
	if (opts) t->o = *opts; else femgpu_transport_default_opts(&t->o);
	if (t->o.scheme < 0 || t->o.scheme > 2 || t->o.precond < 0 || t->o.precond > 5 ||
	    t->o.precond == FEMGPU_PREC_BLOCKDIAG ||
	    (t->o.precond == FEMGPU_PREC_AMG && (t->o.scheme != FEMGPU_CSR || t->o.precision != FEMGPU_FP64)) ||
	    (t->o.precond == FEMGPU_PREC_LEARNED && (t->o.scheme != FEMGPU_CSR || t->o.solver != FEMGPU_FGMRES ||
	                                            t->o.precision != FEMGPU_FP64)) ||
	    t->o.kmax < 1 || t->o.lmax < 1 || t->o.hshock < 0 || t->o.hshock > 3 ||
	    t->o.precision < 0 || t->o.precision > 2 || t->o.solver < 0 || t->o.solver > 1 ||
	    (t->o.precision != FEMGPU_FP64 && (t->o.solver != FEMGPU_FGMRES || t->o.scheme != FEMGPU_CSR)) ||
	    (t->o.precond == FEMGPU_PREC_ILU0 && t->o.scheme != FEMGPU_CSR) ||
	    t->o.ilu_level < 0 || (t->o.ilu_level > 0 && t->o.precond != FEMGPU_PREC_ILU0) ||
	    (t->o.reorder == FEMGPU_REORDER_SYMRCM && t->o.scheme != FEMGPU_CSR)) {
		/* setPreconditioner.c:84-93: ILU is defined for CSR only */
		fgh_set_error("unsupported option combination");
		free(t);
		return FEMGPU_E_ARG;
	}
	*out = NULL;
	t->nnodes = nnodes;
	t->nel = nel;
	t->k = k;
	t->gamma = gamma;
	t->kmax = t->o.kmax;
	CK(cudaStreamCreateWithFlags(&t->own_stream, cudaStreamNonBlocking));
	t->stream = t->own_stream;

	/* Preprocess.c:73-81 numbering */
	t->h_node_id = malloc(sizeof(int) * (size_t)nnodes);
	for (i = 0; i < nnodes; i++) t->h_node_id[i] = (node_type[i] >= 1) ? neq++ : -1;
	t->neq = neq;
	if (neq == 0) { fgh_set_error("no unknowns"); free(t); return FEMGPU_E_MESH; }

	UP(t->x, x, sizeof(double) * (size_t)nnodes);
	UP(t->y, y, sizeof(double) * (size_t)nnodes);
	UP(t->node_type, node_type, sizeof(int) * (size_t)nnodes);
	UP(t->node_id, t->h_node_id, sizeof(int) * (size_t)nnodes);
	UP(t->vert, vert, sizeof(int) * 3 * (size_t)nel);
	UP(t->upresc, upresc, sizeof(double) * (size_t)nnodes);

	/* Coefficients: constant velocity / zero source need no per-element data. */
	t->beta_const = 1;
	if (beta) {
		t->cbx = beta[0]; t->cby = beta[1];
		for (i = 1; i < nel; i++)
			if (beta[2 * i] != t->cbx || beta[2 * i + 1] != t->cby) { t->beta_const = 0; break; }
		if (!t->beta_const) UP(t->beta, beta, sizeof(double) * 2 * (size_t)nel);
	} else {
		t->cbx = const_beta[0]; t->cby = const_beta[1];
	}
	t->fsrc_zero = 1;
	if (fsrc) {
		for (i = 0; i < 3 * nel; i++) if (fsrc[i] != 0.0) { t->fsrc_zero = 0; break; }
		if (!t->fsrc_zero) UP(t->fsrc, fsrc, sizeof(double) * 3 * (size_t)nel);
	}

	DM(t->st, sizeof(fg_status));
	CK(cudaMemsetAsync(t->st, 0, sizeof(fg_status), t->stream));
	CK(cudaMallocHost((void **)&t->st_host, sizeof(fg_status)));
	memset(t->st_host, 0, sizeof(fg_status));
	DM(t->lm, sizeof(int) * 3 * (size_t)nel);
	KR(fg_compute_lm(t));
	KR(fg_build_incidence(t));

	if (t->o.scheme == FEMGPU_CSR) {
		KR(fg_build_csr(t));
		hIA = malloc(sizeof(int) * ((size_t)neq + 1));
		hJA = malloc(sizeof(int) * ((size_t)t->nnz + 1));
		CK(cudaMemcpy(hIA, t->IA, sizeof(int) * ((size_t)neq + 1), cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(hJA, t->JA, sizeof(int) * (size_t)t->nnz, cudaMemcpyDeviceToHost));
		if (t->o.reorder == FEMGPU_REORDER_SYMRCM) {
			rc = reorder_symrcm(t, hIA, hJA);
			if (rc) return rc;
			CK(cudaMemcpy(hIA, t->IA, sizeof(int) * ((size_t)neq + 1), cudaMemcpyDeviceToHost));
			CK(cudaMemcpy(hJA, t->JA, sizeof(int) * (size_t)t->nnz, cudaMemcpyDeviceToHost));
		}
		t->bandwidth = fgh_bandwidth(neq, hIA, hJA);
		rc = build_sell(t, hIA, hJA);
		if (rc) return rc;
		nA = (size_t)t->nnz + 1;
		DM(t->ke, sizeof(double) * 9 * (size_t)nel);
	} else if (t->o.scheme == FEMGPU_EDE) {
		KR(fg_build_ede(t));
		nA = 4 * ((size_t)t->nedge + 1);
		DM(t->ke, sizeof(double) * 9 * (size_t)nel);
	} else {
		nA = 9 * (size_t)nel;
	}
	DM(t->A, sizeof(double) * nA);
	CK(cudaMemsetAsync(t->A, 0, sizeof(double) * nA, t->stream));
	DM(t->fe, sizeof(double) * 3 * (size_t)nel);
	DM(t->u, sizeof(double) * ((size_t)neq + 1));
	DM(t->F, sizeof(double) * ((size_t)neq + 1));
	DM(t->F0, sizeof(double) * ((size_t)neq + 1));
	DM(t->w2, sizeof(double) * ((size_t)neq + 1));
	DM(t->invDiag, sizeof(double) * ((size_t)neq + 1));
	DM(t->invDiag32, sizeof(float) * ((size_t)neq + 1));
	CK(cudaMemsetAsync(t->u, 0, sizeof(double) * ((size_t)neq + 1), t->stream));
	CK(cudaMemsetAsync(t->F, 0, sizeof(double) * ((size_t)neq + 1), t->stream));
	CK(cudaMemsetAsync(t->F0, 0, sizeof(double) * ((size_t)neq + 1), t->stream));
	if (t->o.precision == FEMGPU_MIXED_IR) {
		DM(t->A32, sizeof(float) * nA);
		DM(t->xr, sizeof(double) * ((size_t)neq + 1));
		DM(t->dr, sizeof(double) * ((size_t)neq + 1));
	}

	if (t->o.precond == FEMGPU_PREC_ILU0 || t->o.precond == FEMGPU_PREC_LEARNED) {
		const int *pIA = hIA, *pJA = hJA;
		int *fIA = NULL, *fJA = NULL, *fmap = NULL;
		t->ilu.n = neq;
		t->ilu.nnz = t->nnz;
		if (t->o.precond == FEMGPU_PREC_ILU0 && t->o.ilu_level > 0) {
			/* ILU(p): LEVEL_OF_FILL_lu's pattern on the host, the factor and
			 * sweeps on it (ILUp_precond_setup.c:17-45) */
			fg_ilu_sweeps *S = &t->sweeps;
			rc = fgh_iluk_pattern(neq, hIA, hJA, t->o.ilu_level, &fIA, &fJA, &fmap);
			if (rc) { free(hIA); free(hJA); return rc; }
			S->fnnz = fIA[neq];
			rc = fgh_dmalloc((void **)&S->fIA, sizeof(int) * ((size_t)neq + 1));
			if (!rc) rc = fgh_dmalloc((void **)&S->fJA, sizeof(int) * ((size_t)S->fnnz + 1));
			if (!rc) rc = fgh_dmalloc((void **)&S->fmap, sizeof(int) * ((size_t)t->nnz + 1));
			if (!rc) rc = fgh_dmalloc((void **)&S->fA, sizeof(double) * ((size_t)S->fnnz + 1));
			if (!rc && (cudaMemcpy(S->fIA, fIA, sizeof(int) * ((size_t)neq + 1), cudaMemcpyHostToDevice) ||
			            cudaMemcpy(S->fJA, fJA, sizeof(int) * (size_t)S->fnnz, cudaMemcpyHostToDevice) ||
			            cudaMemcpy(S->fmap, fmap, sizeof(int) * (size_t)t->nnz, cudaMemcpyHostToDevice)))
				rc = FEMGPU_E_CUDA;
			if (rc) { free(fIA); free(fJA); free(fmap); free(hIA); free(hJA); return rc; }
			S->fill = 1;
			t->ilu.nnz = S->fnnz;
			nA = (size_t)S->fnnz + 1;
			pIA = fIA;
			pJA = fJA;
		}
		DM(t->ilu.LU, sizeof(double) * nA);
		DM(t->ilu.Dinv, sizeof(double) * ((size_t)neq + 1));
		rc = fg_ilu_prepare(t, pIA, pJA);
		free(fIA);
		free(fJA);
		free(fmap);
		if (rc) {
			fgh_set_error("ILU(0) sweep programs: %d (%s)", rc, rc > 0 ? cudaGetErrorString((cudaError_t)rc) : "");
			return rc > 0 ? FEMGPU_E_CUDA : rc;
		}
	}
	free(hIA);
	free(hJA);

	/* Krylov workspace (pgmres.c:27-42), allocated once. */
	t->ldv = (((size_t)neq + 1) + 31) & ~(size_t)31;
	DM(t->V, sizeof(double) * t->ldv * ((size_t)t->kmax + 1));
	DM(t->H, sizeof(double) * ((size_t)t->kmax + 1) * ((size_t)t->kmax + 1));
	DM(t->cs, sizeof(double) * ((size_t)t->kmax + 1));
	DM(t->sn, sizeof(double) * ((size_t)t->kmax + 1));
	DM(t->ge, sizeof(double) * ((size_t)t->kmax + 2));
	DM(t->gy, sizeof(double) * ((size_t)t->kmax + 1));
	CK(cudaMemsetAsync(t->V, 0, sizeof(double) * t->ldv * ((size_t)t->kmax + 1), t->stream));
	if (t->o.solver == FEMGPU_FGMRES) {
		if (t->o.precision == FEMGPU_FP64) DM(t->Z, sizeof(double) * t->ldv * (size_t)t->kmax);
		else DM(t->Z32, sizeof(float) * t->ldv * (size_t)t->kmax);
	}
	t->nblk_red = 2 * 152;
	/* reduction partials: one row per basis vector for the CGS multi-dot,
	 * then the projection coefficients */
	DM(t->partials, sizeof(double) * ((size_t)t->nblk_red * ((size_t)t->kmax + 2) + (size_t)t->kmax + 2));
	for (i = 0; i < 4; i++) CK(cudaEventCreate(&t->ev[i]));
	CK(cudaDeviceSynchronize());
	rc = sync_err(t);
	if (rc) return rc;
	*out = t;
	return 0;
}

void femgpu_transport_destroy(femgpu_transport *t)
{
	int i;
	if (!t) return;
	cudaStreamSynchronize(t->stream);
	/* the network outlives this context: give it back its own stream */
	if (t->gnn) femgpu_gnn_set_stream(t->gnn, NULL);
	if (t->amg) femgpu_amg_set_stream(t->amg, NULL);
	void *ptrs[] = { t->x, t->y, t->upresc, t->beta, t->fsrc, t->node_type, t->node_id, t->vert,
		t->lm, t->ri_ptr, t->ri, t->IA, t->JA, t->sbe, t->diag, t->lm2, t->order, t->ec_ptr,
		t->ec, t->e2_ptr, t->e2, t->A, t->ke, t->fe, t->A32, t->u, t->F, t->F0, t->invDiag,
		t->invDiag32, t->ilu.LU, t->ilu.Dinv, t->V, t->H, t->cs, t->sn, t->ge, t->gy, t->w2,
		t->Z, t->Z32, t->xr, t->dr, t->partials, t->st, t->du, t->uold, t->Da, t->re, t->dold,
		t->u1, t->u2, t->uB, t->aB, t->bub, t->uB1, t->uB2, t->la_buf, t->la_flag, t->sell_base, t->sell_w, t->sell_src, t->sell_JA, t->sell_A };
	for (i = 0; i < (int)(sizeof ptrs / sizeof ptrs[0]); i++) if (ptrs[i]) cudaFree(ptrs[i]);
	if (t->la_s) {
		cudaStreamSynchronize(t->la_s);
		cudaEventDestroy(t->la_ev[0]);
		cudaEventDestroy(t->la_ev[1]);
		cudaStreamDestroy(t->la_s);
	}
	if (t->o.precond == FEMGPU_PREC_ILU0 || t->o.precond == FEMGPU_PREC_LEARNED) fg_ilu_free(t);
	if (t->st_host) cudaFreeHost(t->st_host);
	for (i = 0; i < 4; i++) if (t->ev[i]) cudaEventDestroy(t->ev[i]);
	if (t->own_stream) cudaStreamDestroy(t->own_stream);
	free(t->h_node_id);
	free(t);
}

int femgpu_transport_set_stream(femgpu_transport *t, void *stream)
{
	if (!t) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(t->stream));
	t->stream = stream ? (cudaStream_t)stream : t->own_stream;
	if (t->gnn) KR(femgpu_gnn_set_stream(t->gnn, t->stream));
	if (t->amg) KR(femgpu_amg_set_stream(t->amg, t->stream));
	return 0;
}

int femgpu_transport_info(const femgpu_transport *t, int *info)
{
	if (!t || !info) return FEMGPU_E_ARG;
	info[0] = t->neq; info[1] = t->nnz; info[2] = t->nedge; info[3] = t->bandwidth;
	info[4] = t->sweeps.lo64.nlev; info[5] = t->sweeps.up64.nlev;
	info[6] = t->fell_back;
	return 0;
}

int femgpu_transport_ilu_blocks(const femgpu_transport *t, int *first, int cap)
{
	if (!t) return FEMGPU_E_ARG;
	if (!t->sweeps.block_first) return FEMGPU_E_NOT_BUILT;
	int P = t->sweeps.nblocks;
	if (first) {
		if (cap < P + 1) return FEMGPU_E_ARG;
		memcpy(first, t->sweeps.block_first, sizeof(int) * ((size_t)P + 1));
	}
	return P;
}

int femgpu_transport_ilu_chain(const femgpu_transport *t, int *levels)
{
	if (!t) return FEMGPU_E_ARG;
	if (!t->sweeps.block_first) return FEMGPU_E_NOT_BUILT;
	if (levels) {
		levels[0] = t->sweeps.chain ? t->sweeps.lo64c.nlev : 0;
		levels[1] = t->sweeps.chain ? t->sweeps.up64c.nlev : 0;
	}
	return t->sweeps.chain ? 1 : 0;
}

int femgpu_transport_set_sweep_wait(femgpu_transport *t, int spins)
{
	if (!t) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(t->stream));
	t->sweep_wait1 = spins < 0 ? 0 : (spins == 0x7fffffff ? spins : spins + 1);
	CK(cudaMemsetAsync(&t->st->err, 0, sizeof(int), t->stream));
	t->st_host->err = 0;
	CK(cudaStreamSynchronize(t->stream));
	return 0;
}

int femgpu_transport_get_pattern(const femgpu_transport *t, int *IA, int *JA, int *sbe, int *order,
		int *node_id)
{
	if (!t) return FEMGPU_E_ARG;
	if (node_id) memcpy(node_id, t->h_node_id, sizeof(int) * (size_t)t->nnodes);
	if (t->o.scheme == FEMGPU_CSR) {
		if (IA) CK(cudaMemcpy(IA, t->IA, sizeof(int) * ((size_t)t->neq + 1), cudaMemcpyDeviceToHost));
		if (JA) CK(cudaMemcpy(JA, t->JA, sizeof(int) * (size_t)t->nnz, cudaMemcpyDeviceToHost));
		if (sbe) CK(cudaMemcpy(sbe, t->sbe, sizeof(int) * 9 * (size_t)t->nel, cudaMemcpyDeviceToHost));
	} else if (t->o.scheme == FEMGPU_EDE) {
		if (JA) CK(cudaMemcpy(JA, t->lm2, sizeof(int) * 2 * (size_t)t->nedge, cudaMemcpyDeviceToHost));
		if (sbe) CK(cudaMemcpy(sbe, t->sbe, sizeof(int) * 3 * (size_t)t->nel, cudaMemcpyDeviceToHost));
		if (order) CK(cudaMemcpy(order, t->order, sizeof(int) * 3 * (size_t)t->nel, cudaMemcpyDeviceToHost));
	}
	return 0;
}

static size_t storage_len(const femgpu_transport *t)
{
	if (t->o.scheme == FEMGPU_CSR) return (size_t)t->nnz + 1;
	if (t->o.scheme == FEMGPU_EDE) return 4 * ((size_t)t->nedge + 1);
	return 9 * (size_t)t->nel;
}

/* ---------------------------------------------------------------- build */
int femgpu_transport_build_dev(femgpu_transport *t)
{
	if (!t) return FEMGPU_E_ARG;
	CK(cudaEventRecord(t->ev[0], t->stream));
	KR(fg_build_elements(t));
	KR(fg_assemble(t));
	CK(cudaEventRecord(t->ev[1], t->stream));
	t->built = 1;
	t->factored = 0;
	return 0;
}

int femgpu_transport_build(femgpu_transport *t, const double *u_host, double *F_host, double *A_host)
{
	int rc;
	if (!t) return FEMGPU_E_ARG;
	if (u_host)
		CK(cudaMemcpyAsync(t->u, u_host, sizeof(double) * ((size_t)t->neq + 1), cudaMemcpyHostToDevice,
		                   t->stream));
	rc = femgpu_transport_build_dev(t);
	if (rc) return rc;
	if (F_host)
		CK(cudaMemcpyAsync(F_host, t->F, sizeof(double) * ((size_t)t->neq + 1), cudaMemcpyDeviceToHost,
		                   t->stream));
	if (A_host)
		CK(cudaMemcpyAsync(A_host, t->A, sizeof(double) * storage_len(t), cudaMemcpyDeviceToHost, t->stream));
	return sync_err(t);
}

/* ------------------------------------------------------- preconditioner */
/* The AMG hierarchy of the current CSR matrix (set up on the host). */
static int amg_rebuild(femgpu_transport *t)
{
	int rc, n = t->neq;
	int *IA, *JA;
	double *AA;
	if (!t->amg) { fgh_set_error("AMG preconditioner not set"); return FEMGPU_E_NOT_BUILT; }
	IA = malloc(sizeof(int) * ((size_t)n + 1));
	JA = malloc(sizeof(int) * (size_t)(t->nnz ? t->nnz : 1));
	AA = malloc(sizeof(double) * (size_t)(t->nnz ? t->nnz : 1));
	rc = (IA && JA && AA) ? 0 : FEMGPU_E_NOMEM;
	if (!rc && (cudaMemcpyAsync(IA, t->IA, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, t->stream) ||
	            cudaMemcpyAsync(JA, t->JA, sizeof(int) * (size_t)t->nnz, cudaMemcpyDeviceToHost, t->stream) ||
	            cudaMemcpyAsync(AA, t->A, sizeof(double) * (size_t)t->nnz, cudaMemcpyDeviceToHost, t->stream) ||
	            cudaStreamSynchronize(t->stream)))
		rc = FEMGPU_E_CUDA;
	if (!rc) rc = femgpu_amg_setup(t->amg, n, IA, JA, AA);
	free(IA); free(JA); free(AA);
	return rc;
}

int femgpu_transport_precond_setup_dev(femgpu_transport *t, int tag)
{
	(void)tag;   /* the symbolic phase of tag == 1 is done once at create */
	if (!t) return FEMGPU_E_ARG;
	if (!t->built) { fgh_set_error("precond_setup before Build"); return FEMGPU_E_NOT_BUILT; }
	CK(cudaMemcpyAsync(t->F0, t->F, sizeof(double) * ((size_t)t->neq + 1), cudaMemcpyDeviceToDevice,
	                   t->stream));
	/* Left preconditioning (the reference's pgmres) solves M^-1 A x = M^-1 F,
	 * so precond_setup also applies M^-1 to F; the right-preconditioned
	 * solver keeps F as is. */
	if (t->o.precond == FEMGPU_PREC_ILU0) {
		KR(fg_ilu0_factor(t));
		if (t->o.solver == FEMGPU_PGMRES) KR(fg_precond(t, t->F, t->F, NULL));
	} else if (t->o.precond == FEMGPU_PREC_LEARNED) {
		/* re-attach the network to the new matrix; ILU(0) is factored only
		 * if a solve falls back to it */
		if (!t->gnn) { fgh_set_error("learned preconditioner not set"); return FEMGPU_E_NOT_BUILT; }
		KR(femgpu_gnn_attach_csr_dev(t->gnn, t->neq, t->nnz, t->IA, t->JA, t->A));
		t->fell_back = 0;
	} else if (t->o.precond == FEMGPU_PREC_AMG) {
		/* AMG_precond_setup (amg_precond.c:26-100): the hierarchy of the
		 * current matrix on the host, then F := M^-1 F for pgmres */
		int rc = amg_rebuild(t);
		if (rc) return rc;
		if (t->o.solver == FEMGPU_PGMRES) KR(fg_precond(t, t->F, t->F, NULL));
	} else if (t->o.precond == FEMGPU_PREC_DIAG) {
		KR(fg_diag_setup(t));
	}
	if (t->o.precision == FEMGPU_MIXED_IR) KR(fg_to_f32(t->A, t->A32, (long long)storage_len(t), t->stream));
	CK(cudaEventRecord(t->ev[2], t->stream));
	t->factored = 1;
	return 0;
}

int femgpu_transport_precond_setup(femgpu_transport *t, int tag, double *F_host)
{
	int rc = femgpu_transport_precond_setup_dev(t, tag);
	if (rc) return rc;
	if (F_host)
		CK(cudaMemcpyAsync(F_host, t->F, sizeof(double) * ((size_t)t->neq + 1), cudaMemcpyDeviceToHost,
		                   t->stream));
	return sync_err(t);
}

int femgpu_transport_precond_dev(femgpu_transport *t, const double *p, double *z)
{
	if (!t || !p || !z) return FEMGPU_E_ARG;
	if (!t->factored && t->o.precond != FEMGPU_PREC_NOT) {
		fgh_set_error("precond before precond_setup");
		return FEMGPU_E_NOT_BUILT;
	}
	KR(fg_precond(t, p, z, NULL));
	return 0;
}

int fg_precond32(femgpu_transport *t, const double *p, float *z, const int *active);

int femgpu_transport_precond32_dev(femgpu_transport *t, const double *p, float *z)
{
	if (!t || !p || !z) return FEMGPU_E_ARG;
	if (!t->factored && t->o.precond != FEMGPU_PREC_NOT) {
		fgh_set_error("precond before precond_setup");
		return FEMGPU_E_NOT_BUILT;
	}
	KR(fg_precond32(t, p, z, NULL));
	return 0;
}

int femgpu_transport_precond(femgpu_transport *t, const double *p_host, double *z_host)
{
	int rc;
	size_t n1;
	if (!t || !p_host || !z_host) return FEMGPU_E_ARG;
	n1 = (size_t)t->neq + 1;
	CK(cudaMemcpyAsync(t->w2, p_host, sizeof(double) * n1, cudaMemcpyHostToDevice, t->stream));
	rc = femgpu_transport_precond_dev(t, t->w2, t->w2);
	if (rc) return rc;
	CK(cudaMemcpyAsync(z_host, t->w2, sizeof(double) * t->neq, cudaMemcpyDeviceToHost, t->stream));
	return sync_err(t);
}

/* --------------------------------------------------------------- matvec */
int femgpu_transport_matvec_dev(femgpu_transport *t, const double *P, double *Q)
{
	if (!t || !P || !Q) return FEMGPU_E_ARG;
	KR(fg_matvec(t, P, Q, NULL));
	return 0;
}

int femgpu_transport_matvec(femgpu_transport *t, const double *P_host, double *Q_host)
{
	int rc;
	size_t n1;
	double *P, *Q;
	if (!t || !P_host || !Q_host) return FEMGPU_E_ARG;
	n1 = (size_t)t->neq + 1;
	P = t->V;
	Q = t->V + t->ldv;
	CK(cudaMemcpyAsync(P, P_host, sizeof(double) * n1, cudaMemcpyHostToDevice, t->stream));
	rc = femgpu_transport_matvec_dev(t, P, Q);
	if (rc) return rc;
	/* csrmv.c leaves Q[neq] alone; ebemv.c / edemv.c zero P[neq] and Q[neq] */
	CK(cudaMemcpyAsync(Q_host, Q, sizeof(double) * (t->o.scheme == FEMGPU_CSR ? n1 - 1 : n1),
	                   cudaMemcpyDeviceToHost, t->stream));
	rc = sync_err(t);
	if (rc) return rc;
	if (t->o.scheme != FEMGPU_CSR) { ((double *)P_host)[t->neq] = 0.0; Q_host[t->neq] = 0.0; }
	return 0;
}

/* ---------------------------------------------------------------- GMRES */
static int dot_host(femgpu_transport *t, const double *a, const double *b, double *out)
{
	KR(fg_dot(t, a, b, t->neq, &t->st->hdiag));
	CK(cudaMemcpyAsync(&t->st_host->hdiag, &t->st->hdiag, sizeof(double), cudaMemcpyDeviceToHost,
	                   t->stream));
	CK(cudaStreamSynchronize(t->stream));
	*out = t->st_host->hdiag;
	return 0;
}

/* Restart cycles of the context's solver (fgh_kry_cycles). */
static int cycles(femgpu_transport *t, const double *B, double *X, int kind, double eps, int lmax,
                  int *iters)
{
	fg_krylov k;
	fg_linop op;
	fg_transport_krylov(t, &k, &op);
	return fgh_kry_cycles(&k, &op, B, X, kind, eps, lmax, iters);
}

/* FGMRES with the learned right preconditioner: a restart cycle that leaves
 * the residual above stall_ratio times its value at the cycle's start
 * switches the rest of the solve to ILU(0) (factored then), continuing from
 * the current iterate; a breakdown (zero or NaN Arnoldi norm) restarts the
 * solve from X = 0 with ILU(0).  With an AMG context attached
 * (femgpu_transport_set_amg) the fallback is its V-cycle instead. */
static int fall_back(femgpu_transport *t)
{
	if (t->amg) {
		int rc = amg_rebuild(t);
		if (rc) return rc;
		t->fell_back = 2;
		return 0;
	}
	KR(fg_ilu0_factor(t));
	t->fell_back = 1;
	return 0;
}

static int learned_cycles(femgpu_transport *t, const double *B, double *X, double eps, double rho0,
                          int *iters)
{
	fg_krylov k;
	fg_linop op;
	int l = 0, c = 0, rc, done = 0;            /* c: cycles since the solve (re)started */
	double prev = rho0;
	fg_transport_krylov(t, &k, &op);
	if ((rc = fgh_kry_begin(&k, eps))) return rc;
	do {
		rc = fgh_kry_cycle(&k, &op, B, X, 0, c++);
		l++;
		if (rc == FEMGPU_E_BREAKDOWN && !t->fell_back) {
			done += k.st_host->total;
			CK(cudaMemsetAsync(X, 0, sizeof(double) * (size_t)t->neq, t->stream));
			if ((rc = fall_back(t))) return rc;
			prev = rho0;
			c = 0;
			if ((rc = fgh_kry_begin(&k, eps))) return rc;
			continue;
		}
		if (rc) return rc;
		if (k.st_host->rho <= eps) {
			/* accept on the unpreconditioned residual ||B - A X||, not the estimate */
			KR(fg_kry_true_rho(&k, &op, B, X));
			CK(cudaMemcpyAsync(k.st_host, k.st, sizeof(fg_status), cudaMemcpyDeviceToHost, t->stream));
			CK(cudaStreamSynchronize(t->stream));
			if (k.st_host->rho <= eps) break;
			continue;
		}
		if (!t->fell_back && !(k.st_host->rho <= t->o.stall_ratio * prev) && (rc = fall_back(t))) return rc;
		prev = k.st_host->rho;
	} while (l < t->o.lmax);
	*iters += done + k.st_host->total;
	if (k.st_host->rho > eps) {
		fgh_set_error("FGMRES (learned): %d restarts, rho %.3e > eps %.3e", l, k.st_host->rho, eps);
		return FEMGPU_E_NOT_CONVERGED;
	}
	return 0;
}

int femgpu_transport_set_amg(femgpu_transport *t, femgpu_amg *g)
{
	if (!t || !g || (t->o.precond != FEMGPU_PREC_AMG && t->o.precond != FEMGPU_PREC_LEARNED)) return FEMGPU_E_ARG;
	KR(femgpu_amg_set_stream(g, t->stream));
	t->amg = g;
	t->factored = 0;
	return 0;
}

int femgpu_transport_set_learned(femgpu_transport *t, femgpu_gnn *g)
{
	if (!t || !g || t->o.precond != FEMGPU_PREC_LEARNED) return FEMGPU_E_ARG;
	KR(femgpu_gnn_set_stream(g, t->stream));
	t->gnn = g;
	t->factored = 0;
	return 0;
}

int femgpu_transport_csr_dev(femgpu_transport *t, const int **IA, const int **JA, const double **AA)
{
	if (!t || t->o.scheme != FEMGPU_CSR || !IA || !JA || !AA) return FEMGPU_E_ARG;
	*IA = t->IA;
	*JA = t->JA;
	*AA = t->A;
	return 0;
}

int femgpu_transport_krylov_pairs(femgpu_transport *t, int max, double *V, double *Z, int ld)
{
	int i, m;
	if (!t || max < 0 || !V || !Z || ld < t->neq || !t->Z) return FEMGPU_E_ARG;
	m = t->st_host->inner < max ? t->st_host->inner : max;
	for (i = 0; i < m; i++) {
		CK(cudaMemcpyAsync(V + (size_t)i * ld, t->V + (size_t)i * t->ldv, sizeof(double) * (size_t)t->neq,
		                   cudaMemcpyDeviceToDevice, t->stream));
		CK(cudaMemcpyAsync(Z + (size_t)i * ld, t->Z + (size_t)i * t->ldv, sizeof(double) * (size_t)t->neq,
		                   cudaMemcpyDeviceToDevice, t->stream));
	}
	CK(cudaStreamSynchronize(t->stream));
	return m;
}

static int gmres(femgpu_transport *t, const double *B, double *X, int *iters);

/* The context's solver on device vectors (X := solve(B)), for the drivers
 * built on a transport context (the transient time loop). */
int fgh_transport_gmres(femgpu_transport *t, const double *B, double *X, int *iters)
{
	return gmres(t, B, X, iters);
}

static int gmres(femgpu_transport *t, const double *B, double *X, int *iters)
{
	int n = t->neq, it = 0, rc;
	double normb2, eps;
	if (!t->factored && t->o.precond != FEMGPU_PREC_NOT) {
		fgh_set_error("solve before precond_setup");
		return FEMGPU_E_NOT_BUILT;
	}
	if (iters) *iters = 0;
	CK(cudaMemsetAsync(X, 0, sizeof(double) * (size_t)n, t->stream));          /* pgmres.c:46 */
	rc = dot_host(t, B, B, &normb2);
	if (rc) return rc;
	if (!(normb2 > 0.0)) {
		/* B == 0: X = 0 is the solution (pgmres.c would divide 0 by 0). */
		return (normb2 == 0.0) ? 0 : FEMGPU_E_BREAKDOWN;
	}
	eps = t->o.tol * sqrt(normb2);                                               /* pgmres.c:49-53 */
	if (t->o.solver == FEMGPU_PGMRES) {
		rc = cycles(t, B, X, -1, eps, t->o.lmax, &it);
	} else if (t->o.precond == FEMGPU_PREC_LEARNED) {
		rc = learned_cycles(t, B, X, eps, sqrt(normb2), &it);
	} else if (t->o.precision != FEMGPU_MIXED_IR) {
		rc = cycles(t, B, X, t->o.precision == FEMGPU_MIXED ? 1 : 0, eps, t->o.lmax, &it);
	} else {
		/* FP64 iterative refinement around FP32 inner solves:
		 * r = B - A x (FP64), solve A d = r to inner_tol in FP32, x += d. */
		int sweep;
		double itol = t->o.inner_tol > 0 ? t->o.inner_tol : 1e-4;
		rc = FEMGPU_E_NOT_CONVERGED;
		for (sweep = 0; sweep < t->o.ir_max; sweep++) {
			double r2;
			int rci;
			KR(fg_axpy_resid(t, B, t->xr));
			rci = dot_host(t, t->xr, t->xr, &r2);
			if (rci) return rci;
			if (!(r2 == r2)) { rc = FEMGPU_E_BREAKDOWN; break; }
			if (sqrt(r2) <= eps) { rc = 0; break; }
			CK(cudaMemsetAsync(t->dr, 0, sizeof(double) * (size_t)n, t->stream));
			rci = cycles(t, t->xr, t->dr, 2, fmax(itol * sqrt(r2), 0.5 * eps), t->o.lmax, &it);
			if (rci && rci != FEMGPU_E_NOT_CONVERGED) return rci;
			KR(fg_add(X, t->dr, n, t->stream));
		}
		if (rc) fgh_set_error("iterative refinement: %d sweeps without reaching tol", sweep);
	}
	if (iters) *iters = it;
	return rc;
}

int femgpu_transport_solve_dev(femgpu_transport *t, int *iters)
{
	int rc;
	if (!t) return FEMGPU_E_ARG;
	rc = gmres(t, t->F, t->u, iters);
	CK(cudaEventRecord(t->ev[3], t->stream));
	return rc;
}

int femgpu_transport_solve(femgpu_transport *t, double *X_host, int *iters)
{
	int rc = femgpu_transport_solve_dev(t, iters);
	if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;
	if (X_host)
		CK(cudaMemcpyAsync(X_host, t->u, sizeof(double) * (size_t)t->neq, cudaMemcpyDeviceToHost, t->stream));
	CK(cudaStreamSynchronize(t->stream));
	return rc;
}

int femgpu_transport_solve_bx(femgpu_transport *t, const double *B_host, double *X_host, int *iters)
{
	int rc;
	if (!t || !B_host || !X_host) return FEMGPU_E_ARG;
	CK(cudaMemcpyAsync(t->w2, B_host, sizeof(double) * (size_t)t->neq, cudaMemcpyHostToDevice, t->stream));
	rc = gmres(t, t->w2, t->u, iters);
	if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;
	CK(cudaMemcpyAsync(X_host, t->u, sizeof(double) * (size_t)t->neq, cudaMemcpyDeviceToHost, t->stream));
	CK(cudaStreamSynchronize(t->stream));
	return rc;
}

double *femgpu_transport_u_dev(femgpu_transport *t) { return t ? t->u : NULL; }
double *femgpu_transport_F_dev(femgpu_transport *t) { return t ? t->F : NULL; }

int fg_operator(femgpu_transport *t, const double *p, double *q);

int femgpu_transport_operator_dev(femgpu_transport *t, const double *P, double *Q)
{
	if (!t || !P || !Q) return FEMGPU_E_ARG;
	KR(fg_operator(t, P, Q));
	return 0;
}

/* -------------------------------------------------------------- Process */
int femgpu_transport_process(femgpu_transport *t, int npicard, double *u_hist, int *iters)
{
	int it = 0, rc;
	size_t n1;
	double *uold;
	if (!t || npicard < 1) return FEMGPU_E_ARG;
	n1 = (size_t)t->neq + 1;
	uold = t->w2;
	CK(cudaMemsetAsync(t->u, 0, sizeof(double) * n1, t->stream));                  /* Process.c:289 */
	while (it < npicard) {
		int nit = 0;
		it++;
		CK(cudaMemcpyAsync(uold, t->u, sizeof(double) * (size_t)t->neq, cudaMemcpyDeviceToDevice, t->stream));
		rc = femgpu_transport_build_dev(t);
		if (rc) return rc;
		rc = femgpu_transport_precond_setup_dev(t, it);
		if (rc) return rc;
		rc = femgpu_transport_solve_dev(t, &nit);
		if (rc && rc != FEMGPU_E_NOT_CONVERGED) return rc;
		if (iters) iters[it - 1] = nit;
		if (u_hist)
			CK(cudaMemcpyAsync(u_hist + (size_t)(it - 1) * n1, t->u, sizeof(double) * n1,
			                   cudaMemcpyDeviceToHost, t->stream));
		if (t->o.nonlin_tol > 0.0) {
			KR(fg_maxabsdiff(t, t->u, uold, t->neq, &t->st->hdiag));
			CK(cudaMemcpyAsync(&t->st_host->hdiag, &t->st->hdiag, sizeof(double), cudaMemcpyDeviceToHost,
			                   t->stream));
			CK(cudaStreamSynchronize(t->stream));
			if (!(t->st_host->hdiag > t->o.nonlin_tol)) break;
		}
	}
	CK(cudaStreamSynchronize(t->stream));
	return it;
}

int femgpu_transport_true_residual(femgpu_transport *t, double *relres)
{
	double r2, b2;
	if (!t || !relres) return FEMGPU_E_ARG;
	KR(fg_residual_norm(t, t->F0, t->u, &t->st->hdiag));
	KR(fg_dot(t, t->F0, t->F0, t->neq, &t->st->rho));
	CK(cudaMemcpyAsync(t->st_host, t->st, sizeof(fg_status), cudaMemcpyDeviceToHost, t->stream));
	CK(cudaStreamSynchronize(t->stream));
	r2 = t->st_host->hdiag;
	b2 = t->st_host->rho;
	*relres = (b2 > 0) ? sqrt(r2 / b2) : sqrt(r2);
	return 0;
}

int femgpu_transport_last_times(const femgpu_transport *t, float *tm)
{
	if (!t || !tm) return FEMGPU_E_ARG;
	CK(cudaEventSynchronize(t->ev[3]));
	CK(cudaEventElapsedTime(&tm[0], t->ev[0], t->ev[1]));
	CK(cudaEventElapsedTime(&tm[1], t->ev[1], t->ev[2]));
	CK(cudaEventElapsedTime(&tm[2], t->ev[2], t->ev[3]));
	return 0;
}

/* ------------------------------------------------------- host utilities */
int femgpu_symrcm(int n, const int *IA, const int *JA, int *perm)
{
	if (n <= 0 || !IA || !JA || !perm) return FEMGPU_E_ARG;
	return fgh_symrcm(n, IA, JA, perm);
}

int femgpu_ilu_levels(int n, const int *IA, const int *JA, int lower)
{
	int *rows, *task = NULL, ntask = 0, nlev = 0, rc;
	if (n <= 0 || !IA || !JA) return FEMGPU_E_ARG;
	rows = malloc(sizeof(int) * (size_t)n);
	if (!rows) return FEMGPU_E_NOMEM;
	rc = fgh_levels(n, IA, JA, lower, rows, &task, &ntask, &nlev);
	free(rows);
	free(task);
	return rc ? rc : nlev;
}

/* -------------------------------------------------- stateless kernels */
int femgpu_csrmv_f64(int n, const int *IA, const int *JA, const double *AA, const double *P, double *Q,
		void *stream)
{
	if (n < 0 || !IA || !JA || !AA || !P || !Q) return FEMGPU_E_ARG;
	KR(fg_csrmv64(n, IA, JA, AA, P, Q, NULL, (cudaStream_t)stream));
	return 0;
}

int femgpu_csrmv_f64_fused(int n, const int *IA, const int *JA, const double *AA, const double *P, double *Q,
		void *stream)
{
	if (n < 0 || !IA || !JA || !AA || !P || !Q) return FEMGPU_E_ARG;
	KR(fg_csrmv64_fused(n, IA, JA, AA, P, Q, NULL, (cudaStream_t)stream));
	return 0;
}

int femgpu_csrmv_f32(int n, const int *IA, const int *JA, const float *AA, const float *P, float *Q,
		void *stream)
{
	if (n < 0 || !IA || !JA || !AA || !P || !Q) return FEMGPU_E_ARG;
	KR(fg_csrmv32(n, IA, JA, AA, P, Q, NULL, (cudaStream_t)stream));
	return 0;
}
