/*
 * Host side of the learned preconditioner (mesh graph network): parameter
 * storage, graph attachment to a CSR matrix, inference, the loss gradient of
 * one (residual, correction) pair and the Adam step.  No reference
 * counterpart.  Plain C.
 */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_gnn.h"

#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)
#define FREE(p) do { if (p) { cudaFree(p); (p) = NULL; } } while (0)

int femgpu_gnn_nparams(void) { return GNN_NPARAMS; }

static void free_graph(fg_gnn *g)
{
	int l;
	FREE(g->gptr); FREE(g->gcol); FREE(g->wA); FREE(g->wT); FREE(g->d); FREE(g->x);
	for (l = 0; l <= GNN_LAYERS; l++) { FREE(g->h[l]); FREE(g->mask[l]); }
	for (l = 0; l < GNN_LAYERS; l++) { FREE(g->m1[l]); FREE(g->m2[l]); }
	FREE(g->gh[0]); FREE(g->gh[1]); FREE(g->gm1); FREE(g->gm2); FREE(g->gz); FREE(g->res);
	g->cap_n = g->cap_e = 0;
}

static int create(fg_gnn *g, int bf16_act, const float *theta)
{
	size_t P = sizeof(float) * GNN_NPARAMS;
	g->bf16 = bf16_act ? 1 : 0;
	CK(cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking));
	g->stream = g->own_stream;
	DM(g->theta, P); DM(g->grad, P); DM(g->am, P); DM(g->av, P);
	DM(g->part, sizeof(float) * GNN_RED_BLOCKS * GNN_LAYER_SIZE);
	DM(g->rpart, sizeof(double) * 2 * GNN_RED_BLOCKS);
	DM(g->sums, sizeof(double) * 2); DM(g->stats, sizeof(double) * 2);
	DM(g->lsums, sizeof(double) * 4); DM(g->lsums2, sizeof(double) * 4);
	DM(g->err, sizeof(int));
	CK(cudaMemsetAsync(g->err, 0, sizeof(int), g->stream));
	CK(cudaMemsetAsync(g->grad, 0, P, g->stream));
	return femgpu_gnn_set_params(g, theta);
}

int femgpu_gnn_create(femgpu_gnn **out, int bf16_act, const float *theta)
{
	fg_gnn *g;
	int rc;
	if (!out) return FEMGPU_E_ARG;
	*out = NULL;
	g = calloc(1, sizeof *g);
	if (!g) return FEMGPU_E_NOMEM;
	rc = create(g, bf16_act, theta);
	if (rc) { femgpu_gnn_destroy(g); return rc; }
	*out = g;
	return 0;
}

void femgpu_gnn_destroy(femgpu_gnn *g)
{
	if (!g) return;
	if (g->stream) cudaStreamSynchronize(g->stream);
	free_graph(g);
	FREE(g->theta); FREE(g->grad); FREE(g->am); FREE(g->av); FREE(g->part); FREE(g->rpart);
	FREE(g->sums); FREE(g->lsums); FREE(g->lsums2); FREE(g->stats); FREE(g->err);
	if (g->own_stream) cudaStreamDestroy(g->own_stream);
	free(g);
}

int femgpu_gnn_set_stream(femgpu_gnn *g, void *stream)
{
	if (!g) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(g->stream));
	g->stream = stream ? (cudaStream_t)stream : g->own_stream;
	return 0;
}

int femgpu_gnn_set_params(femgpu_gnn *g, const float *theta)
{
	size_t P = sizeof(float) * GNN_NPARAMS;
	if (!g) return FEMGPU_E_ARG;
	if (theta) CK(cudaMemcpyAsync(g->theta, theta, P, cudaMemcpyHostToDevice, g->stream));
	else CK(cudaMemsetAsync(g->theta, 0, P, g->stream));
	CK(cudaMemsetAsync(g->am, 0, P, g->stream));
	CK(cudaMemsetAsync(g->av, 0, P, g->stream));
	g->step = 0;
	CK(cudaStreamSynchronize(g->stream));
	return 0;
}

int femgpu_gnn_get_params(femgpu_gnn *g, float *theta)
{
	if (!g || !theta) return FEMGPU_E_ARG;
	CK(cudaMemcpyAsync(theta, g->theta, sizeof(float) * GNN_NPARAMS, cudaMemcpyDeviceToHost, g->stream));
	CK(cudaStreamSynchronize(g->stream));
	return 0;
}

int femgpu_gnn_get_grad(femgpu_gnn *g, float *grad)
{
	if (!g || !grad) return FEMGPU_E_ARG;
	CK(cudaMemcpyAsync(grad, g->grad, sizeof(float) * GNN_NPARAMS, cudaMemcpyDeviceToHost, g->stream));
	CK(cudaStreamSynchronize(g->stream));
	return 0;
}

static int ensure(fg_gnn *g, int n, int ne)
{
	size_t sa = g->bf16 ? 2 : 4, row = (size_t)GNN_WIDTH;
	int l;
	if (n <= g->cap_n && ne <= g->cap_e) return 0;
	free_graph(g);
	DM(g->gptr, sizeof(int) * ((size_t)n + 1));
	DM(g->gcol, sizeof(int) * (size_t)(ne ? ne : 1));
	DM(g->wA, sizeof(float) * (size_t)(ne ? ne : 1));
	DM(g->wT, sizeof(float) * (size_t)(ne ? ne : 1));
	DM(g->d, sizeof(double) * (size_t)n);
	DM(g->x, 8 * (size_t)n);
	for (l = 0; l <= GNN_LAYERS; l++) {
		DM(g->h[l], sa * row * (size_t)n);
		DM(g->mask[l], sizeof(unsigned) * (size_t)n);
	}
	for (l = 0; l < GNN_LAYERS; l++) {
		DM(g->m1[l], sa * row * (size_t)n);
		DM(g->m2[l], sa * row * (size_t)n);
	}
	DM(g->gh[0], 4 * row * (size_t)n); DM(g->gh[1], 4 * row * (size_t)n);
	DM(g->gm1, 4 * row * (size_t)n); DM(g->gm2, 4 * row * (size_t)n);
	DM(g->gz, sizeof(double) * (size_t)n); DM(g->res, sizeof(double) * (size_t)n);
	g->cap_n = n;
	g->cap_e = ne;
	return 0;
}

static int check_err(fg_gnn *g)
{
	int e = 0;
	CK(cudaMemcpyAsync(&e, g->err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
	CK(cudaStreamSynchronize(g->stream));
	if (e) {
		CK(cudaMemsetAsync(g->err, 0, sizeof(int), g->stream));
		fgh_set_error("gnn: matrix graph needs one nonzero diagonal per row and a symmetric pattern");
		return e;
	}
	return 0;
}

int femgpu_gnn_attach_csr_dev(femgpu_gnn *g, int n, int nnz, const int *IA, const int *JA, const double *AA)
{
	int rc;
	if (!g || n <= 0 || nnz < n || !IA || !JA || !AA) return FEMGPU_E_ARG;
	rc = ensure(g, n, nnz - n);
	if (rc) return rc;
	g->n = n;
	g->nedge = nnz - n;
	KR(fg_gnn_graph(g, n, IA, JA, AA));
	return check_err(g);
}

int femgpu_gnn_attach_csr(femgpu_gnn *g, int n, const int *IA, const int *JA, const double *AA)
{
	int *dIA = NULL, *dJA = NULL, nnz, rc;
	double *dAA = NULL;
	if (!g || n <= 0 || !IA || !JA || !AA) return FEMGPU_E_ARG;
	nnz = IA[n];
	rc = fgh_dmalloc((void **)&dIA, sizeof(int) * ((size_t)n + 1));
	if (!rc) rc = fgh_dmalloc((void **)&dJA, sizeof(int) * (size_t)nnz);
	if (!rc) rc = fgh_dmalloc((void **)&dAA, sizeof(double) * (size_t)nnz);
	if (!rc && (cudaMemcpyAsync(dIA, IA, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice, g->stream) ||
	            cudaMemcpyAsync(dJA, JA, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, g->stream) ||
	            cudaMemcpyAsync(dAA, AA, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, g->stream))) {
		fgh_set_error("gnn: upload failed");
		rc = FEMGPU_E_CUDA;
	}
	if (!rc) rc = femgpu_gnn_attach_csr_dev(g, n, nnz, dIA, dJA, dAA);
	cudaStreamSynchronize(g->stream);
	if (dIA) cudaFree(dIA);
	if (dJA) cudaFree(dJA);
	if (dAA) cudaFree(dAA);
	return rc;
}

int femgpu_gnn_apply_dev(femgpu_gnn *g, const double *r, double *z)
{
	if (!g || !r || !z) return FEMGPU_E_ARG;
	if (!g->n) { fgh_set_error("gnn: no graph attached"); return FEMGPU_E_NOT_BUILT; }
	KR(fg_gnn_forward(g, r, z, 0, NULL));
	return 0;
}

int femgpu_gnn_loss_grad_dev(femgpu_gnn *g, const double *r, const double *t, double *z, int accumulate,
                             double *loss)
{
	if (!g || !r || !t || !z) return FEMGPU_E_ARG;
	if (!g->n) { fgh_set_error("gnn: no graph attached"); return FEMGPU_E_NOT_BUILT; }
	KR(fg_gnn_forward(g, r, z, 1, NULL));
	KR(fg_gnn_backward(g, r, z, t, accumulate));
	if (loss) {
		double a[4], b[4];
		CK(cudaMemcpyAsync(a, g->lsums, sizeof a, cudaMemcpyDeviceToHost, g->stream));
		CK(cudaMemcpyAsync(b, g->lsums2, sizeof b, cudaMemcpyDeviceToHost, g->stream));
		CK(cudaStreamSynchronize(g->stream));
		*loss = a[0] > 0.0 ? a[1] / a[0] : 0.0;
		if (g->loss_kind == GNN_LOSS_BOTH && b[0] > 0.0) *loss += b[1] / b[0];
	}
	return 0;
}

int femgpu_gnn_set_loss(femgpu_gnn *g, int kind)
{
	if (!g || kind < GNN_LOSS_SUPERVISED || kind > GNN_LOSS_BOTH) return FEMGPU_E_ARG;
	g->loss_kind = kind;
	return 0;
}

int femgpu_gnn_adam_step(femgpu_gnn *g, float lr, float gscale)
{
	if (!g) return FEMGPU_E_ARG;
	KR(fg_gnn_adam(g, lr, gscale));
	return 0;
}

/* Host-buffer forms (vectors of n entries). */
static int up(double **d, const double *h, int n, cudaStream_t s)
{
	int rc = fgh_dmalloc((void **)d, sizeof(double) * (size_t)n);
	if (rc) return rc;
	CK(cudaMemcpyAsync(*d, h, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, s));
	return 0;
}

int femgpu_gnn_apply(femgpu_gnn *g, const double *r, double *z)
{
	double *dr = NULL, *dz = NULL;
	int rc;
	if (!g || !r || !z || !g->n) return FEMGPU_E_ARG;
	rc = up(&dr, r, g->n, g->stream);
	if (!rc) rc = fgh_dmalloc((void **)&dz, sizeof(double) * (size_t)g->n);
	if (!rc) rc = femgpu_gnn_apply_dev(g, dr, dz);
	if (!rc && cudaMemcpyAsync(z, dz, sizeof(double) * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream))
		rc = FEMGPU_E_CUDA;
	cudaStreamSynchronize(g->stream);
	if (dr) cudaFree(dr);
	if (dz) cudaFree(dz);
	return rc;
}

int femgpu_gnn_loss_grad(femgpu_gnn *g, const double *r, const double *t, double *loss, float *grad, double *z)
{
	double *dr = NULL, *dt = NULL, *dz = NULL;
	int rc;
	if (!g || !r || !t || !g->n) return FEMGPU_E_ARG;
	rc = up(&dr, r, g->n, g->stream);
	if (!rc) rc = up(&dt, t, g->n, g->stream);
	if (!rc) rc = fgh_dmalloc((void **)&dz, sizeof(double) * (size_t)g->n);
	if (!rc) rc = femgpu_gnn_loss_grad_dev(g, dr, dt, dz, 0, loss);
	if (!rc && z && cudaMemcpyAsync(z, dz, sizeof(double) * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream))
		rc = FEMGPU_E_CUDA;
	if (!rc && grad) rc = femgpu_gnn_get_grad(g, grad);
	cudaStreamSynchronize(g->stream);
	if (dr) cudaFree(dr);
	if (dt) cudaFree(dt);
	if (dz) cudaFree(dz);
	return rc;
}
