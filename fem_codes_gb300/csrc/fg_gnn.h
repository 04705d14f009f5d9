/* State of the learned preconditioner (mesh graph network, width 32, three
 * message-passing layers).  Plain C; shared by gnn.cu and host/gnn.c.
 *
 * Parameter vector (FP32, GNN_NPARAMS entries):
 *   We [2][32] | be [32] | per layer l: Wh [32][32] | W1 [32][32] | W2 [32][32] | b [32] | Wd [32] | bd
 * (row-major [in][out]).  Device buffers of an attached graph with n nodes:
 * off-diagonal CSR graph gptr [n+1], gcol [E], edge weights wA, wT [E] (FP32),
 * diagonal d [n]; activations h [L+1][n][32], m1, m2 [L][n][32] (bf16 or
 * FP32), ReLU masks [L+1][n] (one bit per feature), encoder inputs x [n]
 * (float2); gradients gh [2][n][32], gm1, gm2 [n][32] (FP32). */
#ifndef FG_GNN_H
#define FG_GNN_H
#include <cuda_runtime_api.h>
#include "femgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GNN_WIDTH 32
#define GNN_LAYERS 3
#define GNN_OFF_WE 0
#define GNN_OFF_BE 64
#define GNN_LAYER_SIZE (3 * 32 * 32 + 32)
#define GNN_OFF_L(l) (96 + (l) * GNN_LAYER_SIZE)
#define GNN_OFF_WD (96 + GNN_LAYERS * GNN_LAYER_SIZE)
#define GNN_OFF_BD (GNN_OFF_WD + 32)
#define GNN_NPARAMS (GNN_OFF_BD + 1)
#define GNN_RED_BLOCKS 304
#define GNN_LOSS_SUPERVISED 0   /* ||z - t||^2 / ||t||^2, t = M^-1 v (ILU target) */
#define GNN_LOSS_RESIDUAL 1     /* ||A z - v||^2 / ||v||^2                      */
#define GNN_LOSS_BOTH 2         /* the sum of the two                           */

struct femgpu_gnn {
	int bf16;                      /* activations stored as bfloat16          */
	cudaStream_t stream, own_stream;
	float *theta, *grad, *am, *av; /* parameters, gradient, Adam moments      */
	int step;                      /* Adam steps taken                        */
	/* attached graph */
	int n, nedge, cap_n, cap_e;
	int *gptr, *gcol;
	float *wA, *wT;
	double *d;
	void *h[GNN_LAYERS + 1], *m1[GNN_LAYERS], *m2[GNN_LAYERS];
	unsigned *mask[GNN_LAYERS + 1];
	void *x;                       /* float2 [n]                              */
	float *gh[2], *gm1, *gm2;
	float *part;                   /* weight-gradient partial sums            */
	double *rpart;                 /* [2*GNN_RED_BLOCKS] reduction partials   */
	double *sums, *stats;          /* [2] each (device)                       */
	double *lsums, *lsums2;        /* [4] loss sums: supervised / residual    */
	double *gz, *res;              /* [n] dL/dz, A z - v                      */
	int loss_kind;                 /* GNN_LOSS_*                              */
	int *err;                      /* device error flag                       */
};
typedef struct femgpu_gnn fg_gnn;

int fg_gnn_graph(fg_gnn *g, int n, const int *IA, const int *JA, const double *AA);
/* z = N(r); train != 0 keeps every layer's activations and masks; active
 * (device flag, may be NULL) skips the work when zero. */
int fg_gnn_forward(fg_gnn *g, const double *r, double *z, int train, const int *active);
/* Gradient of the training loss (loss_kind) of the pair (r, t) after a
 * train forward that produced z (accumulate: add to the stored gradient). */
int fg_gnn_backward(fg_gnn *g, const double *r, const double *z, const double *t, int accumulate);
int fg_gnn_adam(fg_gnn *g, float lr, float gscale);

#ifdef __cplusplus
}
#endif
#endif
