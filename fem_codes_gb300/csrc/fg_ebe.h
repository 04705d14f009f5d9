/* State of a multi-dof element-by-element operator (Euler ndof 4, Navier-
 * Stokes ndof 3).  Plain C; shared by ebe_block.cu and host/ebe.c.
 * Device layout: lm [nel*m] (m = 3*ndof), element matrices A [nel*m*m]
 * row-major as the reference stores them, dof-row incidence lists ri
 * (code e*m + a, ascending e), node incidence lists ni (code e*3 + a),
 * nodal blocks BD / invBD [nnodes*ndof*ndof]. */
#ifndef FG_EBE_H
#define FG_EBE_H
#include <cuda_runtime_api.h>
#include "femgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

struct femgpu_ebe {
	int ndof, m, nnodes, nel, neq;
	cudaStream_t stream, own_stream;
	int *vert, *node_id, *lm;
	int *ri_ptr, *ri, *ni_ptr, *ni;
	double *A, *BD, *invBD;
	float *A32;             /* FP32 copy of A (mixed-precision solves)  */
	double *P, *Q;          /* scratch for the host-buffer entry points */
	int have_bd;
};

int fg_ebe_lm(femgpu_ebe *c);
int fg_ebe_matvec(femgpu_ebe *c, const double *P, double *Q, int offdiag);
int fg_ebe_blockdiag_setup(femgpu_ebe *c);
/* Block_scaling_EBE's element step (ndof 4): identity rows/columns for the
 * prescribed dofs, each vertex's row block times its invBD. */
int fg_ebe_block_scale(femgpu_ebe *c);
int fg_ebe_blockdiag_apply(femgpu_ebe *c, const double *p, double *z, int mode);
/* Mixed precision: A32 = (float) A; Q = A32 P with FP32 element rows and
 * FP64 row totals; z = D^-1 p in FP64 arithmetic, stored in FP32. */
int fg_ebe_to_f32(femgpu_ebe *c);
int fg_ebe_matvec32(femgpu_ebe *c, const float *P, double *Q);
int fg_ebe_blockdiag_apply32(femgpu_ebe *c, const double *p, float *z);

#ifdef __cplusplus
}
#endif
#endif
