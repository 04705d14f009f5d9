/*
 * Host side of the multi-dof element-by-element operators (Euler / Navier-
 * Stokes storage): set-up of the numbering and incidence lists on the device,
 * and the host-buffer / device-pointer entry points of femgpu.h.  Plain C.
 */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_ebe.h"


int femgpu_ebe_create(femgpu_ebe **out, int ndof, int nnodes, int nel, const int *vert,
		const int *node_id, int neq)
{
	femgpu_ebe *c;
	int i;
	size_t m2;
	if (!out || (ndof != 3 && ndof != 4) || nnodes <= 0 || nel <= 0 || neq <= 0 || !vert || !node_id) {
		fgh_set_error("femgpu_ebe_create: bad argument");
		return FEMGPU_E_ARG;
	}
	for (i = 0; i < 3 * nel; i++)
		if (vert[i] < 0 || vert[i] >= nnodes) { fgh_set_error("vertex out of range"); return FEMGPU_E_MESH; }
	for (i = 0; i < nnodes * ndof; i++)
		if (node_id[i] < -1 || node_id[i] >= neq) { fgh_set_error("node id out of range"); return FEMGPU_E_MESH; }
	c = calloc(1, sizeof *c);
	if (!c) return FEMGPU_E_NOMEM;
	c->ndof = ndof; c->m = 3 * ndof; c->nnodes = nnodes; c->nel = nel; c->neq = neq;
	m2 = (size_t)c->m * c->m;
	CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
	c->stream = c->own_stream;
	CK(cudaMalloc((void **)&c->vert, sizeof(int) * 3 * (size_t)nel));
	CK(cudaMalloc((void **)&c->node_id, sizeof(int) * (size_t)nnodes * ndof));
	CK(cudaMalloc((void **)&c->lm, sizeof(int) * (size_t)nel * c->m));
	CK(cudaMalloc((void **)&c->A, sizeof(double) * (size_t)nel * m2));
	CK(cudaMalloc((void **)&c->BD, sizeof(double) * (size_t)nnodes * ndof * ndof));
	CK(cudaMalloc((void **)&c->invBD, sizeof(double) * (size_t)nnodes * ndof * ndof));
	CK(cudaMalloc((void **)&c->P, sizeof(double) * ((size_t)neq + 1)));
	CK(cudaMalloc((void **)&c->Q, sizeof(double) * ((size_t)neq + 1)));
	CK(cudaMemcpy(c->vert, vert, sizeof(int) * 3 * (size_t)nel, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->node_id, node_id, sizeof(int) * (size_t)nnodes * ndof, cudaMemcpyHostToDevice));
	CK(cudaMemsetAsync(c->A, 0, sizeof(double) * (size_t)nel * m2, c->stream));
	KR(fg_ebe_lm(c));
	CK(cudaDeviceSynchronize());
	*out = c;
	return 0;
}

void femgpu_ebe_destroy(femgpu_ebe *c)
{
	int i;
	if (!c) return;
	cudaStreamSynchronize(c->stream);
	{
		void *p[] = { c->vert, c->node_id, c->lm, c->ri_ptr, c->ri, c->ni_ptr, c->ni, c->A, c->BD,
		              c->invBD, c->P, c->Q, c->A32 };
		for (i = 0; i < (int)(sizeof p / sizeof p[0]); i++) if (p[i]) cudaFree(p[i]);
	}
	if (c->own_stream) cudaStreamDestroy(c->own_stream);
	free(c);
}

int femgpu_ebe_set_stream(femgpu_ebe *c, void *stream)
{
	if (!c) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(c->stream));
	c->stream = stream ? (cudaStream_t)stream : c->own_stream;
	return 0;
}

int femgpu_ebe_set_matrix(femgpu_ebe *c, const double *A_host)
{
	if (!c || !A_host) return FEMGPU_E_ARG;
	CK(cudaMemcpyAsync(c->A, A_host, sizeof(double) * (size_t)c->nel * c->m * c->m, cudaMemcpyHostToDevice,
	                   c->stream));
	c->have_bd = 0;
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

double *femgpu_ebe_A_dev(femgpu_ebe *c) { return c ? c->A : NULL; }

int femgpu_ebe_matvec_dev(femgpu_ebe *c, const double *P, double *Q)
{
	if (!c || !P || !Q) return FEMGPU_E_ARG;
	KR(fg_ebe_matvec(c, P, Q, 0));
	return 0;
}

int femgpu_ebe_matvec32_dev(femgpu_ebe *c, const float *P, double *Q)
{
	if (!c || !P || !Q) return FEMGPU_E_ARG;
	if (!c->A32) { fgh_set_error("no FP32 element matrices"); return FEMGPU_E_NOT_BUILT; }
	KR(fg_ebe_matvec32(c, P, Q));
	return 0;
}

int femgpu_ebe_matvec(femgpu_ebe *c, const double *P_host, double *Q_host)
{
	size_t n1;
	if (!c || !P_host || !Q_host) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	CK(cudaMemcpyAsync(c->P, P_host, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	KR(fg_ebe_matvec(c, c->P, c->Q, 0));
	CK(cudaMemcpyAsync(Q_host, c->Q, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_ebe_matvec2_dev(femgpu_ebe *c, const double *P, double *Q, int with_inverse)
{
	if (!c || !P || !Q || c->ndof != 4) return FEMGPU_E_ARG;
	if (!c->have_bd) { fgh_set_error("matvec2 before blockdiag_setup"); return FEMGPU_E_NOT_BUILT; }
	KR(fg_ebe_matvec(c, P, Q, 1));
	KR(fg_ebe_blockdiag_apply(c, P, Q, with_inverse ? 1 : 2));
	return 0;
}

int femgpu_ebe_matvec2(femgpu_ebe *c, const double *P_host, double *Q_host, int with_inverse)
{
	size_t n1;
	int rc;
	if (!c || !P_host || !Q_host) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	CK(cudaMemcpyAsync(c->P, P_host, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	rc = femgpu_ebe_matvec2_dev(c, c->P, c->Q, with_inverse);
	if (rc) return rc;
	CK(cudaMemcpyAsync(Q_host, c->Q, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_ebe_blockdiag_setup(femgpu_ebe *c, double *F_host, double *BD_host, double *invBD_host)
{
	size_t n1, nb;
	if (!c) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	nb = (size_t)c->nnodes * c->ndof * c->ndof;
	KR(fg_ebe_blockdiag_setup(c));
	c->have_bd = 1;
	if (F_host) {
		CK(cudaMemcpyAsync(c->P, F_host, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
		KR(fg_ebe_blockdiag_apply(c, c->P, c->P, 0));
		CK(cudaMemcpyAsync(F_host, c->P, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	}
	if (BD_host) CK(cudaMemcpyAsync(BD_host, c->BD, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
	if (invBD_host) CK(cudaMemcpyAsync(invBD_host, c->invBD, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}

int femgpu_ebe_blockdiag_apply_dev(femgpu_ebe *c, const double *p, double *z)
{
	if (!c || !p || !z) return FEMGPU_E_ARG;
	if (!c->have_bd) { fgh_set_error("blockdiag apply before setup"); return FEMGPU_E_NOT_BUILT; }
	KR(fg_ebe_blockdiag_apply(c, p, z, 0));
	return 0;
}

int femgpu_ebe_blockdiag_apply(femgpu_ebe *c, const double *p_host, double *z_host)
{
	size_t n1;
	int rc;
	if (!c || !p_host || !z_host) return FEMGPU_E_ARG;
	n1 = (size_t)c->neq + 1;
	CK(cudaMemcpyAsync(c->P, p_host, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
	rc = femgpu_ebe_blockdiag_apply_dev(c, c->P, c->P);
	if (rc) return rc;
	CK(cudaMemcpyAsync(z_host, c->P, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return 0;
}
