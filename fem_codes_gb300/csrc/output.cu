// Nodal values for output (Paraview_Output.c:24-29 / :38-44): the solution
// of a node's equation, or the node's prescribed value.
#include "fg_common.cuh"

__global__ void k_nodal_values(const double *__restrict__ u, const int *__restrict__ node_id,
                               const double *__restrict__ upresc, int nnodes, double *out)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nnodes; I += gridDim.x * blockDim.x) {
		const int id = node_id[I];
		out[I] = id >= 0 ? u[id] : upresc[I];
	}
}

extern "C" int fg_nodal_values(const double *u, const int *node_id, const double *upresc, int nnodes, double *out,
                               cudaStream_t s)
{
	k_nodal_values<<<fg_grid(nnodes), FG_TPB, 0, s>>>(u, node_id, upresc, nnodes, out);
	return (int)cudaGetLastError();
}
