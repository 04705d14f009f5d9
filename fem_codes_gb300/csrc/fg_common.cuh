// Device helpers shared by the libfemgpu kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fg_internal.h"

#define FG_SMS 152               // GB300 streaming multiprocessors
#define FG_TPB 256

#define FG_TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return (int)e_; } while (0)

static inline int fg_grid(long long n, int tpb = FG_TPB, int per_sm = 16)
{
	long long g = (n + tpb - 1) / tpb;
	long long cap = (long long)FG_SMS * per_sm;
	if (g > cap) g = cap;
	if (g < 1) g = 1;
	return (int)g;
}

__device__ __forceinline__ double fg_warp_sum(double v)
{
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

__device__ __forceinline__ float fg_warp_sumf(float v)
{
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// Record the first device-side error code (never traps).
__device__ __forceinline__ void fg_set_err(int *err, int code)
{
	atomicCAS(err, 0, code);
}

// Exclusive scan of n ints (n+1 outputs, out[n] = total); in may equal out.
int fg_scan(const int *in, int *out, int n, cudaStream_t s);
// Lists of the indices i (0 <= i < m) grouped by target[i*stride] in [0, T),
// each list ascending; targets outside [0, T) are skipped.  Allocates *ptr
// (T+1) and *list.
int fg_invert_map(const int *target, int stride, int m, int T, int **ptr, int **list,
                  cudaStream_t s);
