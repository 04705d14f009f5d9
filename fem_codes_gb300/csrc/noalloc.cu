// Allocation-free residual norm: ||F - A u||^2 and ||F||^2 of a CSR system,
// for callers that cannot allocate device memory (see femgpu.h).
//
// The block partial sums and the last-block ticket live in one file-scope
// __device__ array, so this entry point performs no cudaMalloc / cudaFree and
// calls no allocating library routine.  Every GPU that loads the library
// holds the array until the process exits.  All calls share it: calls that
// overlap on the GPU (different streams, or host threads) race and must be
// serialised by the caller.
#include "fg_common.cuh"
#include <mutex>

#define NA_TPB 256
#define NA_ROWS_PER_THREAD 8
#define NA_MAX_BLOCKS 2048
// Largest system accepted: NA_MAX_BLOCKS * NA_TPB * NA_ROWS_PER_THREAD rows.
#define NA_MAX_ROWS (NA_MAX_BLOCKS * NA_TPB * NA_ROWS_PER_THREAD)
#define NA_MAX_DEVICES 64

// [2*b] = ||r||^2 partial of block b, [2*b+1] = ||F||^2 partial, and the last
// slot is the ticket counter (cleared before each call).
static __device__ __align__(256) double g_na_scratch[2 * NA_MAX_BLOCKS + 32];

__global__ void __launch_bounds__(NA_TPB)
k_resnorm_noalloc(int n, const int *__restrict__ IA, const int *__restrict__ JA,
                  const double *__restrict__ AA, const double *__restrict__ u,
                  const double *__restrict__ F, double *scratch, double *out2)
{
	__shared__ double sr[32], sb[32];
	__shared__ bool last;
	unsigned *ticket = (unsigned *)(scratch + 2 * NA_MAX_BLOCKS);
	double r2 = 0.0, b2 = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double q = 0.0;
		for (int j = IA[i]; j < IA[i + 1]; j++) q = fma(AA[j], u[JA[j]], q);
		double f = F[i], r = f - q;
		r2 = fma(r, r, r2);
		b2 = fma(f, f, b2);
	}
	r2 = fg_warp_sum(r2);
	b2 = fg_warp_sum(b2);
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (lane == 0) { sr[wid] = r2; sb[wid] = b2; }
	__syncthreads();
	if (threadIdx.x == 0) {
		double a = 0.0, c = 0.0;
		for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a += sr[w]; c += sb[w]; }
		scratch[2 * blockIdx.x] = a;
		scratch[2 * blockIdx.x + 1] = c;
		__threadfence();
		last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
	}
	__syncthreads();
	if (last && threadIdx.x == 0) {
		double a = 0.0, c = 0.0;
		for (int b = 0; b < (int)gridDim.x; b++) { a += __ldcg(&scratch[2 * b]); c += __ldcg(&scratch[2 * b + 1]); }
		out2[0] = a;
		out2[1] = c;
		*ticket = 0u;
	}
}

// Device address of the scratch array, looked up with the device current
// (the host-side symbol is only a stand-in, not an address): on a device's
// first call, and again on every call whose stream is not being captured, so
// that after a device reset, or with another context current on the device,
// the call uses the address valid now; a call on a capturing stream reuses
// the address its device's last lookup gave.
static double *g_na_ptr[NA_MAX_DEVICES];
static std::mutex g_na_mu;

static int na_scratch(cudaStream_t s, double **out)
{
	int dev = 0;
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	FG_TRY(cudaGetDevice(&dev));
	if (dev < 0 || dev >= NA_MAX_DEVICES) return FEMGPU_E_ARG;
	FG_TRY(cudaStreamIsCapturing(s, &cap));
	std::lock_guard<std::mutex> lk(g_na_mu);
	if (!g_na_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
		double *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress((void **)&p, g_na_scratch);
		if (e != cudaSuccess || !p) return e != cudaSuccess ? (int)e : FEMGPU_E_CUDA;
		g_na_ptr[dev] = p;
	}
	*out = g_na_ptr[dev];
	return 0;
}

extern "C" int femgpu_csr_resnorm_noalloc(int n, const int *IA, const int *JA, const double *AA,
                                          const double *u, const double *F, double *out2, void *stream)
{
	if (n <= 0 || !IA || !JA || !AA || !u || !F || !out2) return FEMGPU_E_ARG;
	if (n > NA_MAX_ROWS) return FEMGPU_E_ARG;          // beyond the static scratch
	double *scratch = nullptr;
	cudaStream_t s = (cudaStream_t)stream;
	int rc = na_scratch(s, &scratch);
	if (rc) return rc > 0 ? FEMGPU_E_CUDA : rc;
	int blocks = (n + NA_TPB * NA_ROWS_PER_THREAD - 1) / (NA_TPB * NA_ROWS_PER_THREAD);
	if (blocks > NA_MAX_BLOCKS) return FEMGPU_E_ARG;
	// the ticket must start at zero (a previous call may have been cut short)
	if (cudaMemsetAsync(scratch + 2 * NA_MAX_BLOCKS, 0, sizeof(double), s) != cudaSuccess) return FEMGPU_E_CUDA;
	k_resnorm_noalloc<<<blocks, NA_TPB, 0, s>>>(n, IA, JA, AA, u, F, scratch, out2);
	return cudaGetLastError() == cudaSuccess ? 0 : FEMGPU_E_CUDA;
}
