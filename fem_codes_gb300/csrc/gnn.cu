// Learned preconditioner: a mesh graph network on the graph of the CSR
// matrix, with hand-written forward and backward kernels (no reference
// counterpart; the CPU restatement used by the tests is the oracle's
// gnn_oracle.py).
//
//   s = rms(r), dbar = mean|a_ii|, x_i = [r_i/s, (r_i/s) dbar / a_ii]
//   h0 = relu(We^T x + be)
//   3 layers: m1_i = sum_j (a_ij/a_ii) h_j, m2_i = sum_j (a_ji/a_jj) h_j,
//             h <- h + relu(Wh^T h + W1^T m1 + W2^T m2 + b)
//   z_i = s (Wd . h_i + bd) dbar / a_ii
//
// Weights FP32; activations (h, m1, m2) stored as TA = bf16 (or FP32 for
// exact checks), every accumulation in FP32.  Layout of activations:
// node-major [n][32], one 64-byte (bf16) row per node, so a warp gathers a
// neighbour's row with one coalesced access.  Aggregations run one warp per
// node (lane = feature); the 96->32 updates and their weight gradients run on
// tiles of 64 nodes staged in shared memory.  Weight gradients are reduced
// per block into partial sums, then over blocks in block order
// (deterministic).
#include <algorithm>
#include <type_traits>

#include <cuda_bf16.h>

#include "fg_common.cuh"
#include "fg_gnn.h"

#define W 32
#define TILE 64
#define UPD_TPB 256
#define PAD (3 * W + 1)

template <typename TA> __device__ __forceinline__ float ld_act(const TA *p);
template <> __device__ __forceinline__ float ld_act<float>(const float *p) { return *p; }
template <> __device__ __forceinline__ float ld_act<__nv_bfloat16>(const __nv_bfloat16 *p)
{
	return __bfloat162float(*p);
}
template <typename TA> __device__ __forceinline__ TA st_act(float v);
template <> __device__ __forceinline__ float st_act<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 st_act<__nv_bfloat16>(float v)
{
	return __float2bfloat16_rn(v);
}

// ------------------------------------------------------------ graph set-up
// Off-diagonal graph of a CSR matrix with exactly one diagonal entry per row:
// gptr[i] = IA[i] - i; for each off-diagonal (i, j): col j, wA = a_ij / a_ii,
// wT = a_ji / a_jj (the transposed entry found by binary search in row j).
__global__ void k_gnn_graph(int n, const int *IA, const int *JA, const double *AA, int *gptr, int *gcol,
                            float *wA, float *wT, double *d, int *err)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int lo = IA[i], hi = IA[i + 1], o = lo - i, nd = 0;
		double di = 0.0;
		for (int p = lo; p < hi; p++) if (JA[p] == i) { di = AA[p]; nd++; }
		gptr[i] = o;
		if (i == n - 1) gptr[n] = IA[n] - n;
		d[i] = di;
		if (nd != 1 || di == 0.0) { fg_set_err(err, FEMGPU_E_MESH); continue; }
		for (int p = lo; p < hi; p++) {
			int j = JA[p];
			if (j == i) continue;
			int a = IA[j], b = IA[j + 1] - 1, q = -1;
			while (a <= b) {
				int mid = (a + b) >> 1, c = JA[mid];
				if (c == i) { q = mid; break; }
				if (c < i) a = mid + 1; else b = mid - 1;
			}
			double dj = 0.0;
			for (int t = IA[j]; t < IA[j + 1]; t++) if (JA[t] == j) dj = AA[t];
			gcol[o] = j;
			wA[o] = (float)(AA[p] / di);
			wT[o] = (q >= 0 && dj != 0.0) ? (float)(AA[q] / dj) : 0.0f;
			if (q < 0) fg_set_err(err, FEMGPU_E_MESH);
			o++;
		}
	}
}

// --------------------------------------------------- small deterministic sums
#define RTPB 256
__device__ __forceinline__ double blk_sum(double v, double *sh)
{
	v = fg_warp_sum(v);
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (lane == 0) sh[wid] = v;
	__syncthreads();
	double r = 0.0;
	if (wid == 0) {
		r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
		r = fg_warp_sum(r);
	}
	__syncthreads();
	return r;
}

// Per-block partial sums: part[2b] = sum a_i^2 (or |a_i| when absval),
// part[2b+1] = sum (b_i - a_i)^2 when b != NULL; then one thread adds the
// partials in block order (deterministic).
__global__ void __launch_bounds__(RTPB) k_gnn_psums(int n, const double *a, const double *b, int absval,
                                                    double *part, const int *active)
{
	if (active && !*active) return;
	__shared__ double sh[32];
	double s0 = 0.0, s1 = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double v = a[i];
		s0 += absval ? fabs(v) : v * v;
		if (b) { double e = b[i] - v; s1 += e * e; }
	}
	s0 = blk_sum(s0, sh);
	s1 = blk_sum(s1, sh);
	if (threadIdx.x == 0) { part[2 * blockIdx.x] = s0; part[2 * blockIdx.x + 1] = s1; }
}

// One block of 256 threads: thread t adds partials t, t+256, ... in order,
// then a fixed shuffle tree (deterministic for a given block count).
__global__ void __launch_bounds__(RTPB) k_gnn_fsums(int nblk, const double *part, double *out, const int *active)
{
	if (active && !*active) return;
	__shared__ double sh[32];
	double s0 = 0.0, s1 = 0.0;
	for (int b = threadIdx.x; b < nblk; b += blockDim.x) { s0 += part[2 * b]; s1 += part[2 * b + 1]; }
	s0 = blk_sum(s0, sh);
	s1 = blk_sum(s1, sh);
	if (threadIdx.x == 0) { out[0] = s0; out[1] = s1; }
}

// ------------------------------------------------------------------ forward
// stats: [0] = s (rms of r, 1 if zero), [1] = dbar.
// A warp takes 32 consecutive nodes: lane q computes node q's scaled inputs
// (the FP64 arithmetic once per node), then for each node of the group the
// lanes compute its 32 features (lane = feature) and store one 64-byte row.
template <typename TA>
__global__ void k_gnn_encode(int n, const double *r, const double *stats, const double *d,
                             const float *__restrict__ th, TA *h0, unsigned *mask0, float2 *x, const int *active)
{
	if (active && !*active) return;
	const int lane = threadIdx.x & 31;
	const float w0 = th[GNN_OFF_WE + lane], w1 = th[GNN_OFF_WE + W + lane], b = th[GNN_OFF_BE + lane];
	const double s = stats[0], dbar = stats[1];
	int warps = (gridDim.x * blockDim.x) >> 5;
	for (int g0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; g0 < n; g0 += warps * 32) {
		int i = g0 + lane;
		float rh = 0.0f, x1 = 0.0f;
		if (i < n) {
			rh = (float)(r[i] / s);
			x1 = rh * (float)dbar / (float)d[i];
			if (x) x[i] = make_float2(rh, x1);
		}
		unsigned mine = 0;
		int cnt = min(32, n - g0);
		for (int q = 0; q < cnt; q++) {
			float a = __shfl_sync(0xffffffffu, rh, q), c = __shfl_sync(0xffffffffu, x1, q);
			float pre = a * w0 + c * w1 + b;
			unsigned m = __ballot_sync(0xffffffffu, pre > 0.0f);
			if (lane == q) mine = m;
			h0[(size_t)(g0 + q) * W + lane] = st_act<TA>(pre > 0.0f ? pre : 0.0f);
		}
		if (mask0 && i < n) mask0[i] = mine;
	}
}

// m1_i = sum wA h_j, m2_i = sum wT h_j: one warp per node, lane = feature.
// Quarter-warp per node (four nodes in flight per warp): lane l of group
// l/8 owns features 4*(l%8) .. +4 and gathers them with one 8-byte (bf16) or
// 16-byte (FP32) load per neighbour.
template <typename TA>
__global__ void k_gnn_agg(int n, const int *__restrict__ gptr, const int *__restrict__ gcol,
                          const float *__restrict__ wA, const float *__restrict__ wT, const TA *__restrict__ h,
                          TA *m1, TA *m2, const int *active)
{
	if (active && !*active) return;
	typedef typename std::conditional<sizeof(TA) == 2, uint2, uint4>::type V4;
	const int lane = threadIdx.x & 31, sub = lane >> 3, fl = (lane & 7) * 4;
	int groups = (gridDim.x * blockDim.x) >> 3;
	for (int i = ((blockIdx.x * blockDim.x + threadIdx.x) >> 3); i - sub < n; i += groups) {
		float a1[4] = {0.0f, 0.0f, 0.0f, 0.0f}, a2[4] = {0.0f, 0.0f, 0.0f, 0.0f};
		if (i < n) {
			int lo = __ldg(&gptr[i]), hi = __ldg(&gptr[i + 1]);
			#pragma unroll 2
			for (int p = lo; p < hi; p++) {
				int j = __ldg(&gcol[p]);
				float wa = __ldg(&wA[p]), wt = __ldg(&wT[p]);
				V4 raw = __ldg(reinterpret_cast<const V4 *>(&h[(size_t)j * W + fl]));
				const TA *v = reinterpret_cast<const TA *>(&raw);
				#pragma unroll
				for (int q = 0; q < 4; q++) {
					float hv = ld_act(&v[q]);
					a1[q] += wa * hv;
					a2[q] += wt * hv;
				}
			}
			V4 o1, o2;
			TA *p1 = reinterpret_cast<TA *>(&o1), *p2 = reinterpret_cast<TA *>(&o2);
			#pragma unroll
			for (int q = 0; q < 4; q++) { p1[q] = st_act<TA>(a1[q]); p2[q] = st_act<TA>(a2[q]); }
			*reinterpret_cast<V4 *>(&m1[(size_t)i * W + fl]) = o1;
			*reinterpret_cast<V4 *>(&m2[(size_t)i * W + fl]) = o2;
		}
	}
}

// h_out = h + relu(Wh^T h + W1^T m1 + W2^T m2 + b) on tiles of UTILE = 128
// nodes; thread t computes outputs 8*(t%4) .. +8 of nodes t/4 + 64 q (q < 2),
// so each shared-memory weight load feeds two nodes.  Inputs are staged as
// FP32 rows of 96 (+1 pad) in shared memory with 16-byte global loads.
#define UTILE 128
#define UNODE (UTILE / (UPD_TPB / 4))
template <typename TA>
__global__ void __launch_bounds__(UPD_TPB) k_gnn_update(int n, const float *__restrict__ th, const TA *h,
		const TA *m1, const TA *m2, TA *hout, unsigned *mask, const int *active)
{
	if (active && !*active) return;
	extern __shared__ __align__(16) float dyn[];
	float *sW = dyn;                                   // [3*W*W + W]
	float *sin_ = dyn + 3 * W * W + W;                 // [UTILE][PAD]
	for (int k = threadIdx.x; k < 3 * W * W + W; k += blockDim.x) sW[k] = th[k];
	const int t = threadIdx.x, node = t >> 2, fo = (t & 3) * 8;
	constexpr int VEC = 16 / sizeof(TA);               // elements per 16-byte load
	int ntile = (n + UTILE - 1) / UTILE;
	for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
		int base = tile * UTILE;
		__syncthreads();
		for (int e = t; e < UTILE * 3 * W / VEC; e += blockDim.x) {
			int nd = e / (3 * W / VEC), kv = (e - nd * (3 * W / VEC)) * VEC, i = base + nd;
			const TA *src = kv < W ? h : (kv < 2 * W ? m1 : m2);
			float *dst = &sin_[nd * PAD + kv];
			if (i < n) {
				uint4 raw = *reinterpret_cast<const uint4 *>(&src[(size_t)i * W + (kv & (W - 1))]);
				const TA *v = reinterpret_cast<const TA *>(&raw);
				#pragma unroll
				for (int q = 0; q < VEC; q++) dst[q] = ld_act(&v[q]);
			} else {
				#pragma unroll
				for (int q = 0; q < VEC; q++) dst[q] = 0.0f;
			}
		}
		__syncthreads();
		float acc[UNODE][8];
		#pragma unroll
		for (int q = 0; q < UNODE; q++)
			#pragma unroll
			for (int j = 0; j < 8; j++) acc[q][j] = sW[3 * W * W + fo + j];
		#pragma unroll 4
		for (int k = 0; k < 3 * W; k++) {
			const float4 *wr = reinterpret_cast<const float4 *>(&sW[k * W + fo]);
			float4 w0 = wr[0], w1 = wr[1];
			#pragma unroll
			for (int q = 0; q < UNODE; q++) {
				float v = sin_[(node + 64 * q) * PAD + k];
				acc[q][0] += v * w0.x; acc[q][1] += v * w0.y; acc[q][2] += v * w0.z; acc[q][3] += v * w0.w;
				acc[q][4] += v * w1.x; acc[q][5] += v * w1.y; acc[q][6] += v * w1.z; acc[q][7] += v * w1.w;
			}
		}
		#pragma unroll
		for (int q = 0; q < UNODE; q++) {
			int nd = node + 64 * q, i = base + nd;
			const float *in = &sin_[nd * PAD];
			unsigned bits = 0;
			#pragma unroll
			for (int j = 0; j < 8; j++) {
				float u = acc[q][j];
				bits |= (u > 0.0f ? 1u : 0u) << (fo + j);
				if (i < n) hout[(size_t)i * W + fo + j] = st_act<TA>(in[fo + j] + (u > 0.0f ? u : 0.0f));
			}
			bits |= __shfl_xor_sync(0xffffffffu, bits, 1);
			bits |= __shfl_xor_sync(0xffffffffu, bits, 2);
			if (mask && i < n && (t & 3) == 0) mask[i] = bits;
		}
	}
}

// The same update for bf16 activations on the tensor cores (mma.sync
// m16n8k16, bf16 operands, FP32 accumulation).  Each FP32 weight is split
// into bf16 parts w = hi + lo (|w - hi - lo| <= 2^-16 |w|) and both parts
// are multiplied, so the product keeps the FP32 weights; the activations are
// bf16 already.  A 128-node tile is staged as bf16 rows of MPAD in shared
// memory (16-byte loads, no conversion); warp w of 8 takes nodes 16w..16w+15
// and all 32 outputs (4 fragments of 8 columns) over K = 96 in 6 steps.  The
// row stride of 104 elements (52 words) puts the 8 rows a fragment load
// touches in 8 distinct groups of 4 banks.
#define MPAD (3 * W + 8)
#define MMA_SMEM ((2 * W * MPAD + UTILE * MPAD) * (int)sizeof(__nv_bfloat16) + W * (int)sizeof(float))
__device__ __forceinline__ unsigned ld_pair(const __nv_bfloat16 *p)
{
	return *reinterpret_cast<const unsigned *>(p);
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1)
{
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	             "{%0,%1,%2,%3};"
	             : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	             : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
__global__ void __launch_bounds__(UPD_TPB) k_gnn_update_mma(int n, const float *__restrict__ th,
		const __nv_bfloat16 *h, const __nv_bfloat16 *m1, const __nv_bfloat16 *m2, __nv_bfloat16 *hout,
		unsigned *mask, const int *active)
{
	if (active && !*active) return;
	extern __shared__ __align__(16) unsigned char dynb[];
	__nv_bfloat16 *sWh = reinterpret_cast<__nv_bfloat16 *>(dynb);   // [W][MPAD]: W^T, row = output
	__nv_bfloat16 *sWl = sWh + W * MPAD;
	__nv_bfloat16 *sA = sWl + W * MPAD;                              // [UTILE][MPAD]: [h, m1, m2]
	float *sB = reinterpret_cast<float *>(sA + UTILE * MPAD);       // bias [W]
	for (int e = threadIdx.x; e < 3 * W * W; e += blockDim.x) {
		int k = e / W, o = e - k * W;
		float w = th[e];
		__nv_bfloat16 hi = __float2bfloat16_rn(w);
		sWh[o * MPAD + k] = hi;
		sWl[o * MPAD + k] = __float2bfloat16_rn(w - __bfloat162float(hi));
	}
	if (threadIdx.x < W) sB[threadIdx.x] = th[3 * W * W + threadIdx.x];
	const int t = threadIdx.x, lane = t & 31, warp = t >> 5, g = lane >> 2, c = (lane & 3) * 2;
	int ntile = (n + UTILE - 1) / UTILE;
	for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
		int base = tile * UTILE;
		__syncthreads();
		for (int e = t; e < UTILE * 12; e += blockDim.x) {          // 3 sources x 4 16-byte parts per node
			int nd = e / 12, q = e - nd * 12, src = q >> 2, part = q & 3, i = base + nd;
			const __nv_bfloat16 *sp = src == 0 ? h : (src == 1 ? m1 : m2);
			uint4 v = make_uint4(0u, 0u, 0u, 0u);
			if (i < n) v = *reinterpret_cast<const uint4 *>(&sp[(size_t)i * W + part * 8]);
			*reinterpret_cast<uint4 *>(&sA[nd * MPAD + src * W + part * 8]) = v;
		}
		__syncthreads();
		float acc[4][4];
		#pragma unroll
		for (int nt = 0; nt < 4; nt++) {
			acc[nt][0] = acc[nt][2] = sB[nt * 8 + c];
			acc[nt][1] = acc[nt][3] = sB[nt * 8 + c + 1];
		}
		const __nv_bfloat16 *r0 = sA + (warp * 16 + g) * MPAD, *r1 = r0 + 8 * MPAD;
		#pragma unroll
		for (int ks = 0; ks < 3 * W / 16; ks++) {
			const int k0 = ks * 16 + c;
			unsigned a0 = ld_pair(r0 + k0), a1 = ld_pair(r1 + k0), a2 = ld_pair(r0 + k0 + 8), a3 = ld_pair(r1 + k0 + 8);
			#pragma unroll
			for (int nt = 0; nt < 4; nt++) {
				const __nv_bfloat16 *bh = sWh + (nt * 8 + g) * MPAD + k0, *bl = sWl + (nt * 8 + g) * MPAD + k0;
				mma_bf16(acc[nt], a0, a1, a2, a3, ld_pair(bh), ld_pair(bh + 8));
				mma_bf16(acc[nt], a0, a1, a2, a3, ld_pair(bl), ld_pair(bl + 8));
			}
		}
		#pragma unroll
		for (int rr = 0; rr < 2; rr++) {
			int nd = warp * 16 + g + 8 * rr, i = base + nd;
			const __nv_bfloat16 *in = sA + nd * MPAD;
			unsigned bits = 0;
			#pragma unroll
			for (int nt = 0; nt < 4; nt++) {
				int col = nt * 8 + c;
				float u0 = acc[nt][2 * rr], u1 = acc[nt][2 * rr + 1];
				bits |= (u0 > 0.0f ? 1u : 0u) << col;
				bits |= (u1 > 0.0f ? 1u : 0u) << (col + 1);
				__nv_bfloat162 o;
				o.x = __float2bfloat16_rn(__bfloat162float(in[col]) + (u0 > 0.0f ? u0 : 0.0f));
				o.y = __float2bfloat16_rn(__bfloat162float(in[col + 1]) + (u1 > 0.0f ? u1 : 0.0f));
				if (i < n) *reinterpret_cast<__nv_bfloat162 *>(&hout[(size_t)i * W + col]) = o;
			}
			bits |= __shfl_xor_sync(0xffffffffu, bits, 1);
			bits |= __shfl_xor_sync(0xffffffffu, bits, 2);
			if (mask && i < n && (lane & 3) == 0) mask[i] = bits;
		}
	}
}

// z_i = s (Wd . h_i + bd) dbar / d_i: a warp reduces the rows of 32
// consecutive nodes (lane = feature), lane q keeps node q's sum and does its
// FP64 scaling (once per node).
template <typename TA>
__global__ void k_gnn_decode(int n, const TA *h, const float *__restrict__ th, const double *stats,
                             const double *d, double *z, const int *active)
{
	if (active && !*active) return;
	const int lane = threadIdx.x & 31;
	const float wd = th[GNN_OFF_WD + lane], bd = th[GNN_OFF_BD];
	const double s = stats[0], dbar = stats[1];
	int warps = (gridDim.x * blockDim.x) >> 5;
	for (int g0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; g0 < n; g0 += warps * 32) {
		int cnt = min(32, n - g0);
		float mine = 0.0f;
		for (int q = 0; q < cnt; q++) {
			float y = fg_warp_sumf(ld_act(&h[(size_t)(g0 + q) * W + lane]) * wd);
			if (lane == q) mine = y;
		}
		int i = g0 + lane;
		if (i < n) z[i] = s * (double)(mine + bd) * dbar / d[i];
	}
}

// Loss gradients dL/dz: supervised (ILU target) 2 (z - t) / sum t^2, and
// residual 2 A^T (A z - v) / sum v^2 with A = diag(d) (I + W) from the graph
// (a_ij = d_i wA_ij; (A^T y)_j = d_j y_j + sum_q wT[q] d_col y_col).
__global__ void k_gnn_gz_sup(int n, const double *z, const double *t, const double *sums, double *gz, int add)
{
	const double T2 = sums[0];
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double g = 2.0 * (z[i] - t[i]) / T2;
		gz[i] = add ? gz[i] + g : g;
	}
}

__global__ void k_gnn_resid(int n, const int *__restrict__ gptr, const int *__restrict__ gcol,
                            const float *__restrict__ wA, const double *d, const double *z, const double *v,
                            double *res)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double s = z[i];
		for (int p = gptr[i]; p < gptr[i + 1]; p++) s += (double)wA[p] * z[gcol[p]];
		res[i] = d[i] * s - v[i];
	}
}

__global__ void k_gnn_gz_res(int n, const int *__restrict__ gptr, const int *__restrict__ gcol,
                             const float *__restrict__ wT, const double *d, const double *res, const double *sums,
                             double scale, double *gz, int add)
{
	const double c = scale * 2.0 / sums[0];
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
		double s = d[j] * res[j];
		for (int q = gptr[j]; q < gptr[j + 1]; q++) {
			int i = gcol[q];
			s += (double)wT[q] * d[i] * res[i];
		}
		gz[j] = add ? gz[j] + c * s : c * s;
	}
}

// gh = gy Wd with gy = gz s dbar / d; partials of gWd (32), gbd (1).
template <typename TA>
__global__ void __launch_bounds__(RTPB) k_gnn_decode_bwd(int n, const double *gzv, const double *stats,
		const double *d, const TA *h, const float *__restrict__ th, float *gh, float *part)
{
	__shared__ float sacc[RTPB / 32][W + 1];
	const double s = stats[0], dbar = stats[1];
	float wd[W];
	#pragma unroll
	for (int f = 0; f < W; f++) wd[f] = th[GNN_OFF_WD + f];
	float acc[W + 1];
	#pragma unroll
	for (int f = 0; f <= W; f++) acc[f] = 0.0f;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		float gy = (float)(gzv[i] * s * dbar / d[i]);
		#pragma unroll
		for (int f = 0; f < W; f++) {
			gh[(size_t)i * W + f] = gy * wd[f];
			acc[f] += gy * ld_act(&h[(size_t)i * W + f]);
		}
		acc[W] += gy;
	}
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	#pragma unroll
	for (int f = 0; f <= W; f++) {
		float v = fg_warp_sumf(acc[f]);
		if (lane == 0) sacc[wid][f] = v;
	}
	__syncthreads();
	if (threadIdx.x <= W) {
		float v = 0.0f;
		for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sacc[w][threadIdx.x];
		part[(size_t)blockIdx.x * (W + 1) + threadIdx.x] = v;
	}
}

// One layer backward on tiles of 64 nodes:
//   gu = gh_out * [u > 0];  gh_in = gh_out + Wh gu;  gm1 = W1 gu;  gm2 = W2 gu
//   partials: gWh, gW1, gW2 (sum over nodes of input (x) gu), gb (sum gu).
template <typename TA>
__global__ void __launch_bounds__(UPD_TPB) k_gnn_update_bwd(int n, const float *__restrict__ th, const TA *h,
		const TA *m1, const TA *m2, const unsigned *mask, const float *gh_out, float *gh_in, float *gm1,
		float *gm2, float *part)
{
	__shared__ __align__(16) float sWT[3 * W * W];     // transposed: sWT[m][f][k] = W_m[k][f]
	__shared__ float sin_[TILE * PAD];
	__shared__ float sgu[TILE * (W + 1)];
	for (int e = threadIdx.x; e < 3 * W * W; e += blockDim.x) {
		int m = e / (W * W), r = e - m * W * W, f = r / W, k = r - f * W;
		sWT[e] = th[m * W * W + k * W + f];
	}
	const int t = threadIdx.x, node = t >> 2, fo = (t & 3) * 8;
	float acc[12], accb = 0.0f;
	#pragma unroll
	for (int q = 0; q < 12; q++) acc[q] = 0.0f;
	int ntile = (n + TILE - 1) / TILE;
	for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
		int base = tile * TILE;
		__syncthreads();
		for (int e = t; e < TILE * 3 * W; e += blockDim.x) {
			int nd = e / (3 * W), k = e - nd * 3 * W, i = base + nd;
			float v = 0.0f;
			if (i < n) {
				const TA *src = k < W ? h : (k < 2 * W ? m1 : m2);
				v = ld_act(&src[(size_t)i * W + (k & (W - 1))]);
			}
			sin_[nd * PAD + k] = v;
		}
		for (int e = t; e < TILE * W; e += blockDim.x) {
			int nd = e / W, f = e - nd * W, i = base + nd;
			float g = 0.0f;
			if (i < n && ((mask[i] >> f) & 1u)) g = gh_out[(size_t)i * W + f];
			sgu[nd * (W + 1) + f] = g;
		}
		__syncthreads();
		// input gradients of this thread's node, features fo..fo+8
		{
			int i = base + node;
			float a0[8], a1[8], a2[8];
			#pragma unroll
			for (int j = 0; j < 8; j++) { a0[j] = 0.0f; a1[j] = 0.0f; a2[j] = 0.0f; }
			const float *gu = &sgu[node * (W + 1)];
			#pragma unroll 4
			for (int f = 0; f < W; f++) {
				float g = gu[f];
				#pragma unroll
				for (int j = 0; j < 8; j++) {
					a0[j] += sWT[0 * W * W + f * W + fo + j] * g;
					a1[j] += sWT[1 * W * W + f * W + fo + j] * g;
					a2[j] += sWT[2 * W * W + f * W + fo + j] * g;
				}
			}
			if (i < n) {
				#pragma unroll
				for (int j = 0; j < 8; j++) {
					size_t o = (size_t)i * W + fo + j;
					gh_in[o] = gh_out[o] + a0[j];
					gm1[o] = a1[j];
					gm2[o] = a2[j];
				}
			}
		}
		// weight-gradient partials: entry e = t + 256 q of the 3 x 32 x 32 block
		#pragma unroll
		for (int q = 0; q < 12; q++) {
			int e = t + UPD_TPB * q, m = e >> 10, k = (e >> 5) & (W - 1), f = e & (W - 1);
			float s = 0.0f;
			for (int nd = 0; nd < TILE; nd++) s += sin_[nd * PAD + m * W + k] * sgu[nd * (W + 1) + f];
			acc[q] += s;
		}
		if (t < W)
			for (int nd = 0; nd < TILE; nd++) accb += sgu[nd * (W + 1) + t];
	}
	float *pb = part + (size_t)blockIdx.x * (3 * W * W + W);
	#pragma unroll
	for (int q = 0; q < 12; q++) pb[t + UPD_TPB * q] = acc[q];
	if (t < W) pb[3 * W * W + t] = accb;
}

// gh_j += sum_q wT[q] gm1[col_q] + wA[q] gm2[col_q] (transpose of k_gnn_agg).
__global__ void k_gnn_agg_bwd(int n, const int *__restrict__ gptr, const int *__restrict__ gcol,
                              const float *__restrict__ wA, const float *__restrict__ wT, const float *gm1,
                              const float *gm2, float *gh)
{
	int lane = threadIdx.x & 31;
	int warps = (gridDim.x * blockDim.x) >> 5;
	for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += warps) {
		float a = 0.0f;
		int lo = __ldg(&gptr[j]), hi = __ldg(&gptr[j + 1]);
		for (int q = lo; q < hi; q++) {
			int i = __ldg(&gcol[q]);
			a += __ldg(&wT[q]) * gm1[(size_t)i * W + lane] + __ldg(&wA[q]) * gm2[(size_t)i * W + lane];
		}
		gh[(size_t)j * W + lane] += a;
	}
}

// gpre = gh * [pre > 0]; partials gWe (2 x 32), gbe (32).
__global__ void __launch_bounds__(RTPB) k_gnn_encode_bwd(int n, const float2 *x, const unsigned *mask0,
                                                         const float *gh, float *part)
{
	__shared__ float sacc[RTPB / 32][3 * W];
	float acc[3 * W];
	#pragma unroll
	for (int f = 0; f < 3 * W; f++) acc[f] = 0.0f;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		float2 xi = x[i];
		unsigned m = mask0[i];
		#pragma unroll
		for (int f = 0; f < W; f++) {
			float g = ((m >> f) & 1u) ? gh[(size_t)i * W + f] : 0.0f;
			acc[f] += xi.x * g;
			acc[W + f] += xi.y * g;
			acc[2 * W + f] += g;
		}
	}
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	#pragma unroll
	for (int f = 0; f < 3 * W; f++) {
		float v = fg_warp_sumf(acc[f]);
		if (lane == 0) sacc[wid][f] = v;
	}
	__syncthreads();
	for (int f = threadIdx.x; f < 3 * W; f += blockDim.x) {
		float v = 0.0f;
		for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sacc[w][f];
		part[(size_t)blockIdx.x * 3 * W + f] = v;
	}
}

// grad[off + e] (+)= sum over blocks of part[b][e], in block order.
__global__ void k_gnn_reduce(int nblk, int cnt, const float *part, float *grad, int accumulate)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += gridDim.x * blockDim.x) {
		float s = 0.0f;
		for (int b = 0; b < nblk; b++) s += part[(size_t)b * cnt + e];
		grad[e] = accumulate ? grad[e] + s : s;
	}
}

__global__ void k_gnn_adam(int P, float *th, const float *g, float *m, float *v, float lr, float b1, float b2,
                           float eps, float c1, float c2, float gscale)
{
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P; k += gridDim.x * blockDim.x) {
		float gk = g[k] * gscale;
		float mk = b1 * m[k] + (1.0f - b1) * gk;
		float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
		m[k] = mk;
		v[k] = vk;
		th[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
	}
}

// ls[0..1] = (sum v^2, -), ls[2..3] = (sum res^2, -) -> ls[1] = sum res^2.
__global__ void k_gnn_fix_sums(double *ls) { ls[1] = ls[2]; }

__global__ void k_gnn_stats(const double *sums, int n, double *stats, const int *active)
{
	if (active && !*active) return;
	double s = sqrt(sums[0] / n);
	stats[0] = s > 0.0 ? s : 1.0;
}

__global__ void k_gnn_dbar(const double *sums, int n, double *stats) { stats[1] = sums[0] / n; }

// ---------------------------------------------------------------- launchers
#define UPD_SMEM ((3 * W * W + W + UTILE * PAD) * (int)sizeof(float))

static int update_attrs()
{
	static int done = 0;
	if (!done) {
		FG_TRY(cudaFuncSetAttribute(k_gnn_update<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, UPD_SMEM));
		FG_TRY(cudaFuncSetAttribute(k_gnn_update<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                            UPD_SMEM));
		FG_TRY(cudaFuncSetAttribute(k_gnn_update_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, MMA_SMEM));
		done = 1;
	}
	return 0;
}
// bf16 activations take the tensor-core update unless FEMGPU_GNN_MMA=0
// (read at every launch: the FP32-core form stays available for comparison)
static bool update_mma()
{
	const char *e = getenv("FEMGPU_GNN_MMA");
	return !(e && e[0] == '0');
}
static int nb(long long n, int tpb, int cap)
{
	return (int)std::max<long long>(1, std::min<long long>((n + tpb - 1) / tpb, cap));
}

static void sums(fg_gnn *g, int n, const double *a, const double *b, int absval, double *out,
                 const int *active = nullptr)
{
	k_gnn_psums<<<GNN_RED_BLOCKS, RTPB, 0, g->stream>>>(n, a, b, absval, g->rpart, active);
	k_gnn_fsums<<<1, RTPB, 0, g->stream>>>(GNN_RED_BLOCKS, g->rpart, out, active);
}

extern "C" int fg_gnn_graph(fg_gnn *g, int n, const int *IA, const int *JA, const double *AA)
{
	k_gnn_graph<<<nb(n, 256, 16 * FG_SMS), 256, 0, g->stream>>>(n, IA, JA, AA, g->gptr, g->gcol, g->wA, g->wT, g->d,
	                                                          &g->err[0]);
	FG_TRY(cudaGetLastError());
	sums(g, n, g->d, nullptr, 1, g->sums);
	k_gnn_dbar<<<1, 1, 0, g->stream>>>(g->sums, n, g->stats);
	return (int)cudaGetLastError();
}

template <typename TA>
static int forward_t(fg_gnn *g, const double *r, double *z, int train, const int *active)
{
	cudaStream_t s = g->stream;
	int n = g->n;
	TA **H = (TA **)g->h, **M1 = (TA **)g->m1, **M2 = (TA **)g->m2;
	FG_TRY((cudaError_t)update_attrs());
	sums(g, n, r, nullptr, 0, g->sums, active);
	k_gnn_stats<<<1, 1, 0, s>>>(g->sums, n, g->stats, active);
	k_gnn_encode<TA><<<nb(n, 256, 16 * FG_SMS), 256, 0, s>>>(n, r, g->stats, g->d, g->theta, H[0],
	                                                         train ? g->mask[0] : nullptr,
	                                                         train ? (float2 *)g->x : nullptr, active);
	for (int l = 0; l < GNN_LAYERS; l++) {
		int cur = train ? l : (l & 1), nxt = train ? l + 1 : ((l + 1) & 1);
		int ml = train ? l : 0;
		k_gnn_agg<TA><<<nb(8LL * n, 256, 32 * FG_SMS), 256, 0, s>>>(n, g->gptr, g->gcol, g->wA, g->wT, H[cur],
		                                                            M1[ml], M2[ml], active);
		if constexpr (std::is_same<TA, __nv_bfloat16>::value) {
			if (update_mma())
				k_gnn_update_mma<<<nb(n, UTILE, 4 * FG_SMS), UPD_TPB, MMA_SMEM, s>>>(
					n, g->theta + GNN_OFF_L(l), H[cur], M1[ml], M2[ml], H[nxt],
					train ? g->mask[l + 1] : nullptr, active);
			else
				k_gnn_update<TA><<<nb(n, UTILE, 4 * FG_SMS), UPD_TPB, UPD_SMEM, s>>>(
					n, g->theta + GNN_OFF_L(l), H[cur], M1[ml], M2[ml], H[nxt],
					train ? g->mask[l + 1] : nullptr, active);
		} else {
			k_gnn_update<TA><<<nb(n, UTILE, 4 * FG_SMS), UPD_TPB, UPD_SMEM, s>>>(n, g->theta + GNN_OFF_L(l), H[cur],
			                                                             M1[ml], M2[ml], H[nxt],
			                                                             train ? g->mask[l + 1] : nullptr, active);
		}
	}
	int last = train ? GNN_LAYERS : (GNN_LAYERS & 1);
	k_gnn_decode<TA><<<nb(n, 256, 16 * FG_SMS), 256, 0, s>>>(n, H[last], g->theta, g->stats, g->d, z,
	                                                                active);
	return (int)cudaGetLastError();
}

extern "C" int fg_gnn_forward(fg_gnn *g, const double *r, double *z, int train, const int *active)
{
	return g->bf16 ? forward_t<__nv_bfloat16>(g, r, z, train, active)
	               : forward_t<float>(g, r, z, train, active);
}

template <typename TA>
static int backward_t(fg_gnn *g, const double *r, const double *z, const double *t, int accumulate)
{
	cudaStream_t s = g->stream;
	int n = g->n;
	TA **H = (TA **)g->h, **M1 = (TA **)g->m1, **M2 = (TA **)g->m2;
	const int PL = 3 * W * W + W;
	int gn = nb(n, 256, 16 * FG_SMS);
	// loss sums in g->lsums: [0] = normaliser, [1] = squared error (loss = [1]/[0])
	if (g->loss_kind != GNN_LOSS_RESIDUAL) {
		sums(g, n, t, z, 0, g->lsums);            // sum t^2, sum (z - t)^2
		k_gnn_gz_sup<<<gn, 256, 0, s>>>(n, z, t, g->lsums, g->gz, 0);
	}
	if (g->loss_kind != GNN_LOSS_SUPERVISED) {
		double *ls = g->loss_kind == GNN_LOSS_RESIDUAL ? g->lsums : g->lsums2;
		k_gnn_resid<<<gn, 256, 0, s>>>(n, g->gptr, g->gcol, g->wA, g->d, z, r, g->res);
		sums(g, n, r, nullptr, 0, ls);            // sum r^2 (the input residual)
		sums(g, n, g->res, nullptr, 0, ls + 2);   // sum (A z - v)^2
		k_gnn_fix_sums<<<1, 1, 0, s>>>(ls);
		k_gnn_gz_res<<<gn, 256, 0, s>>>(n, g->gptr, g->gcol, g->wT, g->d, g->res, ls, 1.0, g->gz,
		                                g->loss_kind == GNN_LOSS_BOTH);
	}
	int gd = nb(n, RTPB, 2 * FG_SMS);
	k_gnn_decode_bwd<TA><<<gd, RTPB, 0, s>>>(n, g->gz, g->stats, g->d, H[GNN_LAYERS], g->theta, g->gh[0],
	                                         g->part);
	k_gnn_reduce<<<1, 64, 0, s>>>(gd, W + 1, g->part, g->grad + GNN_OFF_WD, accumulate);
	int cur = 0;
	int gu = nb(n, TILE, 2 * FG_SMS);
	for (int l = GNN_LAYERS - 1; l >= 0; l--) {
		k_gnn_update_bwd<TA><<<gu, UPD_TPB, 0, s>>>(n, g->theta + GNN_OFF_L(l), H[l], M1[l], M2[l], g->mask[l + 1],
		                                            g->gh[cur], g->gh[cur ^ 1], g->gm1, g->gm2, g->part);
		k_gnn_reduce<<<nb(PL, 256, 64), 256, 0, s>>>(gu, PL, g->part, g->grad + GNN_OFF_L(l), accumulate);
		k_gnn_agg_bwd<<<nb(32LL * n, 256, 32 * FG_SMS), 256, 0, s>>>(n, g->gptr, g->gcol, g->wA, g->wT, g->gm1,
		                                                            g->gm2, g->gh[cur ^ 1]);
		cur ^= 1;
	}
	int ge = nb(n, RTPB, 2 * FG_SMS);
	k_gnn_encode_bwd<<<ge, RTPB, 0, s>>>(n, (const float2 *)g->x, g->mask[0], g->gh[cur], g->part);
	k_gnn_reduce<<<1, 128, 0, s>>>(ge, 3 * W, g->part, g->grad + GNN_OFF_WE, accumulate);
	return (int)cudaGetLastError();
}

extern "C" int fg_gnn_backward(fg_gnn *g, const double *r, const double *z, const double *t, int accumulate)
{
	return g->bf16 ? backward_t<__nv_bfloat16>(g, r, z, t, accumulate)
	               : backward_t<float>(g, r, z, t, accumulate);
}

extern "C" int fg_gnn_adam(fg_gnn *g, float lr, float gscale)
{
	const float b1 = 0.9f, b2 = 0.999f;
	g->step++;
	float c1 = 1.0f - powf(b1, (float)g->step), c2 = 1.0f - powf(b2, (float)g->step);
	k_gnn_adam<<<nb(GNN_NPARAMS, 256, 64), 256, 0, g->stream>>>(GNN_NPARAMS, g->theta, g->grad, g->am, g->av, lr, b1,
	                                                            b2, 1e-8f, c1, c2, gscale);
	return (int)cudaGetLastError();
}
