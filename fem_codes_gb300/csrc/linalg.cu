// Linear algebra of the solve loop on the device:
//   * matvecs csrmv.c / ebemv.c / edemv.c as per-row gathers (no atomics; the
//     additions of each row happen in the reference's order), plus FP32-value
//     CSR products for the mixed-precision solve;
//   * diagonal preconditioner (Diag_precond*_setup.c, Diag_precond.c);
//   * the restarted GMRES of pgmres.c:4-211 (left preconditioned) and a
//     flexible, right-preconditioned GMRES judged by the unpreconditioned
//     residual, with Arnoldi, Givens and back-substitution on the device; the
//     inner loop is predicated on a device flag so a whole restart cycle is
//     enqueued without host synchronisation.
// Products and sums in the FP64 parity kernels use __dmul_rn/__dadd_rn so
// they are rounded exactly like the reference compiled without contraction.
// ILU(0) lives in ilu.cu.
#include "fg_common.cuh"
#include "fg_ds.cuh"
#include "fg_gnn.h"
#include "fg_amg.h"
#include <math.h>
#include <stdlib.h>

// ============================================================= matvecs ====
// csrmv.c:15-20, Q[i] = sum_j AA[j] P[JA[j]] in column order, over tiles of
// MV_ROWS consecutive rows.  A block streams its tile's slice of AA and JA
// with coalesced loads (thread t takes entries t, t + MV_ROWS, ...), forms
// each rounded product into shared memory, and then each thread adds up its
// own row's products in column order -- the reference's rounding sequence,
// so the FP64 product is bit-identical while no load is strided by the row
// length.  A tile whose entries exceed MV_CAP is taken in runs of rows that
// fit (a row longer than MV_CAP alone is gathered by its own thread).
// FUSED: the row sums are fused multiply-adds q = fma(a, p, q) over staged
// values and inputs (one FP64 operation per entry instead of two: on this
// part the separately rounded form is bound by the FP64 pipe, the fused one
// by HBM); the FGMRES operator, not bit-identical to csrmv.c.
#define MV_ROWS 256
#define MV_CAP 4096

template <typename T> struct mv_ops;
template <> struct mv_ops<double> {
	static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
	static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};
template <> struct mv_ops<float> {
	static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
	static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};

// The product's output type: FP64, FP32, or double-single.
template <typename TO> __device__ __forceinline__ TO mv_out(double q);
template <> __device__ __forceinline__ double mv_out<double>(double q) { return q; }
template <> __device__ __forceinline__ float mv_out<float>(double q) { return (float)q; }
template <> __device__ __forceinline__ dsf mv_out<dsf>(double q) { return ds_from(q); }

template <typename TA, typename TP, typename TACC, typename TO, bool FUSED>
__global__ void __launch_bounds__(MV_ROWS) k_csrmv_tile(int n, const int *__restrict__ IA,
                                                        const int *__restrict__ JA, const TA *__restrict__ AA,
                                                        const TP *__restrict__ P, TO *__restrict__ Q,
                                                        const int *active)
{
	typedef mv_ops<TACC> op;
	constexpr int CAP = FUSED ? MV_CAP / 2 : MV_CAP;
	if (active && !*active) return;
	__shared__ TACC prod[MV_CAP];                         // FUSED: values [0, CAP), inputs [CAP, 2 CAP)
	__shared__ int kpos[2];
	const int tid = threadIdx.x;
	const int r0 = blockIdx.x * MV_ROWS, r1 = min(r0 + MV_ROWS, n), i = r0 + tid;
	const bool mine = i < r1;
	const int kb = mine ? __ldg(&IA[i]) : 0, ke = mine ? __ldg(&IA[i + 1]) : 0;
	int rs = r0;
	while (rs < r1) {                                     // rs, re, k0, k1 are uniform over the block
		if (i == rs) kpos[0] = kb;
		__syncthreads();
		const int k0 = kpos[0];
		const int re = rs + __syncthreads_count(mine && i >= rs && ke - k0 <= CAP);
		if (re == rs) {                                   // a row longer than CAP
			if (i == rs) {
				TACC q = TACC(0);
				for (int j = kb; j < ke; j++) {
					const TACC a = (TACC)__ldg(&AA[j]), x = (TACC)__ldg(&P[__ldg(&JA[j])]);
					q = FUSED ? fma(a, x, q) : op::add(q, op::mul(a, x));
				}
				Q[i] = mv_out<TO>(q);
			}
			rs = re + 1;
			continue;
		}
		if (i == re - 1) kpos[1] = ke;
		__syncthreads();
		const int k1 = kpos[1];
		int k = k0 + tid;
		for (; k + 3 * MV_ROWS < k1; k += 4 * MV_ROWS) {
			const TA a0 = __ldcs(&AA[k]), a1 = __ldcs(&AA[k + MV_ROWS]);
			const TA a2 = __ldcs(&AA[k + 2 * MV_ROWS]), a3 = __ldcs(&AA[k + 3 * MV_ROWS]);
			const int c0 = __ldcs(&JA[k]), c1 = __ldcs(&JA[k + MV_ROWS]);
			const int c2 = __ldcs(&JA[k + 2 * MV_ROWS]), c3 = __ldcs(&JA[k + 3 * MV_ROWS]);
			const TP p0 = __ldg(&P[c0]), p1 = __ldg(&P[c1]), p2 = __ldg(&P[c2]), p3 = __ldg(&P[c3]);
			if (FUSED) {
				prod[k - k0] = (TACC)a0; prod[CAP + k - k0] = (TACC)p0;
				prod[k - k0 + MV_ROWS] = (TACC)a1; prod[CAP + k - k0 + MV_ROWS] = (TACC)p1;
				prod[k - k0 + 2 * MV_ROWS] = (TACC)a2; prod[CAP + k - k0 + 2 * MV_ROWS] = (TACC)p2;
				prod[k - k0 + 3 * MV_ROWS] = (TACC)a3; prod[CAP + k - k0 + 3 * MV_ROWS] = (TACC)p3;
			} else {
				prod[k - k0] = op::mul((TACC)a0, (TACC)p0);
				prod[k - k0 + MV_ROWS] = op::mul((TACC)a1, (TACC)p1);
				prod[k - k0 + 2 * MV_ROWS] = op::mul((TACC)a2, (TACC)p2);
				prod[k - k0 + 3 * MV_ROWS] = op::mul((TACC)a3, (TACC)p3);
			}
		}
		for (; k < k1; k += MV_ROWS) {
			const TACC a = (TACC)__ldcs(&AA[k]), x = (TACC)__ldg(&P[__ldcs(&JA[k])]);
			if (FUSED) { prod[k - k0] = a; prod[CAP + k - k0] = x; }
			else prod[k - k0] = op::mul(a, x);
		}
		__syncthreads();
		if (i >= rs && i < re) {
			TACC q = TACC(0);
			if (FUSED)
				for (int j = kb - k0; j < ke - k0; j++) q = fma(prod[j], prod[CAP + j], q);
			else
				for (int j = kb - k0; j < ke - k0; j++) q = op::add(q, prod[j]);
			Q[i] = mv_out<TO>(q);
		}
		__syncthreads();                                  // prod and kpos are reused by the next run
		rs = re;
	}
}

template <typename TA, typename TP, typename TACC, typename TO, bool FUSED = false>
static int launch_csrmv(int n, const int *IA, const int *JA, const TA *AA, const TP *P, TO *Q, const int *active,
                        cudaStream_t s)
{
	if (n <= 0) return 0;
	k_csrmv_tile<TA, TP, TACC, TO, FUSED><<<(n + MV_ROWS - 1) / MV_ROWS, MV_ROWS, 0, s>>>(n, IA, JA, AA, P, Q,
	                                                                                     active);
	return (int)cudaGetLastError();
}

extern "C" int fg_csrmv64_fused(int n, const int *IA, const int *JA, const double *AA, const double *P,
                                double *Q, const int *active, cudaStream_t s)
{
	return launch_csrmv<double, double, double, double, true>(n, IA, JA, AA, P, Q, active, s);
}

// The fused product with its result in double-single (the Krylov basis of
// the double-single Arnoldi).
extern "C" int fg_csrmv64_fused_ds(int n, const int *IA, const int *JA, const double *AA, const double *P,
                                   void *Q, const int *active, cudaStream_t s)
{
	return launch_csrmv<double, double, double, dsf, true>(n, IA, JA, AA, P, (dsf *)Q, active, s);
}

extern "C" int fg_csrmv64(int n, const int *IA, const int *JA, const double *AA, const double *P,
                          double *Q, const int *active, cudaStream_t s)
{
	return launch_csrmv<double, double, double, double>(n, IA, JA, AA, P, Q, active, s);
}

extern "C" int fg_csrmv32(int n, const int *IA, const int *JA, const float *AA, const float *P,
                          float *Q, const int *active, cudaStream_t s)
{
	return launch_csrmv<float, float, float, float>(n, IA, JA, AA, P, Q, active, s);
}

// csrmv.c:15-20 over the SELL-32 copy of the matrix: one thread per row,
// the row's entries in column order (separately rounded, as the reference,
// or fused), each warp's loads of an entry index coalesced across its 32
// rows (the slice is stored column by column).  Eight entries per round keep
// eight independent loads in flight.
#define SELL_UNR 8
// GATHER: each result also goes, as a double-single value, to slot dpos[i]
// of G (the ILU sweeps' gathered input, so the look-ahead step's
// preconditioner needs no gather of its own).
template <typename TO, bool FUSED, bool GATHER = false>
__global__ void __launch_bounds__(256) k_sellmv(int n, const long long *__restrict__ base, const int *__restrict__ width,
                                                const int *__restrict__ IA, const int *__restrict__ JS,
                                                const double *__restrict__ AS, const double *__restrict__ P,
                                                TO *__restrict__ Q, const int *active,
                                                const int *__restrict__ dpos = nullptr, dsf *__restrict__ G = nullptr)
{
	if (active && !*active) return;
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int sl = i >> 5;
	const long long b = __ldg(&base[sl]) + (i & 31);
	const int w = __ldg(&width[sl]), len = __ldg(&IA[i + 1]) - __ldg(&IA[i]);
	double q = 0.0;
	for (int j = 0; j < w; j += SELL_UNR) {
		double a[SELL_UNR], p[SELL_UNR];
#pragma unroll
		for (int u = 0; u < SELL_UNR; u++) {
			const bool on = j + u < len;
			a[u] = on ? __ldcs(&AS[b + 32LL * (j + u)]) : 0.0;
			const int c = on ? __ldcs(&JS[b + 32LL * (j + u)]) : 0;
			p[u] = on ? __ldg(&P[c]) : 0.0;
		}
#pragma unroll
		for (int u = 0; u < SELL_UNR; u++)
			if (j + u < len) q = FUSED ? fma(a[u], p[u], q) : __dadd_rn(q, __dmul_rn(a[u], p[u]));
	}
	Q[i] = mv_out<TO>(q);
	if (GATHER) G[__ldg(&dpos[i])] = ds_from(q);
}

__global__ void k_sell_refresh(long long nslot, const int *__restrict__ src, const double *__restrict__ AA,
                               double *__restrict__ AS)
{
	for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nslot;
	     k += (long long)gridDim.x * blockDim.x) {
		const int q = src[k];
		AS[k] = q >= 0 ? AA[q] : 0.0;
	}
}

extern "C" int fg_sell_refresh(femgpu_transport *t)
{
	if (!t->sell_A) return 0;
	k_sell_refresh<<<fg_grid(t->nslot), FG_TPB, 0, t->stream>>>(t->nslot, t->sell_src, t->A, t->sell_A);
	return (int)cudaGetLastError();
}

// The FGMRES operator (fused form) that also writes the ILU sweeps' gathered
// double-single input.
static int sellmv_gather(femgpu_transport *t, const double *P, double *Q, const int *active)
{
	const int n = t->neq, g = (n + 255) / 256;
	k_sellmv<double, true, true><<<g, 256, 0, t->stream>>>(n, t->sell_base, t->sell_w, t->IA, t->sell_JA, t->sell_A, P,
	                                                      Q, active, t->sweeps.dpos, (dsf *)t->sweeps.bl64);
	return (int)cudaGetLastError();
}

extern "C" int fg_sellmv(femgpu_transport *t, const double *P, void *Q, int fused, int ds_out, const int *active)
{
	const int n = t->neq, g = (n + 255) / 256;
	cudaStream_t s = t->stream;
	if (ds_out)
		k_sellmv<dsf, true><<<g, 256, 0, s>>>(n, t->sell_base, t->sell_w, t->IA, t->sell_JA, t->sell_A, P, (dsf *)Q,
		                                     active);
	else if (fused)
		k_sellmv<double, true><<<g, 256, 0, s>>>(n, t->sell_base, t->sell_w, t->IA, t->sell_JA, t->sell_A, P,
		                                        (double *)Q, active);
	else
		k_sellmv<double, false><<<g, 256, 0, s>>>(n, t->sell_base, t->sell_w, t->IA, t->sell_JA, t->sell_A, P,
		                                         (double *)Q, active);
	return (int)cudaGetLastError();
}

// ebemv.c:42-63 gathered per row: for each incident element (ascending),
// Q += A[3a]*p1 + A[3a+1]*p2 + A[3a+2]*p3 with P[neq] read as 0.
__global__ void k_ebemv(int neq, const int *__restrict__ ri_ptr, const int *__restrict__ ri,
                        const int *__restrict__ lm, const double *__restrict__ A,
                        const double *__restrict__ P, double *__restrict__ Q, const int *active)
{
	if (active && !*active) return;
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double q = 0.0;
		if (I < neq) {
			for (int k = __ldg(&ri_ptr[I]); k < __ldg(&ri_ptr[I + 1]); k++) {
				int code = __ldg(&ri[k]), e = code / 3, a = code - 3 * e;
				int l0 = __ldg(&lm[3 * e]), l1 = __ldg(&lm[3 * e + 1]), l2 = __ldg(&lm[3 * e + 2]);
				double p0 = (l0 == neq) ? 0.0 : __ldg(&P[l0]);
				double p1 = (l1 == neq) ? 0.0 : __ldg(&P[l1]);
				double p2 = (l2 == neq) ? 0.0 : __ldg(&P[l2]);
				const double *r = A + 9LL * e + 3 * a;
				double t = __dadd_rn(__dadd_rn(__dmul_rn(__ldg(&r[0]), p0), __dmul_rn(__ldg(&r[1]), p1)),
				                     __dmul_rn(__ldg(&r[2]), p2));
				q = __dadd_rn(q, t);
			}
		}
		Q[I] = q;
	}
}

// edemv.c:90-103 gathered per row: edges (J, I) with J < I (ascending edge
// index) contribute A2*pJ + A3*pI, then edges (I, J) contribute A0*pI + A1*pJ.
__global__ void k_edemv(int neq, const int *__restrict__ first, const int *__restrict__ e2_ptr,
                        const int *__restrict__ e2, const int *__restrict__ lm2,
                        const double *__restrict__ A, const double *__restrict__ P,
                        double *__restrict__ Q, const int *active)
{
	if (active && !*active) return;
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double q = 0.0;
		if (I < neq) {
			double pI = __ldg(&P[I]);
			for (int k = __ldg(&e2_ptr[I]); k < __ldg(&e2_ptr[I + 1]); k++) {
				int E = __ldg(&e2[k]), J = __ldg(&lm2[2 * E]);
				double t = __dadd_rn(__dmul_rn(__ldg(&A[4LL * E + 2]), __ldg(&P[J])),
				                     __dmul_rn(__ldg(&A[4LL * E + 3]), pI));
				q = __dadd_rn(q, t);
			}
			for (int E = __ldg(&first[I]); E < __ldg(&first[I + 1]); E++) {
				int J = __ldg(&lm2[2 * E + 1]);
				double pJ = (J == neq) ? 0.0 : __ldg(&P[J]);
				double t = __dadd_rn(__dmul_rn(__ldg(&A[4LL * E]), pI), __dmul_rn(__ldg(&A[4LL * E + 1]), pJ));
				q = __dadd_rn(q, t);
			}
		}
		Q[I] = q;
	}
}

extern "C" int fg_matvec(femgpu_transport *t, const double *P, double *Q, const int *active)
{
	cudaStream_t s = t->stream;
	if (t->o.scheme == FEMGPU_CSR) {
		if (t->sell_A) return fg_sellmv(t, P, Q, 0, 0, active);
		return fg_csrmv64(t->neq, t->IA, t->JA, t->A, P, Q, active, s);
	}
	if (t->o.scheme == FEMGPU_EBE)
		k_ebemv<<<fg_grid(t->neq + 1LL, 128, 32), 128, 0, s>>>(t->neq, t->ri_ptr, t->ri, t->lm, t->A, P, Q,
		                                                      active);
	else
		k_edemv<<<fg_grid(t->neq + 1LL, 128, 32), 128, 0, s>>>(t->neq, t->IA, t->e2_ptr, t->e2, t->lm2,
		                                                      t->A, P, Q, active);
	return (int)cudaGetLastError();
}

// Operator applied to an FP32 vector (mixed precision, CSR): FP64 values
// with FP64 accumulation (op32 == 0) or FP32 values with FP32 accumulation.
static int matvec_xf(femgpu_transport *t, const float *P, double *Q, const int *active, int op32)
{
	if (op32) return launch_csrmv<float, float, float, double>(t->neq, t->IA, t->JA, t->A32, P, Q, active, t->stream);
	return launch_csrmv<double, float, double, double>(t->neq, t->IA, t->JA, t->A, P, Q, active, t->stream);
}

// ============================================================ diagonal ====
// Diag_precond_CSR_setup.c:13-26, Diag_precond_EBE_setup.c:15-33,
// Diag_precond_EDE_setup.c:14-31: diagonal (summed in the reference's
// order), inverted, then F := F / D (unless the solve is right preconditioned).
__global__ void k_diag_setup(int scheme, int neq, const int *diag, const int *ri_ptr, const int *ri,
                             const int *first, const int *e2_ptr, const int *e2, const double *A,
                             double *invDiag, float *invDiag32, double *F)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x) {
		double d = 0.0;
		if (scheme == FEMGPU_CSR) d = A[diag[I]];
		else if (scheme == FEMGPU_EBE) {
			for (int k = ri_ptr[I]; k < ri_ptr[I + 1]; k++) {
				int code = ri[k], e = code / 3, a = code - 3 * e;
				d = __dadd_rn(d, A[9LL * e + 4 * a]);
			}
		} else {
			for (int k = e2_ptr[I]; k < e2_ptr[I + 1]; k++) d = __dadd_rn(d, A[4LL * e2[k] + 3]);
			for (int E = first[I]; E < first[I + 1]; E++) d = __dadd_rn(d, A[4LL * E]);
		}
		double inv = 1.0 / d;
		invDiag[I] = inv;
		invDiag32[I] = (float)inv;
		if (F) F[I] = __dmul_rn(F[I], inv);
	}
}

__global__ void k_diag_apply(int n, const double *invDiag, const double *p, double *z, const int *active)
{
	if (active && !*active) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		z[i] = __dmul_rn(p[i], invDiag[i]);
}

__global__ void k_diag_apply32(int n, const float *invDiag, const double *p, float *z, const int *active)
{
	if (active && !*active) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		z[i] = (float)p[i] * invDiag[i];
}

__global__ void k_copy_f32(int n, const double *p, float *z, const int *active)
{
	if (active && !*active) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] = (float)p[i];
}

extern "C" int fg_diag_setup(femgpu_transport *t)
{
	k_diag_setup<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(t->o.scheme, t->neq, t->diag, t->ri_ptr, t->ri,
		t->IA, t->e2_ptr, t->e2, t->A, t->invDiag, t->invDiag32,
		t->o.solver == FEMGPU_FGMRES ? nullptr : t->F);
	return (int)cudaGetLastError();
}

// precond / ILUp_precond / Diag_precond in FP64; p may equal z.
extern "C" int fg_precond(femgpu_transport *t, const double *p, double *z, const int *active)
{
	cudaStream_t s = t->stream;
	if (t->o.precond == FEMGPU_PREC_LEARNED && !t->fell_back) return fg_gnn_forward(t->gnn, p, z, 0, active);
	if (t->o.precond == FEMGPU_PREC_AMG || (t->o.precond == FEMGPU_PREC_LEARNED && t->fell_back == 2))
		return fg_amg_vcycle(t->amg, p, z, active);
	if (t->o.precond == FEMGPU_PREC_NOT) {
		if (p != z) FG_TRY(cudaMemcpyAsync(z, p, sizeof(double) * t->neq, cudaMemcpyDeviceToDevice, s));
		return 0;
	}
	if (t->o.precond == FEMGPU_PREC_DIAG) {
		k_diag_apply<<<fg_grid(t->neq), FG_TPB, 0, s>>>(t->neq, t->invDiag, p, z, active);
		return (int)cudaGetLastError();
	}
	return fg_ilu0_apply64(t, p, z, active);
}

// The same preconditioner computed in FP32.
extern "C" int fg_precond32(femgpu_transport *t, const double *p, float *z, const int *active)
{
	cudaStream_t s = t->stream;
	if (t->o.precond == FEMGPU_PREC_NOT) {
		k_copy_f32<<<fg_grid(t->neq), FG_TPB, 0, s>>>(t->neq, p, z, active);
		return (int)cudaGetLastError();
	}
	if (t->o.precond == FEMGPU_PREC_DIAG) {
		k_diag_apply32<<<fg_grid(t->neq), FG_TPB, 0, s>>>(t->neq, t->invDiag32, p, z, active);
		return (int)cudaGetLastError();
	}
	return fg_ilu0_apply32(t, p, z, active);
}

// ========================================================== reductions ====
// Deterministic reduction: block partials, then the last block (by ticket)
// sums them in block order.
#define RED_TPB 256

__device__ __forceinline__ double block_sum(double v, double *sh)
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
	return r;   // valid in thread 0
}

// Returns true in thread 0 of the last block, with *total the ordered sum.
__device__ __forceinline__ bool last_block_total(double part, double *partials, unsigned *ticket,
                                                 double *total, double *sh)
{
	__shared__ bool last;
	if (threadIdx.x == 0) {
		partials[blockIdx.x] = part;
		__threadfence();
		unsigned tk = atomicAdd(ticket, 1u);
		last = (tk == gridDim.x - 1);
	}
	__syncthreads();
	if (!last) return false;
	double v = 0.0;
	for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(&partials[b]);
	v = block_sum(v, sh);
	if (threadIdx.x == 0) { *total = v; *ticket = 0u; }
	return threadIdx.x == 0;
}

__device__ __forceinline__ bool gmres_live(const fg_status *st) { return st->active != 0; }

// MGS step j of iteration i (pgmres.c:107-121), fused:
//   j == 0:       h(0,i) = u0 . w
//   0 < j <= i:   w -= h(j-1,i) u_{j-1};  h(j,i) = u_j . w
//   j == i+1:     w -= h(i,i) u_i;        h(i+1,i) = ||w||
__global__ void __launch_bounds__(RED_TPB) k_mgs(const double *V, size_t ldv, int n, int i, int j,
                                                 double *H, int ldh, double *partials, fg_status *st)
{
	if (!gmres_live(st)) return;
	__shared__ double sh[32];
	double *w = (double *)V + (size_t)(i + 1) * ldv;
	const double *uj = V + (size_t)j * ldv;
	const double *um = (j > 0) ? V + (size_t)(j - 1) * ldv : nullptr;
	double hm = (j > 0) ? H[(j - 1) * ldh + i] : 0.0;
	double part = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double wk = w[k];
		if (j > 0) { wk = __dadd_rn(wk, __dmul_rn(-hm, um[k])); w[k] = wk; }
		part += (j <= i) ? uj[k] * wk : wk * wk;
	}
	part = block_sum(part, sh);
	double tot;
	if (last_block_total(part, partials, &st->ticket, &tot, sh))
		H[j * ldh + i] = (j <= i) ? tot : sqrt(tot);
}

// Classical Gram-Schmidt for FGMRES (the flexible solver's own
// orthogonalisation; the left-preconditioned pgmres keeps the reference's
// MGS above).  One projection = a fused multi-dot h = V^T w over the m basis
// vectors (partial sums per block, then a fixed-order finish: deterministic)
// and one update w -= V h, which can also form ||w||^2.
#define MD_J 8                        // basis vectors per multi-dot block row

__global__ void __launch_bounds__(RED_TPB) k_mdot(const double *V, size_t ldv, int n, int m, const double *w,
                                                  double *partials, fg_status *st)
{
	if (!gmres_live(st)) return;
	__shared__ double sh[MD_J][RED_TPB / 32];
	const int j0 = blockIdx.y * MD_J, G = gridDim.x;
	double acc[MD_J];
#pragma unroll
	for (int q = 0; q < MD_J; q++) acc[q] = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += G * blockDim.x) {
		double wk = w[k];
#pragma unroll
		for (int q = 0; q < MD_J; q++)
			if (j0 + q < m) acc[q] += V[(size_t)(j0 + q) * ldv + k] * wk;
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
	for (int q = 0; q < MD_J; q++) {
		double v = fg_warp_sum(acc[q]);
		if (lane == 0) sh[q][wid] = v;
	}
	__syncthreads();
	if (threadIdx.x < MD_J && j0 + (int)threadIdx.x < m) {
		double t = 0.0;
		for (int q = 0; q < RED_TPB / 32; q++) t += sh[threadIdx.x][q];
		partials[(size_t)(j0 + threadIdx.x) * G + blockIdx.x] = t;
	}
}

// h[j] = sum over blocks of partials[j][.]; H(j, i) = h[j] (accumulate: +=).
__global__ void k_mdot_fin(const double *partials, int G, int m, double *h, double *Hcol, int ldh, int accumulate,
                           fg_status *st)
{
	if (!gmres_live(st)) return;
	const int j = blockIdx.x;
	double t = 0.0;
	for (int b = threadIdx.x; b < G; b += 32) t += partials[(size_t)j * G + b];
	t = fg_warp_sum(t);
	if (threadIdx.x == 0) {
		h[j] = t;
		Hcol[(size_t)j * ldh] = accumulate ? Hcol[(size_t)j * ldh] + t : t;
	}
}

// w = win - sum_j h[j] v_j (win may be w); norm != 0: Hn = ||w|| (last
// block).  The basis entries of a thread's element are loaded CGS_UNR at a
// time ahead of the dependent subtractions (the same order of subtractions),
// so a warp keeps CGS_UNR coalesced loads in flight; the kernel runs on
// CGS_GRID x the reduction grid.  Dynamic shared memory: the m coefficients.
#define CGS_UNR 8
#define CGS_GRID 4
__global__ void __launch_bounds__(RED_TPB) k_cgs_update(const double *V, size_t ldv, int n, int m, const double *win,
                                                        double *w, const double *h, int norm, double *Hn,
                                                        double *partials, fg_status *st)
{
	if (!gmres_live(st)) return;
	extern __shared__ double hsh[];
	__shared__ double sh[32];
	for (int j = threadIdx.x; j < m; j += blockDim.x) hsh[j] = h[j];
	__syncthreads();
	double part = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double x = win[k];
		int j = 0;
		for (; j + CGS_UNR <= m; j += CGS_UNR) {
			double v[CGS_UNR];
#pragma unroll
			for (int u = 0; u < CGS_UNR; u++) v[u] = V[(size_t)(j + u) * ldv + k];
#pragma unroll
			for (int u = 0; u < CGS_UNR; u++) x -= hsh[j + u] * v[u];
		}
		for (; j < m; j++) x -= hsh[j] * V[(size_t)j * ldv + k];
		w[k] = x;
		part += x * x;
	}
	if (!norm) return;
	part = block_sum(part, sh);
	double tot;
	if (last_block_total(part, partials, &st->ticket, &tot, sh)) *Hn = sqrt(tot);
}

// The same CGS kernels and the scaling with the basis in double-single (the
// FGMRES basis on the FP32 pipes: a basis entry is a float pair of 8 bytes
// like an FP64 one, each product and sum is a double-single operation, the
// per-thread partial sums go to FP64 for the block and grid reductions).
__global__ void __launch_bounds__(RED_TPB) k_mdot_ds(const dsf *V, size_t ldv, int n, int m, const dsf *w,
                                                     double *partials, fg_status *st)
{
	if (!gmres_live(st)) return;
	__shared__ double sh[MD_J][RED_TPB / 32];
	const int j0 = blockIdx.y * MD_J, G = gridDim.x;
	dsf acc[MD_J];
#pragma unroll
	for (int q = 0; q < MD_J; q++) acc[q] = dsf{ 0.0f, 0.0f };
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += G * blockDim.x) {
		const dsf wk = w[k];
#pragma unroll
		for (int q = 0; q < MD_J; q++)
			if (j0 + q < m) acc[q] = ds_fma(V[(size_t)(j0 + q) * ldv + k], wk, acc[q]);
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
	for (int q = 0; q < MD_J; q++) {
		double v = fg_warp_sum(ds_to_double(acc[q]));
		if (lane == 0) sh[q][wid] = v;
	}
	__syncthreads();
	if (threadIdx.x < MD_J && j0 + (int)threadIdx.x < m) {
		double t = 0.0;
		for (int q = 0; q < RED_TPB / 32; q++) t += sh[threadIdx.x][q];
		partials[(size_t)(j0 + threadIdx.x) * G + blockIdx.x] = t;
	}
}

// w -= sum_j h[j] v_j; norm != 0: Hn = ||w|| (last block).  Dynamic shared
// memory: m double-single coefficients.
__global__ void __launch_bounds__(RED_TPB) k_cgs_update_ds(const dsf *V, size_t ldv, int n, int m, dsf *w,
                                                           const double *h, int norm, double *Hn,
                                                           double *partials, fg_status *st)
{
	if (!gmres_live(st)) return;
	extern __shared__ dsf hneg[];
	__shared__ double sh[32];
	for (int j = threadIdx.x; j < m; j += blockDim.x) hneg[j] = ds_neg(ds_from(h[j]));
	__syncthreads();
	dsf part = dsf{ 0.0f, 0.0f };
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		dsf x = w[k];
		int j = 0;
		for (; j + CGS_UNR <= m; j += CGS_UNR) {
			dsf v[CGS_UNR];
#pragma unroll
			for (int u = 0; u < CGS_UNR; u++) v[u] = V[(size_t)(j + u) * ldv + k];
#pragma unroll
			for (int u = 0; u < CGS_UNR; u++) x = ds_fma(hneg[j + u], v[u], x);
		}
		for (; j < m; j++) x = ds_fma(hneg[j], V[(size_t)j * ldv + k], x);
		w[k] = x;
		part = ds_fma(x, x, part);
	}
	if (!norm) return;
	double p = block_sum(ds_to_double(part), sh);
	double tot;
	if (last_block_total(p, partials, &st->ticket, &tot, sh)) *Hn = sqrt(tot);
}

// u := u / h in double-single; from_double: u holds FP64 values (read, then
// overwritten in place by their double-single quotients).
__global__ void k_scale_ds(dsf *u, int n, const double *h, int from_double, fg_status *st)
{
	if (!gmres_live(st)) return;
	__shared__ dsf sc;
	if (threadIdx.x == 0) sc = ds_from(1.0 / *h);
	__syncthreads();
	const dsf zero = dsf{ 0.0f, 0.0f };
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		const dsf x = from_double ? ds_from(((const double *)u)[k]) : u[k];
		u[k] = ds_fma(x, sc, zero);
	}
}

// FP64 values to double-single in place (an operator without a double-single
// output).
__global__ void k_to_ds(double *x, int n, const int *active)
{
	if (active && !*active) return;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
		((dsf *)x)[k] = ds_from(x[k]);
}

// Orthogonalisation of the Arnoldi steps of restart cycle `cycle': 0 MGS
// (one fused kernel per basis vector), 1 CGS, 2 CGS with one
// re-orthogonalisation (CGS2), 3 CGS in a solve's first cycle and CGS2 in
// every later one (FEMGPU_GS selects; default 3).  Single-pass CGS is the
// fastest and, within one cycle, converges like MGS on the transport solves
// (8-block ILU(0), FGMRES(80): 56-59 iterations either way); across restarts
// it loses orthogonality (global ILU(0), FGMRES(50) at 2048x1024: 166-216
// iterations against 46-51 for MGS and 45-56 for CGS2).  Re-orthogonalising
// only where the first pass lost more than half of ||w||^2 (the
// Daniel-Gragg-Kaufman-Stewart test) saved nothing: near convergence nearly
// every step fails that test.
static int gs_mode(int cycle)
{
	static int g = -1;
	if (g < 0) {
		const char *e = getenv("FEMGPU_GS");
		int v = e ? atoi(e) : 3;
		g = (v >= 0 && v <= 3) ? v : 3;
	}
	if (g == 3) return cycle == 0 ? 1 : 2;
	return g;
}

// u = u * (1/h), dscal of pgmres.c:85 / :121.
__global__ void k_scale(double *u, int n, const double *h, fg_status *st)
{
	if (!gmres_live(st)) return;
	double sc = 1.0 / *h;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
		u[k] = __dmul_rn(sc, u[k]);
}

// Start of a restart cycle (pgmres.c:77-87): u0 = B - u0, e0 = ||u0||.
// force: run at least one inner iteration (the do-while of pgmres.c:89-163).
__global__ void __launch_bounds__(RED_TPB) k_residual_start(double *u0, const double *B, int n,
                                                            double *ge, double *partials, fg_status *st,
                                                            int force)
{
	__shared__ double sh[32];
	double part = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double r = -__dadd_rn(u0[k], -B[k]);
		u0[k] = r;
		part += r * r;
	}
	part = block_sum(part, sh);
	double tot;
	if (last_block_total(part, partials, &st->ticket, &tot, sh)) {
		ge[0] = sqrt(tot);
		st->rho = ge[0];
		st->inner = 0;
		st->active = (force || st->rho > st->eps) ? 1 : 0;
	}
}

// Givens QR update of column i (pgmres.c:123-163), single thread.
__global__ void k_givens(double *H, int ldh, double *cs, double *sn, double *ge, int i, int kmax,
                         fg_status *st)
{
	if (!gmres_live(st)) return;
	for (int j = 0; j <= i - 1; j++) {
		double hj = H[j * ldh + i], hj1 = H[(j + 1) * ldh + i];
		double h1 = __dadd_rn(__dmul_rn(cs[j], hj), __dmul_rn(sn[j], hj1));
		double h2 = __dadd_rn(__dmul_rn(-sn[j], hj), __dmul_rn(cs[j], hj1));
		H[j * ldh + i] = h1;
		H[(j + 1) * ldh + i] = h2;
	}
	double hii = H[i * ldh + i], hi1 = H[(i + 1) * ldh + i];
	double r = sqrt(__dadd_rn(__dmul_rn(hii, hii), __dmul_rn(hi1, hi1)));
	cs[i] = hii / r;
	sn[i] = hi1 / r;
	H[i * ldh + i] = r;
	H[(i + 1) * ldh + i] = 0.0;
	ge[i + 1] = __dmul_rn(-sn[i], ge[i]);
	ge[i] = __dmul_rn(cs[i], ge[i]);
	double rho = fabs(ge[i + 1]);
	st->rho = rho;
	st->inner = i + 1;
	st->total += 1;
	if (!(rho > st->eps) || i + 1 >= kmax) st->active = 0;
	if (!(rho == rho)) { st->active = 0; fg_set_err(&st->err, FEMGPU_E_BREAKDOWN); }
}

// Back substitution (pgmres.c:165-175), single thread; i = inner - 1.
__global__ void k_backsolve(const double *H, int ldh, const double *ge, double *gy, fg_status *st)
{
	int i = st->inner - 1;
	if (i < 0) return;
	gy[i] = ge[i] / H[i * ldh + i];
	for (int j = i - 1; j >= 0; j--) {
		double soma = 0.0;
		for (int k = j + 1; k <= i; k++) soma = __dadd_rn(soma, __dmul_rn(H[j * ldh + k], gy[k]));
		gy[j] = __dadd_rn(ge[j], -soma) / H[j * ldh + j];
	}
}

// X += sum_j u_j y_j (pgmres.c:177-181), j ascending per entry.
template <typename TV>
__global__ void k_update_x(double *X, const TV *V, size_t ldv, int n, const double *gy, const fg_status *st)
{
	int m = st->inner;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double x = X[k];
		for (int j = 0; j < m; j++) x = __dadd_rn(x, __dmul_rn((double)V[(size_t)j * ldv + k], gy[j]));
		X[k] = x;
	}
}

static int red_grid(femgpu_transport *t) { return t->nblk_red; }

// One restart cycle of pgmres.c:58-184, entirely stream-ordered; the status
// block tells the host afterwards whether to restart.
extern "C" int fg_kry_pgmres_cycle(const fg_krylov *k, const fg_linop *op, const double *B, double *X)
{
	cudaStream_t s = k->stream;
	int n = k->n, kmax = k->kmax, ldh = kmax + 1, G = k->nblk, rc;
	size_t ldv = k->ldv;
	double *V = k->V;
	int *active = &k->st->active;
	// u0 = M^-1 A X  (precondR is the identity in the drivers using pgmres)
	if ((rc = op->matvec(op->ctx, X, V, nullptr))) return rc;
	if (op->precond && (rc = op->precond(op->ctx, V, V, nullptr))) return rc;
	k_residual_start<<<G, RED_TPB, 0, s>>>(V, B, n, k->ge, k->partials, k->st, 1);
	k_scale<<<fg_grid(n), FG_TPB, 0, s>>>(V, n, k->ge, k->st);
	for (int i = 0; i < kmax; i++) {
		double *w = V + (size_t)(i + 1) * ldv;
		if ((rc = op->matvec(op->ctx, V + (size_t)i * ldv, w, active))) return rc;
		if (op->precond && (rc = op->precond(op->ctx, w, w, active))) return rc;
		for (int j = 0; j <= i + 1; j++)
			k_mgs<<<G, RED_TPB, 0, s>>>(V, ldv, n, i, j, k->H, ldh, k->partials, k->st);
		k_scale<<<fg_grid(n), FG_TPB, 0, s>>>(w, n, k->H + (i + 1) * ldh + i, k->st);
		k_givens<<<1, 1, 0, s>>>(k->H, ldh, k->cs, k->sn, k->ge, i, kmax, k->st);
	}
	k_backsolve<<<1, 1, 0, s>>>(k->H, ldh, k->ge, k->gy, k->st);
	k_update_x<double><<<fg_grid(n), FG_TPB, 0, s>>>(X, V, ldv, n, k->gy, k->st);
	return (int)cudaGetLastError();
}

// ------------------------------------------------ look-ahead FGMRES ----
// The step's directions combined with the Gram-Schmidt coefficients of
// column i (read before the Givens rotations overwrite it): t = sum_j H(j,i)
// z_j over m = i + 1 stored directions, and eta = H(i+1,i).  Loads as in
// k_cgs_update.  Dynamic shared memory: the m coefficients.
__global__ void __launch_bounds__(RED_TPB) k_zcombo(const double *Z, size_t ldv, int n, int m, const double *Hcol,
                                                    int ldh, double *t, double *eta, fg_status *st)
{
	if (!gmres_live(st)) return;
	extern __shared__ double hsh[];
	for (int j = threadIdx.x; j < m; j += blockDim.x) hsh[j] = Hcol[(size_t)j * ldh];
	if (blockIdx.x == 0 && threadIdx.x == 0) *eta = Hcol[(size_t)m * ldh];
	__syncthreads();
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double x = 0.0;
		int j = 0;
		for (; j + CGS_UNR <= m; j += CGS_UNR) {
			double v[CGS_UNR];
#pragma unroll
			for (int u = 0; u < CGS_UNR; u++) v[u] = Z[(size_t)(j + u) * ldv + k];
#pragma unroll
			for (int u = 0; u < CGS_UNR; u++) x += hsh[j + u] * v[u];
		}
		for (; j < m; j++) x += hsh[j] * Z[(size_t)j * ldv + k];
		t[k] = x;
	}
}

// z := (z - t) / eta: the next direction from y = M^-1 w (in z) and t.
__global__ void k_la_fin(double *z, const double *t, int n, const double *eta, fg_status *st)
{
	if (!gmres_live(st)) return;
	const double r = 1.0 / *eta;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) z[k] = (z[k] - t[k]) * r;
}

// The same from the preconditioner's double-single output y (natural order).
__global__ void k_la_fin_ds(double *z, const dsf *y, const double *t, int n, const double *eta, fg_status *st)
{
	if (!gmres_live(st)) return;
	const double r = 1.0 / *eta;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		const dsf v = y[k];
		z[k] = (((double)v.hi + (double)v.lo) - t[k]) * r;
	}
}

// The convergence flag as the step starts, for the work on the look-ahead
// stream: a copy that no later kernel changes, so every thread of a sweep
// reads the same value while the Givens kernel of the step may clear the
// flag itself concurrently.
__global__ void k_la_snap(const fg_status *st, int *flag) { *flag = st->active; }

// Dynamic shared memory the Gram-Schmidt kernels of a look-ahead step ask
// for: more than an SM holding an ILU sweep CTA (about 215 KB of its 228 KB)
// has left, so the FP64-heavy blocks run on the other SMs and do not take
// issue slots from the latency-bound sweep.
#ifndef LA_SMEM
#define LA_SMEM (24 * 1024)
#endif

// Look-ahead flexible GMRES cycle.  With w = A z_i and v_(i+1) =
// (w - V h) / eta, linearity of M^-1 gives M^-1 v_(i+1) = (y - Z h) / eta
// for y = M^-1 w and Z = [M^-1 v_0 .. M^-1 v_i].  So y is computed on la_s
// from the raw operator output while the step's Gram-Schmidt runs on the main
// stream (block ILU(0)'s sweeps hold one SM per matrix block, the multi-dot
// and the update the others), t = Z h follows the coefficients, and the step
// then waits only for y and forms z_(i+1) = (y - t) / eta.  The z_i equal
// M^-1 v_i up to rounding; the Arnoldi relation A Z = V H holds for the
// stored z_i whatever their rounding, and, as every FGMRES solve here, the
// solve is accepted on the true residual.
static int fgmres_cycle_la(const fg_krylov *k, const fg_linop *op, const double *B, double *X, int cycle)
{
	cudaStream_t s = k->stream, s2 = k->la_s;
	int n = k->n, kmax = k->kmax, ldh = kmax + 1, G = k->nblk, rc;
	size_t ldv = k->ldv;
	double *V = k->V, *Z = k->Z;
	int *active = &k->st->active;
	const int cgs_grid = G * (CGS_GRID < kmax + 1 ? CGS_GRID : kmax + 1);
	const int gs = gs_mode(cycle);
	// the product writes the preconditioner's gathered input itself
	const bool fused = op->matvec_g && op->precond_g && op->precond_g_out;
	if ((rc = op->matvec(op->ctx, X, V, nullptr))) return rc;
	k_residual_start<<<G, RED_TPB, 0, s>>>(V, B, n, k->ge, k->partials, k->st, 0);
	k_scale<<<fg_grid(n), FG_TPB, 0, s>>>(V, n, k->ge, k->st);
	if ((rc = op->precond(op->ctx, V, Z, active))) return rc;
	for (int i = 0; i < kmax; i++) {
		const int m = i + 1, more = i + 1 < kmax;
		const size_t hs = sizeof(double) * (size_t)m > LA_SMEM ? sizeof(double) * (size_t)m : LA_SMEM;
		double *w = V + (size_t)(i + 1) * ldv, *znext = Z + (size_t)(i + 1) * ldv;
		double *h = k->partials + (size_t)G * (kmax + 1);
		if (fused) rc = op->matvec_g(op->ctx, Z + (size_t)i * ldv, k->la_w, active);
		else rc = op->matvec(op->ctx, Z + (size_t)i * ldv, k->la_w, active);
		if (rc) return rc;
		if (more) {
			k_la_snap<<<1, 1, 0, s>>>(k->st, k->la_flag + i);
			FG_TRY(cudaEventRecord(k->la_ev_w, s));
			FG_TRY(cudaStreamWaitEvent(s2, k->la_ev_w, 0));
			if (fused) rc = op->precond_g(op->ctx, k->la_flag + i, s2);
			else rc = op->precond_s(op->ctx, k->la_w, znext, k->la_flag + i, s2);
			if (rc) return rc;
			FG_TRY(cudaEventRecord(k->la_ev_y, s2));
		}
		for (int pass = 0; pass < gs; pass++) {
			const int last = pass == gs - 1;
			const double *win = pass == 0 ? k->la_w : w;
			k_mdot<<<dim3(G, (m + MD_J - 1) / MD_J), RED_TPB, LA_SMEM, s>>>(V, ldv, n, m, win, k->partials, k->st);
			k_mdot_fin<<<m, 32, 0, s>>>(k->partials, G, m, h, k->H + i, ldh, pass, k->st);
			k_cgs_update<<<cgs_grid, RED_TPB, hs, s>>>(V, ldv, n, m, win, w, h, last, k->H + (i + 1) * ldh + i,
			                                           k->partials, k->st);
		}
		if (more) k_zcombo<<<cgs_grid, RED_TPB, hs, s>>>(Z, ldv, n, m, k->H + i, ldh, k->la_t, k->la_eta, k->st);
		k_scale<<<fg_grid(n), FG_TPB, 0, s>>>(w, n, k->H + (i + 1) * ldh + i, k->st);
		k_givens<<<1, 1, 0, s>>>(k->H, ldh, k->cs, k->sn, k->ge, i, kmax, k->st);
		if (more) {
			FG_TRY(cudaStreamWaitEvent(s, k->la_ev_y, 0));
			if (fused)
				k_la_fin_ds<<<fg_grid(n), FG_TPB, 0, s>>>(znext, (const dsf *)op->precond_g_out(op->ctx), k->la_t, n,
				                                         k->la_eta, k->st);
			else k_la_fin<<<fg_grid(n), FG_TPB, 0, s>>>(znext, k->la_t, n, k->la_eta, k->st);
		}
	}
	k_backsolve<<<1, 1, 0, s>>>(k->H, ldh, k->ge, k->gy, k->st);
	k_update_x<double><<<fg_grid(n), FG_TPB, 0, s>>>(X, Z, ldv, n, k->gy, k->st);
	return (int)cudaGetLastError();
}

// One restart cycle of flexible GMRES with right preconditioning:
// r0 = B - A X, z_i = M^-1 v_i, w = A z_i, MGS, Givens; X += Z y.  The
// Arnoldi residual is the unpreconditioned one.  mixed: 0 FP64 throughout,
// 1 FP32 preconditioner (FP64 operator), 2 FP32 preconditioner and operator.
extern "C" int fg_kry_fgmres_cycle(const fg_krylov *k, const fg_linop *op, const double *B, double *X,
                                   int mixed, int cycle)
{
	cudaStream_t s = k->stream;
	int n = k->n, kmax = k->kmax, ldh = kmax + 1, G = k->nblk, rc;
	size_t ldv = k->ldv;
	double *V = k->V;
	int *active = &k->st->active;
	// the double-single basis (FP64 arithmetic otherwise: the residual, the
	// Hessenberg matrix, the Givens rotations, Z and X stay FP64)
	const bool dsv = k->dsv && !mixed && op->precond_dsin && op->matvec_dsout;
	if (!mixed && !dsv && k->la_s && op->precond_s && k->Z && gs_mode(cycle) != 0)
		return fgmres_cycle_la(k, op, B, X, cycle);
	// the update's grid: its norm partials must stay below the coefficients,
	// which the multi-dot finish stores at partials + G (kmax + 1)
	const int cgs_grid = G * (CGS_GRID < kmax + 1 ? CGS_GRID : kmax + 1);
	if (mixed && (!op->precond32 || !op->matvec_xf || !k->Z32)) return FEMGPU_E_ARG;
	if (!mixed && !k->Z) return FEMGPU_E_ARG;
	if ((rc = op->matvec(op->ctx, X, V, nullptr))) return rc;
	k_residual_start<<<G, RED_TPB, 0, s>>>(V, B, n, k->ge, k->partials, k->st, 0);
	if (dsv) k_scale_ds<<<fg_grid(n), FG_TPB, 0, s>>>((dsf *)V, n, k->ge, 1, k->st);
	else k_scale<<<fg_grid(n), FG_TPB, 0, s>>>(V, n, k->ge, k->st);
	for (int i = 0; i < kmax; i++) {
		double *v = V + (size_t)i * ldv, *w = V + (size_t)(i + 1) * ldv;
		if (mixed) {
			float *z = k->Z32 + (size_t)i * ldv;
			if ((rc = op->precond32(op->ctx, v, z, active))) return rc;
			if ((rc = op->matvec_xf(op->ctx, z, w, active, mixed == 2))) return rc;
		} else if (dsv) {
			double *z = k->Z + (size_t)i * ldv;
			if ((rc = op->precond_dsin(op->ctx, v, z, active))) return rc;
			if ((rc = op->matvec_dsout(op->ctx, z, w, active))) return rc;
		} else {
			double *z = k->Z + (size_t)i * ldv;
			if (op->precond) {
				if ((rc = op->precond(op->ctx, v, z, active))) return rc;
			} else {
				FG_TRY(cudaMemcpyAsync(z, v, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
			}
			if ((rc = op->matvec(op->ctx, z, w, active))) return rc;
		}
		int gs = gs_mode(cycle);
		if (dsv && gs == 0) gs = 1;                        // MGS has no double-single form
		if (dsv) {
			const int m = i + 1;
			double *h = k->partials + (size_t)G * (kmax + 1);
			for (int pass = 0; pass < gs; pass++) {
				const int last = pass == gs - 1;
				k_mdot_ds<<<dim3(G, (m + MD_J - 1) / MD_J), RED_TPB, 0, s>>>((const dsf *)V, ldv, n, m, (const dsf *)w,
				                                                           k->partials, k->st);
				k_mdot_fin<<<m, 32, 0, s>>>(k->partials, G, m, h, k->H + i, ldh, pass, k->st);
				k_cgs_update_ds<<<cgs_grid, RED_TPB, sizeof(dsf) * (size_t)m, s>>>((const dsf *)V, ldv, n, m, (dsf *)w, h, last,
				                                                         k->H + (i + 1) * ldh + i, k->partials,
				                                                         k->st);
			}
			k_scale_ds<<<fg_grid(n), FG_TPB, 0, s>>>((dsf *)w, n, k->H + (i + 1) * ldh + i, 0, k->st);
			k_givens<<<1, 1, 0, s>>>(k->H, ldh, k->cs, k->sn, k->ge, i, kmax, k->st);
			continue;
		}
		if (gs == 0) {
			for (int j = 0; j <= i + 1; j++)
				k_mgs<<<G, RED_TPB, 0, s>>>(V, ldv, n, i, j, k->H, ldh, k->partials, k->st);
		} else {
			const int m = i + 1;
			double *h = k->partials + (size_t)G * (kmax + 1);
			for (int pass = 0; pass < gs; pass++) {
				const int last = pass == gs - 1;
				k_mdot<<<dim3(G, (m + MD_J - 1) / MD_J), RED_TPB, 0, s>>>(V, ldv, n, m, w, k->partials, k->st);
				k_mdot_fin<<<m, 32, 0, s>>>(k->partials, G, m, h, k->H + i, ldh, pass, k->st);
				k_cgs_update<<<cgs_grid, RED_TPB, sizeof(double) * (size_t)m, s>>>(V, ldv, n, m, w, w, h, last,
				                                                                     k->H + (i + 1) * ldh + i,
				                                                                     k->partials, k->st);
			}
		}
		k_scale<<<fg_grid(n), FG_TPB, 0, s>>>(w, n, k->H + (i + 1) * ldh + i, k->st);
		k_givens<<<1, 1, 0, s>>>(k->H, ldh, k->cs, k->sn, k->ge, i, kmax, k->st);
	}
	k_backsolve<<<1, 1, 0, s>>>(k->H, ldh, k->ge, k->gy, k->st);
	if (mixed) k_update_x<float><<<fg_grid(n), FG_TPB, 0, s>>>(X, k->Z32, ldv, n, k->gy, k->st);
	else k_update_x<double><<<fg_grid(n), FG_TPB, 0, s>>>(X, k->Z, ldv, n, k->gy, k->st);
	return (int)cudaGetLastError();
}

// st->rho = ||B - q|| for q = A X (the last cycle's state is left alone).
__global__ void __launch_bounds__(RED_TPB) k_true_rho(const double *q, const double *B, int n, double *partials,
                                                      fg_status *st)
{
	__shared__ double sh[32];
	double part = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double r = -__dadd_rn(q[k], -B[k]);
		part += r * r;
	}
	part = block_sum(part, sh);
	double tot;
	if (last_block_total(part, partials, &st->ticket, &tot, sh)) st->rho = sqrt(tot);
}

// True residual of the current iterate into st->rho; A X goes to V[kmax],
// which holds no Arnoldi vector of a finished cycle.
extern "C" int fg_kry_true_rho(const fg_krylov *k, const fg_linop *op, const double *B, double *X)
{
	int rc;
	double *q = k->V + (size_t)k->kmax * k->ldv;
	if ((rc = op->matvec(op->ctx, X, q, nullptr))) return rc;
	k_true_rho<<<k->nblk, RED_TPB, 0, k->stream>>>(q, B, k->n, k->partials, k->st);
	return (int)cudaGetLastError();
}

// ------------------------------------------- the transport context's view
// The Krylov operator: FGMRES contexts with CSR storage apply the fused
// product (their sweeps are the fused ones too); the reference's GMRES keeps
// csrmv.c's rounding.
static int tr_matvec(void *c, const double *p, double *q, const int *a)
{
	femgpu_transport *t = (femgpu_transport *)c;
	if (t->o.solver == FEMGPU_FGMRES && t->o.scheme == FEMGPU_CSR) {
		if (t->sell_A) return fg_sellmv(t, p, q, 1, 0, a);
		return fg_csrmv64_fused(t->neq, t->IA, t->JA, t->A, p, q, a, t->stream);
	}
	return fg_matvec(t, p, q, a);
}
static int tr_precond(void *c, const double *p, double *z, const int *a)
{
	return fg_precond((femgpu_transport *)c, p, z, a);
}
// The Krylov operator on its own (timing, tests).
extern "C" int fg_operator(femgpu_transport *t, const double *p, double *q)
{
	return tr_matvec(t, p, q, nullptr);
}

extern "C" int fg_ilu0_apply64_dsin(femgpu_transport *t, const void *p, double *z, const int *active);
extern "C" int fg_ilu0_ds_ready(const femgpu_transport *t);
static int tr_precond_dsin(void *c, const void *p, double *z, const int *a)
{
	return fg_ilu0_apply64_dsin((femgpu_transport *)c, p, z, a);
}
static int tr_matvec_dsout(void *c, const double *p, void *q, const int *a)
{
	femgpu_transport *t = (femgpu_transport *)c;
	if (t->o.scheme == FEMGPU_CSR) {
		if (t->sell_A) return fg_sellmv(t, p, q, 1, 1, a);
		return fg_csrmv64_fused_ds(t->neq, t->IA, t->JA, t->A, p, q, a, t->stream);
	}
	int rc = fg_matvec(t, p, (double *)q, a);
	if (rc) return rc;
	k_to_ds<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>((double *)q, t->neq, a);
	return (int)cudaGetLastError();
}

// The double-single basis for FP64 FGMRES with the double-single ILU(0)
// sweeps, on request (FEMGPU_KRYLOV_DS=1): measured at 2048x1024 its
// multi-dot and update kernels take about twice as long as the FP64 ones
// (those are bound by memory latency, not by the FP64 pipe, and a
// double-single product-sum costs a dozen FP32 instructions), so the FP64
// basis is the default.
static int krylov_ds(const femgpu_transport *t)
{
	static int env = -1;
	if (env < 0) {
		const char *e = getenv("FEMGPU_KRYLOV_DS");
		env = (e && e[0] == '1') ? 1 : 0;
	}
	return env && t->o.solver == FEMGPU_FGMRES && t->o.precision == FEMGPU_FP64 &&
	       t->o.precond == FEMGPU_PREC_ILU0 && fg_ilu0_ds_ready(t);
}
// The preconditioner on another stream (the look-ahead step): the ILU(0)
// apply launches everything on the context's stream, which is swapped for
// the call.
static int tr_precond_s(void *c, const double *p, double *z, const int *a, cudaStream_t s)
{
	femgpu_transport *t = (femgpu_transport *)c;
	cudaStream_t keep = t->stream;
	t->stream = s;
	int rc = fg_precond(t, p, z, a);
	t->stream = keep;
	return rc;
}

static int tr_matvec_g(void *c, const double *p, double *q, const int *a)
{
	return sellmv_gather((femgpu_transport *)c, p, q, a);
}
static int tr_precond_g(void *c, const int *a, cudaStream_t s)
{
	femgpu_transport *t = (femgpu_transport *)c;
	cudaStream_t keep = t->stream;
	t->stream = s;
	int rc = fg_ilu0_sweeps_gathered(t, a);
	t->stream = keep;
	return rc;
}
static const void *tr_precond_g_out(void *c) { return ((femgpu_transport *)c)->sweeps.o64; }

// FGMRES with the look-ahead step (fgmres_cycle_la): FP64 block or global
// ILU(p) contexts, unless FEMGPU_LOOKAHEAD=0 (read at every cycle).  Its stream (the highest
// priority, so the sweep CTAs are placed before the Gram-Schmidt blocks
// that become ready with them), events and vectors are made on first use;
// without them the plain cycle runs.
static int lookahead_on(femgpu_transport *t)
{
	const char *e = getenv("FEMGPU_LOOKAHEAD");
	if ((e && e[0] == '0') || t->o.solver != FEMGPU_FGMRES || t->o.precision != FEMGPU_FP64 ||
	    t->o.precond != FEMGPU_PREC_ILU0 || !t->Z)
		return 0;
	if (!t->la_s) {
		int lo = 0, hi = 0;
		cudaStream_t st = nullptr;
		if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
		    cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, hi) != cudaSuccess) {
			cudaGetLastError();
			return 0;
		}
		if (cudaEventCreateWithFlags(&t->la_ev[0], cudaEventDisableTiming) != cudaSuccess ||
		    cudaEventCreateWithFlags(&t->la_ev[1], cudaEventDisableTiming) != cudaSuccess ||
		    cudaMalloc((void **)&t->la_buf, sizeof(double) * (2 * t->ldv + 1)) != cudaSuccess ||
		    cudaMalloc((void **)&t->la_flag, sizeof(int) * ((size_t)t->kmax + 1)) != cudaSuccess) {
			cudaGetLastError();
			cudaStreamDestroy(st);
			return 0;
		}
		t->la_s = st;
	}
	return 1;
}

static int tr_precond32(void *c, const double *p, float *z, const int *a)
{
	return fg_precond32((femgpu_transport *)c, p, z, a);
}
static int tr_matvec_xf(void *c, const float *p, double *q, const int *a, int op32)
{
	return matvec_xf((femgpu_transport *)c, p, q, a, op32);
}

extern "C" void fg_transport_krylov(femgpu_transport *t, fg_krylov *k, fg_linop *op)
{
	k->n = t->neq; k->kmax = t->kmax; k->nblk = red_grid(t); k->ldv = t->ldv; k->stream = t->stream;
	k->V = t->V; k->H = t->H; k->cs = t->cs; k->sn = t->sn; k->ge = t->ge; k->gy = t->gy;
	k->Z = t->Z; k->Z32 = t->Z32; k->partials = t->partials; k->st = t->st; k->st_host = t->st_host;
	op->ctx = t;
	op->matvec = tr_matvec;
	op->precond = tr_precond;
	op->precond32 = tr_precond32;
	op->matvec_xf = tr_matvec_xf;
	op->precond_dsin = tr_precond_dsin;
	op->matvec_dsout = tr_matvec_dsout;
	op->precond_s = tr_precond_s;
	op->matvec_g = nullptr;
	op->precond_g = nullptr;
	op->precond_g_out = nullptr;
	k->dsv = krylov_ds(t);
	k->la_s = nullptr;
	if (!k->dsv && lookahead_on(t)) {
		k->la_s = t->la_s;
		k->la_ev_w = t->la_ev[0];
		k->la_ev_y = t->la_ev[1];
		k->la_w = t->la_buf;
		k->la_t = t->la_buf + t->ldv;
		k->la_eta = t->la_buf + 2 * t->ldv;
		k->la_flag = t->la_flag;
		// the gather fused into the product: CSR over the SELL copy with the
		// double-single sweeps (FEMGPU_LA_GATHER=0: the separate gather)
		const char *e = getenv("FEMGPU_LA_GATHER");
		if (t->o.scheme == FEMGPU_CSR && t->sell_A && t->sweeps.ds && t->sweeps.dpos && !(e && e[0] == '0')) {
			op->matvec_g = tr_matvec_g;
			op->precond_g = tr_precond_g;
			op->precond_g_out = tr_precond_g_out;
		}
	}
}

extern "C" int fg_gmres_cycle(femgpu_transport *t, const double *B, double *X, int first)
{
	fg_krylov k;
	fg_linop op;
	(void)first;
	fg_transport_krylov(t, &k, &op);
	return fg_kry_pgmres_cycle(&k, &op, B, X);
}

extern "C" int fg_fgmres_cycle(femgpu_transport *t, const double *B, double *X, int mixed)
{
	fg_krylov k;
	fg_linop op;
	fg_transport_krylov(t, &k, &op);
	return fg_kry_fgmres_cycle(&k, &op, B, X, mixed, 0);
}

// out = a . b (deterministic), device scalar.
__global__ void __launch_bounds__(RED_TPB) k_dot(const double *a, const double *b, int n,
                                                 double *partials, unsigned *ticket, double *out)
{
	__shared__ double sh[32];
	double part = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
		part += a[k] * b[k];
	part = block_sum(part, sh);
	double tot;
	if (last_block_total(part, partials, ticket, &tot, sh)) *out = tot;
}

extern "C" int fg_kry_dot(const fg_krylov *k, const double *a, const double *b, int n, double *out_dev)
{
	k_dot<<<k->nblk, RED_TPB, 0, k->stream>>>(a, b, n, k->partials, &k->st->ticket, out_dev);
	return (int)cudaGetLastError();
}

extern "C" int fg_dot(femgpu_transport *t, const double *a, const double *b, int n, double *out_dev)
{
	k_dot<<<red_grid(t), RED_TPB, 0, t->stream>>>(a, b, n, t->partials, &t->st->ticket, out_dev);
	return (int)cudaGetLastError();
}

__global__ void __launch_bounds__(RED_TPB) k_resid2(const double *B, const double *Q, int n,
                                                    double *partials, unsigned *ticket, double *out)
{
	__shared__ double sh[32];
	double part = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		double r = B[k] - Q[k];
		part += r * r;
	}
	part = block_sum(part, sh);
	double tot;
	if (last_block_total(part, partials, ticket, &tot, sh)) *out = tot;
}

// max_k |a[k] - b[k]| (the Picard stop test, Process.c:325-328).
__global__ void __launch_bounds__(RED_TPB) k_maxabsdiff(const double *a, const double *b, int n,
                                                        double *partials, unsigned *ticket, double *out)
{
	__shared__ double sh[32];
	__shared__ bool last;
	double m = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
		m = fmax(m, fabs(a[k] - b[k]));
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmax(m, sh[w]);
		partials[blockIdx.x] = m;
		__threadfence();
		last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
	}
	__syncthreads();
	if (last && threadIdx.x == 0) {
		double r = 0.0;
		for (int q = 0; q < (int)gridDim.x; q++) r = fmax(r, __ldcg(&partials[q]));
		*out = r;
		*ticket = 0u;
	}
}

extern "C" int fg_maxabsdiff(femgpu_transport *t, const double *a, const double *b, int n, double *out_dev)
{
	k_maxabsdiff<<<red_grid(t), RED_TPB, 0, t->stream>>>(a, b, n, t->partials, &t->st->ticket, out_dev);
	return (int)cudaGetLastError();
}

// ||B - A X||^2 -> out_dev (A X goes to the scratch vector w2).
extern "C" int fg_residual_norm(femgpu_transport *t, const double *B, const double *X, double *out_dev)
{
	int rc = fg_matvec(t, X, t->w2, nullptr);
	if (rc) return rc;
	k_resid2<<<red_grid(t), RED_TPB, 0, t->stream>>>(B, t->w2, t->neq, t->partials, &t->st->ticket,
	                                                 out_dev);
	return (int)cudaGetLastError();
}

// r = B - A u (FP64), for iterative refinement.
__global__ void k_sub(const double *B, const double *Q, double *r, int n)
{
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) r[k] = B[k] - Q[k];
}

extern "C" int fg_axpy_resid(femgpu_transport *t, const double *B, double *r)
{
	int rc = fg_matvec(t, t->u, t->w2, nullptr);
	if (rc) return rc;
	k_sub<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(B, t->w2, r, t->neq);
	return (int)cudaGetLastError();
}

__global__ void k_add(double *x, const double *d, int n)
{
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) x[k] += d[k];
}

extern "C" int fg_add(double *x, const double *d, int n, cudaStream_t s)
{
	k_add<<<fg_grid(n), FG_TPB, 0, s>>>(x, d, n);
	return (int)cudaGetLastError();
}

__global__ void k_to_f32(const double *a, float *b, long long n)
{
	for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
		b[k] = (float)a[k];
}

extern "C" int fg_to_f32(const double *a, float *b, long long n, cudaStream_t s)
{
	k_to_f32<<<fg_grid(n), FG_TPB, 0, s>>>(a, b, n);
	return (int)cudaGetLastError();
}
