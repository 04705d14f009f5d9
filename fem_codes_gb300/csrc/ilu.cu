// ILU(0) on the device (ILUp_precond_setup.c:66-167 at level of fill 0,
// ILUp_precond.c:26-46).
//
// The triangular sweeps have ~2.5*nx dependency levels after SYMRCM (5118
// for a 2048x1024 grid) of a few hundred rows each, so they are bound by
// per-level latency, not bandwidth.  They run in ONE thread block:
//   * at set-up, each sweep is compiled into a "program": for every level a
//     16-byte aligned block holding the level's rows in ELL layout --
//     dependency codes, factor values (refreshed after every factorisation),
//     output slots and, for the backward sweep, inverted pivots;
//   * the block streams level programs (and the level's slice of the input
//     vector) into shared memory with TMA bulk copies (cp.async.bulk +
//     mbarrier) several levels ahead;
//   * solution values of the most recent levels live in a shared-memory ring
//     indexed by level-order position; older dependencies are read back from
//     global memory (written by the same block, ordered by __syncthreads);
//   * one __syncthreads per level.
// Rows are computed in the reference's order (ascending columns) and the
// FP64 variant rounds each operation separately, so its results are
// bit-identical to the reference's sweeps.  Every mbarrier wait is bounded:
// on timeout the block records FEMGPU_E_TIMEOUT, waits (bounded) for the
// copies it has in flight and returns.
#include "fg_common.cuh"
#include <string.h>
#include <vector>
#include <algorithm>

#define SW_THREADS 1024
#define SW_RING 4096                  // ring slots (power of two)
#define SW_NEAR 0x80000000u           // dependency code: ring slot
#define SW_WAIT_LIMIT (1 << 24)
#define SW_BAR_BYTES 64               // up to 8 mbarriers
#define SW_SMEM_CAP (220 * 1024)

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
	return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
	             :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
	             :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
	unsigned ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
	             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	             "selp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
	return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
	for (int i = 0; i < SW_WAIT_LIMIT; i++)
		if (mbar_try_wait(bar, parity)) return true;
	return false;
}

__device__ __forceinline__ void fence_proxy_async()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

template <typename T> __device__ __forceinline__ T fms(T x, T a, T b);   // x - a*b
template <> __device__ __forceinline__ double fms(double x, double a, double b)
{
	return __dsub_rn(x, __dmul_rn(a, b));
}
template <> __device__ __forceinline__ float fms(float x, float a, float b) { return x - a * b; }
template <typename T> __device__ __forceinline__ T mul(T a, T b);
template <> __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul(float a, float b) { return a * b; }

// Level block: header, dep[w*cp] (int), out[cp] (int), pad to 16,
// val[w*cp] (T), and for the backward sweep dinv[cp] (T).
struct LevHdr { int c, w, start, cp; };

static inline __host__ __device__ long long al16(long long x) { return (x + 15) & ~15LL; }

struct SweepArgs {
	const unsigned char *prog;
	const long long *blk_off;     // [nlev+1]
	const int *lev_pstart;        // [nlev+1] padded start of each level in the input vector
	int nlev, D, stage_bytes;
	int *err;
	const int *active;
};

// Issue the copies of level l into stage s (thread 0 only).
template <typename T>
__device__ __forceinline__ void issue_level(const SweepArgs &a, const T *in, unsigned char *stages,
                                            unsigned long long *bar, int l, int s)
{
	unsigned char *dst = stages + (size_t)s * a.stage_bytes;
	long long b0 = a.blk_off[l];
	unsigned bb = (unsigned)(a.blk_off[l + 1] - b0);
	int p0 = a.lev_pstart[l];
	unsigned vb = (unsigned)al16((long long)(a.lev_pstart[l + 1] - p0) * (long long)sizeof(T));
	mbar_expect_tx(&bar[s], bb + vb);
	bulk_g2s(dst, a.prog + b0, bb, &bar[s]);
	if (vb) bulk_g2s(dst + bb, in + p0, vb, &bar[s]);
}

template <typename T, bool UPPER>
__global__ void __launch_bounds__(SW_THREADS, 1)
k_sweep(SweepArgs a, const T *__restrict__ in, T *out)
{
	if (a.active && !*a.active) return;
	extern __shared__ __align__(128) unsigned char sm[];
	const size_t ring_b = al16((SW_RING + 1) * sizeof(T));
	T *ring = (T *)sm;
	unsigned long long *bar = (unsigned long long *)(sm + ring_b);
	unsigned char *stages = sm + ((ring_b + SW_BAR_BYTES + 127) & ~(size_t)127);
	__shared__ int failed;
	const int tid = threadIdx.x, D = a.D;

	if (tid == 0) {
		failed = 0;
		ring[SW_RING] = T(0);
		for (int s = 0; s < D; s++) mbar_init(&bar[s], 1);
		fence_mbar_init();
		fence_proxy_async();
		for (int l = 0; l < D && l < a.nlev; l++) issue_level<T>(a, in, stages, bar, l, l);
	}
	__syncthreads();
	int l = 0;
	for (; l < a.nlev; l++) {
		const int s = l % D;
		if (!mbar_wait(&bar[s], (unsigned)((l / D) & 1))) failed = 1;
		__syncthreads();
		if (failed) break;
		const unsigned char *st = stages + (size_t)s * a.stage_bytes;
		const LevHdr h = *(const LevHdr *)st;
		const int *dep = (const int *)(st + 16);
		const int *outp = dep + h.w * h.cp;
		const T *val = (const T *)(st + al16(16 + (long long)(h.w + 1) * h.cp * 4));
		const T *dinv = val + h.w * h.cp;
		const T *bv = (const T *)(st + (a.blk_off[l + 1] - a.blk_off[l]));
		for (int r = tid; r < h.c; r += SW_THREADS) {
			T x = bv[r];
			for (int k = 0; k < h.w; k++) {
				unsigned d = (unsigned)dep[k * h.cp + r];
				T xd = (d & SW_NEAR) ? ring[d & ~SW_NEAR] : __ldcg(&out[d]);
				x = fms(x, xd, val[k * h.cp + r]);
			}
			if (UPPER) x = mul(x, dinv[r]);
			ring[(h.start + r) & (SW_RING - 1)] = x;
			out[outp[r]] = x;
		}
		__syncthreads();
		if (tid == 0 && l + D < a.nlev) {
			fence_proxy_async();
			issue_level<T>(a, in, stages, bar, l + D, s);
		}
	}
	if (failed && tid == 0) {
		fg_set_err(a.err, FEMGPU_E_TIMEOUT);
		// copies in flight: levels l .. l+D-1 (bounded waits)
		for (int q = l; q < l + D && q < a.nlev; q++) (void)mbar_wait(&bar[q % D], (unsigned)((q / D) & 1));
	}
}

// Gather the sweep input into padded level order: in[ppos[i]] = (T) p[rows[i]].
template <typename T, typename TI>
__global__ void k_perm_in(const TI *__restrict__ p, const int *__restrict__ rows,
                          const int *__restrict__ ppos, int n, T *in)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		in[ppos[i]] = (T)p[rows[i]];
}

// Refresh the value slots of a program from the factor (after every factorisation).
template <typename T>
__global__ void k_refresh(unsigned char *prog, const long long *val_off, const int *val_src, long long nval,
                          const double *LU, const double *Dinv)
{
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nval;
	     i += (long long)gridDim.x * blockDim.x) {
		int s = val_src[i];
		double v = (s >= 0) ? LU[s] : (s == -1 ? 0.0 : Dinv[-2 - s]);
		*(T *)(prog + val_off[i]) = (T)v;
	}
}

// ---------------------------------------------------------- factor ------
// IKJ ILU(0) in level order in one block: rows of a level in parallel, one
// __syncthreads per level; U parts and pivots of earlier levels were written
// by this block before a barrier, so plain loads see them.
#define FAC_CAP 32
__global__ void __launch_bounds__(SW_THREADS, 1)
k_ilu0_factor_cta(const int *__restrict__ IA, const int *__restrict__ JA, const double *__restrict__ AA,
                  const int *__restrict__ rows, const int *__restrict__ lev_start, int nlev,
                  double *LU, double *Dinv, int *err)
{
	for (int l = 0; l < nlev; l++) {
		int b = lev_start[l], e = lev_start[l + 1];
		for (int q0 = b + threadIdx.x; q0 < e; q0 += SW_THREADS) {
			int r = rows[q0];
			int rb = IA[r], len = IA[r + 1] - rb;
			if (len > FAC_CAP) { fg_set_err(err, FEMGPU_E_MESH); continue; }
			int cols[FAC_CAP];
			double vals[FAC_CAP];
			int dpos = -1;
			for (int q = 0; q < len; q++) {
				cols[q] = JA[rb + q];
				vals[q] = AA[rb + q];
				if (cols[q] == r) dpos = q;
			}
			double d = (dpos >= 0) ? vals[dpos] : 0.0;
			for (int q = 0; q < len && cols[q] < r; q++) {
				int jrow = cols[q];
				vals[q] = __dmul_rn(vals[q], Dinv[jrow]);
				int kb = IA[jrow], ke = IA[jrow + 1];
				for (int k = kb; k < ke; k++) {
					int col = JA[k];
					if (col <= jrow) continue;
					int pos = -1;
					for (int m = 0; m < len; m++) if (cols[m] == col) { pos = m; break; }
					if (pos < 0) continue;
					double prod = __dmul_rn(vals[q], LU[k]);
					if (col == r) d = __dsub_rn(d, prod);
					else vals[pos] = __dsub_rn(vals[pos], prod);
				}
			}
			for (int q = 0; q < len; q++) LU[rb + q] = (q == dpos) ? d : vals[q];
			if (d == 0.0) { fg_set_err(err, FEMGPU_E_ZERO_PIVOT); Dinv[r] = 0.0; }
			else Dinv[r] = 1.0 / d;
		}
		__syncthreads();
	}
}

// ------------------------------------------------------- host: programs
struct HostLevels {
	int nlev;
	std::vector<int> start, pstart, rows, pos, ppos;   // pos/ppos indexed by row
};

static HostLevels host_levels(const int *IA, const int *JA, int n, bool lower)
{
	HostLevels H;
	std::vector<int> lev(n, 0);
	int nlev = 0;
	if (lower) {
		for (int i = 0; i < n; i++) {
			int L = 0;
			for (int k = IA[i]; k < IA[i + 1] && JA[k] < i; k++) L = std::max(L, lev[JA[k]] + 1);
			lev[i] = L; nlev = std::max(nlev, L + 1);
		}
	} else {
		for (int i = n - 1; i >= 0; i--) {
			int L = 0;
			for (int k = IA[i]; k < IA[i + 1]; k++) if (JA[k] > i) L = std::max(L, lev[JA[k]] + 1);
			lev[i] = L; nlev = std::max(nlev, L + 1);
		}
	}
	H.nlev = nlev;
	H.start.assign(nlev + 1, 0);
	H.pstart.assign(nlev + 1, 0);
	for (int i = 0; i < n; i++) H.start[lev[i] + 1]++;
	for (int l = 0; l < nlev; l++) {
		int c = H.start[l + 1];
		H.start[l + 1] += H.start[l];
		H.pstart[l + 1] = H.pstart[l] + ((c + 3) & ~3);      // 16-byte aligned level slices
	}
	std::vector<int> fill(H.start.begin(), H.start.end() - 1);
	H.rows.assign(n, 0);
	H.pos.assign(n, 0);
	H.ppos.assign(n, 0);
	for (int i = 0; i < n; i++) {
		int p = fill[lev[i]]++;
		H.rows[p] = i;
		H.pos[i] = p;
		H.ppos[i] = H.pstart[lev[i]] + (p - H.start[lev[i]]);
	}
	return H;
}

template <typename X>
static int up_vec(X **d, const std::vector<X> &h)
{
	FG_TRY(cudaMalloc((void **)d, sizeof(X) * (h.size() + 1)));
	if (!h.empty()) FG_TRY(cudaMemcpy(*d, h.data(), sizeof(X) * h.size(), cudaMemcpyHostToDevice));
	return 0;
}

// One sweep program.  Forward (lower): L part, outputs to the backward
// sweep's padded level order (target = the U levels' ppos).  Backward: U part
// and pivots, outputs in natural order.
static int build_prog(const int *IA, const int *JA, int n, const HostLevels &H, bool lower,
                      const HostLevels *target, size_t tsize, fg_sweep &sw)
{
	int nlev = H.nlev;
	std::vector<long long> off(nlev + 1, 0);
	std::vector<int> width(nlev, 0);
	long long maxblk = 0;
	for (int l = 0; l < nlev; l++) {
		int c = H.start[l + 1] - H.start[l], w = 0;
		for (int p = H.start[l]; p < H.start[l + 1]; p++) {
			int r = H.rows[p], cnt = 0;
			for (int k = IA[r]; k < IA[r + 1]; k++) if (lower ? JA[k] < r : JA[k] > r) cnt++;
			w = std::max(w, cnt);
		}
		width[l] = w;
		int cp = (c + 3) & ~3;
		long long sz = al16(16 + (long long)(w + 1) * cp * 4) + (long long)w * cp * (long long)tsize
		               + (lower ? 0 : (long long)cp * (long long)tsize);
		off[l + 1] = off[l] + al16(sz);
		maxblk = std::max(maxblk, al16(sz) + al16((long long)cp * (long long)tsize));
	}
	std::vector<unsigned char> prog((size_t)off[nlev] + 16, 0);
	std::vector<long long> val_off;
	std::vector<int> val_src;
	val_off.reserve((size_t)IA[n] + n);
	val_src.reserve((size_t)IA[n] + n);
	for (int l = 0; l < nlev; l++) {
		int c = H.start[l + 1] - H.start[l], w = width[l], cp = (c + 3) & ~3, start = H.start[l];
		int end = H.start[l + 1];
		unsigned char *b = prog.data() + off[l];
		LevHdr h = { c, w, start, cp };
		memcpy(b, &h, sizeof h);
		int *dep = (int *)(b + 16), *outp = dep + (size_t)w * cp;
		long long voff = al16(16 + (long long)(w + 1) * cp * 4);
		for (int k = 0; k < w * cp; k++) dep[k] = (int)(SW_NEAR | SW_RING);       // the zero slot
		for (int j = 0; j < c; j++) {
			int r = H.rows[start + j], k = 0;
			outp[j] = lower ? target->ppos[r] : r;
			for (int q = IA[r]; q < IA[r + 1]; q++) {
				int col = JA[q];
				if (lower ? !(col < r) : !(col > r)) continue;
				int p = H.pos[col];
				unsigned code = (end - p <= SW_RING) ? (SW_NEAR | (unsigned)(p & (SW_RING - 1)))
				                                     : (unsigned)(lower ? target->ppos[col] : col);
				dep[(size_t)k * cp + j] = (int)code;
				val_off.push_back(off[l] + voff + ((long long)k * cp + j) * (long long)tsize);
				val_src.push_back(q);
				k++;
			}
			for (; k < w; k++) {
				val_off.push_back(off[l] + voff + ((long long)k * cp + j) * (long long)tsize);
				val_src.push_back(-1);
			}
			if (!lower) {
				val_off.push_back(off[l] + voff + ((long long)w * cp + j) * (long long)tsize);
				val_src.push_back(-2 - r);
			}
		}
	}
	sw.nlev = nlev;
	sw.bytes = off[nlev];
	sw.maxblk = maxblk;
	sw.nval = (long long)val_off.size();
	sw.npad = H.pstart[nlev];
	int rc;
	FG_TRY(cudaMalloc((void **)&sw.prog, prog.size()));
	FG_TRY(cudaMemcpy(sw.prog, prog.data(), prog.size(), cudaMemcpyHostToDevice));
	if ((rc = up_vec(&sw.blk_off, off))) return rc;
	if ((rc = up_vec(&sw.lev_start, H.start))) return rc;
	if ((rc = up_vec(&sw.lev_pstart, H.pstart))) return rc;
	if ((rc = up_vec(&sw.rows, H.rows))) return rc;
	std::vector<int> ppos_by_pos(n);
	for (int p = 0; p < n; p++) ppos_by_pos[p] = H.ppos[H.rows[p]];
	if ((rc = up_vec(&sw.ppos, ppos_by_pos))) return rc;
	if ((rc = up_vec(&sw.val_off, val_off))) return rc;
	if ((rc = up_vec(&sw.val_src, val_src))) return rc;
	return 0;
}

static int sweep_smem(const fg_sweep &sw, size_t tsize, int *D, int *stage_bytes)
{
	size_t fixed = ((al16((SW_RING + 1) * tsize) + SW_BAR_BYTES + 127) & ~(size_t)127);
	size_t sb = (size_t)((sw.maxblk + 127) & ~127LL);
	if (fixed + 2 * sb > SW_SMEM_CAP) return FEMGPU_E_MESH;   // a level too wide to stage
	int d = (int)((SW_SMEM_CAP - fixed) / sb);
	if (d > 6) d = 6;
	*D = d;
	*stage_bytes = (int)sb;
	return (int)(fixed + (size_t)d * sb);
}

extern "C" int fg_ilu_prepare(femgpu_transport *t, const int *hIA, const int *hJA)
{
	int n = t->neq, rc, D, sb;
	fg_ilu_sweeps &S = t->sweeps;
	HostLevels Lo = host_levels(hIA, hJA, n, true), Up = host_levels(hIA, hJA, n, false);
	if ((rc = build_prog(hIA, hJA, n, Up, false, nullptr, sizeof(double), S.up64))) return rc;
	if ((rc = build_prog(hIA, hJA, n, Lo, true, &Up, sizeof(double), S.lo64))) return rc;
	if ((rc = build_prog(hIA, hJA, n, Up, false, nullptr, sizeof(float), S.up32))) return rc;
	if ((rc = build_prog(hIA, hJA, n, Lo, true, &Up, sizeof(float), S.lo32))) return rc;
	size_t nb = (size_t)std::max(Lo.pstart[Lo.nlev], Up.pstart[Up.nlev]) + 64;
	FG_TRY(cudaMalloc((void **)&S.bl64, sizeof(double) * nb));
	FG_TRY(cudaMalloc((void **)&S.y64, sizeof(double) * nb));
	FG_TRY(cudaMalloc((void **)&S.bl32, sizeof(float) * nb));
	FG_TRY(cudaMalloc((void **)&S.y32, sizeof(float) * nb));
	FG_TRY(cudaMemset(S.bl64, 0, sizeof(double) * nb));
	FG_TRY(cudaMemset(S.y64, 0, sizeof(double) * nb));
	FG_TRY(cudaMemset(S.bl32, 0, sizeof(float) * nb));
	FG_TRY(cudaMemset(S.y32, 0, sizeof(float) * nb));
	const fg_sweep *all[4] = { &S.lo64, &S.up64, &S.lo32, &S.up32 };
	for (int i = 0; i < 4; i++) {
		rc = sweep_smem(*all[i], i < 2 ? sizeof(double) : sizeof(float), &D, &sb);
		if (rc < 0) return rc;
	}
	FG_TRY(cudaFuncSetAttribute(k_sweep<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP));
	FG_TRY(cudaFuncSetAttribute(k_sweep<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP));
	FG_TRY(cudaFuncSetAttribute(k_sweep<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP));
	FG_TRY(cudaFuncSetAttribute(k_sweep<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP));
	return 0;
}

extern "C" int fg_ilu0_factor(femgpu_transport *t)
{
	cudaStream_t s = t->stream;
	fg_ilu_sweeps &S = t->sweeps;
	k_ilu0_factor_cta<<<1, SW_THREADS, 0, s>>>(t->IA, t->JA, t->A, S.lo64.rows, S.lo64.lev_start, S.lo64.nlev,
	                                           t->ilu.LU, t->ilu.Dinv, &t->st->err);
	fg_sweep *pr[4] = { &S.lo64, &S.up64, &S.lo32, &S.up32 };
	for (int i = 0; i < 4; i++) {
		int g = fg_grid(pr[i]->nval);
		if (i < 2) k_refresh<double><<<g, FG_TPB, 0, s>>>(pr[i]->prog, pr[i]->val_off, pr[i]->val_src,
		                                                 pr[i]->nval, t->ilu.LU, t->ilu.Dinv);
		else k_refresh<float><<<g, FG_TPB, 0, s>>>(pr[i]->prog, pr[i]->val_off, pr[i]->val_src,
		                                          pr[i]->nval, t->ilu.LU, t->ilu.Dinv);
	}
	return (int)cudaGetLastError();
}

template <typename T, typename TI, typename TO>
static int apply_t(femgpu_transport *t, const fg_sweep &lo, const fg_sweep &up, T *bl, T *y,
                   const TI *p, TO *z, const int *active)
{
	cudaStream_t s = t->stream;
	int n = t->neq, D, sb, bytes;
	k_perm_in<T, TI><<<fg_grid(n), FG_TPB, 0, s>>>(p, lo.rows, lo.ppos, n, bl);
	SweepArgs a;
	a.err = &t->st->err;
	a.active = active;
	bytes = sweep_smem(lo, sizeof(T), &D, &sb);
	if (bytes < 0) return bytes;
	a.prog = lo.prog; a.blk_off = lo.blk_off; a.lev_pstart = lo.lev_pstart; a.nlev = lo.nlev;
	a.D = D; a.stage_bytes = sb;
	k_sweep<T, false><<<1, SW_THREADS, bytes, s>>>(a, bl, y);
	bytes = sweep_smem(up, sizeof(T), &D, &sb);
	if (bytes < 0) return bytes;
	a.prog = up.prog; a.blk_off = up.blk_off; a.lev_pstart = up.lev_pstart; a.nlev = up.nlev;
	a.D = D; a.stage_bytes = sb;
	k_sweep<T, true><<<1, SW_THREADS, bytes, s>>>(a, y, (T *)z);
	return (int)cudaGetLastError();
}

extern "C" int fg_ilu0_apply64(femgpu_transport *t, const double *p, double *z, const int *active)
{
	fg_ilu_sweeps &S = t->sweeps;
	return apply_t<double, double, double>(t, S.lo64, S.up64, S.bl64, S.y64, p, z, active);
}

extern "C" int fg_ilu0_apply32(femgpu_transport *t, const double *p, float *z, const int *active)
{
	fg_ilu_sweeps &S = t->sweeps;
	return apply_t<float, double, float>(t, S.lo32, S.up32, S.bl32, S.y32, p, z, active);
}

extern "C" void fg_ilu_free(femgpu_transport *t)
{
	fg_ilu_sweeps &S = t->sweeps;
	fg_sweep *all[4] = { &S.lo64, &S.up64, &S.lo32, &S.up32 };
	for (int i = 0; i < 4; i++) {
		void *p[] = { all[i]->prog, all[i]->blk_off, all[i]->lev_start, all[i]->lev_pstart, all[i]->rows,
		              all[i]->ppos, all[i]->val_off, all[i]->val_src };
		for (void *q : p) if (q) cudaFree(q);
	}
	void *v[] = { S.bl64, S.y64, S.bl32, S.y32 };
	for (void *q : v) if (q) cudaFree(q);
}
