// ILU(0) on the device (ILUp_precond_setup.c:66-167 at level of fill 0,
// ILUp_precond.c:26-46).
//
// The triangular sweeps have ~2.5*nx dependency levels after SYMRCM (5118
// for a 2048x1024 grid) of a few hundred rows each, so they are bound by
// per-level latency, not bandwidth.  Each matrix block is swept by ONE
// thread block:
//   * at set-up, each sweep is compiled into a "program": every level is cut
//     into sub-blocks of at most SW_SUB rows, 16-byte aligned -- one record
//     per row (dependency codes, output slot, factor values, the inverted
//     pivot backward; k_sweep_rec / k_sweep_df) when no row has more than 16
//     dependencies, else ELL arrays (k_sweep); factor values are refreshed
//     after every factorisation;
//   * one producer warp streams sub-blocks (and their slice of the input
//     vector) into a ring of shared-memory stages with TMA bulk copies
//     (cp.async.bulk, completion on a "full" mbarrier; stage reuse gated by an
//     "empty" mbarrier the consumer warps arrive on);
//   * consumer warps compute a level, publish its values in a shared-memory
//     ring indexed by level-order position (older dependencies are re-read
//     from global memory) and synchronise either with one named barrier per
//     level (k_sweep, k_sweep_rec) or through per-warp progress flags that a
//     warp waits on only for the warps it reads from (k_sweep_df, the
//     default for records).
// Rows are computed in the reference's order (ascending columns) and the
// FP64 variant rounds each operation separately, so its results are
// bit-identical to the reference's sweeps; FGMRES uses the fused
// multiply-subtract variant.
//
// Block ILU(0) (ilu_blocks = P > 1): the rows are cut into P contiguous runs
// of the (reordered) numbering (make_blocks: by default at equal spans of the
// full factor's dependency levels) and couplings between runs are dropped, so
// each block factorises and sweeps independently: its levels form a
// contiguous run of the program (levels are numbered block by block) and one
// thread block per matrix block runs them, P thread blocks at once.  The
// factorisation runs one thread-block cluster per matrix block.  Every wait is
// bounded: on timeout the block records FEMGPU_E_TIMEOUT, waits (bounded) for
// the copies it has in flight and returns.
#include "fg_common.cuh"
#include <string.h>
#include <vector>
#include <algorithm>

#ifndef FG_SW2_CW
#define FG_SW2_CW 16
#endif
#define SW_SUB (FG_SW2_CW * 32)       // max rows of a sub-block
#define SW_MAXW 8                     // dependencies per row on the unrolled path
#define SW_RPT 4                      // rows per consumer thread per pass
#define FAC_THREADS 1024
#define SW_RING 4096                  // ring slots (power of two)
#define SW_NEAR 0x80000000u           // dependency code: ring slot
#define SW_WAIT_LIMIT (1 << 24)
#define SW_MAXD 12                    // max stages
#define SW_BAR_BYTES (2 * SW_MAXD * 8)
#define SW_SMEM_CAP (220 * 1024)
#define SW_HDR 32

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

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(bar)) : "memory");
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

// Wait for a phase, giving up when the bound is hit or another warp failed.
__device__ __forceinline__ bool mbar_wait_or_fail(unsigned long long *bar, unsigned parity, volatile int *failed)
{
	for (int i = 0; i < SW_WAIT_LIMIT; i++) {
		if (mbar_try_wait(bar, parity)) return true;
		if (*failed) return false;
	}
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

// Release store / acquire load of a shared-memory flag (CTA scope).
__device__ __forceinline__ void st_release_cta(int *p, int v)
{
	asm volatile("st.release.cta.shared.s32 [%0], %1;" :: "r"(smem_u32(p)), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_acquire_cta(const int *p)
{
	int v;
	asm volatile("ld.acquire.cta.shared.s32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
	return v;
}

// Synchronise the CW consumer warps (shared-memory ordering included).
template <int CW>
__device__ __forceinline__ void consumer_sync()
{
	if (CW == 1) __syncwarp();
	else asm volatile("bar.sync 1, %0;" :: "r"(CW * 32) : "memory");
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

// x - a*b: separately rounded (bit-identical to the reference) or fused.
template <typename T, bool FMA> __device__ __forceinline__ T fmsub(T x, T a, T b)
{
	if (FMA) return fma(-a, b, x);
	return fms(x, a, b);
}

// ---------------------------------------------------- double-single values
// (fg_ds.cuh): the sweeps' values, multipliers and ring in float pairs.
#include "fg_ds.cuh"

template <> __device__ __forceinline__ dsf fmsub<dsf, true>(dsf x, dsf a, dsf b) { return ds_fma(ds_neg(a), b, x); }
template <> __device__ __forceinline__ dsf mul(dsf a, dsf b) { return ds_fma(a, b, dsf{ 0.0f, 0.0f }); }

// zero, FP64 -> T, and the cache-global load / warp shuffle of a T
template <typename T> __device__ __forceinline__ T zero_t() { return T(0); }
template <> __device__ __forceinline__ dsf zero_t<dsf>() { return dsf{ 0.0f, 0.0f }; }
template <typename T> __device__ __forceinline__ T from_d(double v) { return (T)v; }
template <> __device__ __forceinline__ dsf from_d<dsf>(double v) { return ds_from(v); }
template <typename T> __device__ __forceinline__ T ld_cg(const T *p) { return __ldcg(p); }
template <> __device__ __forceinline__ dsf ld_cg<dsf>(const dsf *p)
{
	const float2 v = __ldcg((const float2 *)p);
	return dsf{ v.x, v.y };
}
template <typename T> __device__ __forceinline__ T shfl_up_t(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
template <> __device__ __forceinline__ dsf shfl_up_t<dsf>(dsf v, int d)
{
	return dsf{ __shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d) };
}

// Sub-block: 32-byte header, dep[w*cp] (int), out[cp] (int), pad to 16,
// val[w*cp] (T), and for the backward sweep dinv[cp] (T); the stage then
// holds the sub-block's slice of the input vector.  Header: rows c, ELL
// width w, level-order position of the first row, padded rows cp, number of
// sub-blocks of the level, a flag set when some dependency is older than the
// ring holds (read from global memory instead), and the byte offsets of the
// values and of the input slice.
struct LevHdr { int c, w, start, cp, nsub, hasfar, voff, boff; };

static inline __host__ __device__ long long al16(long long x) { return (x + 15) & ~15LL; }

template <typename T, bool UPPER>
__host__ __device__ __forceinline__ long long blk_bytes(int w, int cp)
{
	long long voff = al16(SW_HDR + (long long)(w + 1) * cp * 4);
	return al16(voff + (long long)w * cp * (long long)sizeof(T) + (UPPER ? (long long)cp * sizeof(T) : 0));
}

struct SweepArgs {
	const unsigned char *prog;
	const long long *blk_off;     // [nsb+1] byte offset of each sub-block
	const int *sb_in;             // [nsb] padded start of the sub-block's input slice
	const int *sb_inb;            // [nsb] bytes of that slice
	int nlev, nsb, D, stage_bytes;
	int *err;
	const int *active;
	const int *chunk_sb;          // [P+1] first sub-block of each matrix block (NULL: one block)
	const int *chunk_lev;         // [P+1] first level of each matrix block
	int bvo, cmax;                // record layout: input slice offset, most rows of a sub-block
	int skew;                     // dataflow: levels a warp may run ahead of the slowest one
	int wait;                     // spins of a warp waiting for the rows it depends on
};

// The producer warp of every sweep kernel: streams this thread block's
// sub-blocks [sb0, sb1) and their input slices into the D-stage ring with
// cp.async.bulk (completion on full[s]), reusing a stage once the consumers
// have released it (empty[s]); stops when a consumer has failed.  The input
// slice lands at the stage's fixed offset a.bvo (record layouts,
// slice_at_bvo) or right after the sub-block (ELL layout).
template <typename T>
__device__ __forceinline__ void sweep_producer(const SweepArgs &a, const T *in, unsigned char *stages,
                                               unsigned sbytes, unsigned long long *full,
                                               unsigned long long *empty, int D, int sb0, int sb1, int lane,
                                               volatile int *vfailed, int *issued, int *pdone, bool slice_at_bvo)
{
	bool stop = false;
	int s = 0;
	unsigned ph = 0;                                      // phase of empty[s] to wait for
	for (int base = sb0; base < sb1 && !stop; base += 32) {
		// each lane fetches the offsets of one upcoming sub-block
		int i = base + lane;
		long long b0 = 0, b1 = 0;
		int p0 = 0, vb = 0;
		if (i < sb1) { b0 = a.blk_off[i]; b1 = a.blk_off[i + 1]; p0 = a.sb_in[i]; vb = a.sb_inb[i]; }
		for (int j = 0; j < 32 && base + j < sb1; j++) {
			long long B0 = __shfl_sync(0xffffffffu, b0, j), B1 = __shfl_sync(0xffffffffu, b1, j);
			int P0 = __shfl_sync(0xffffffffu, p0, j), VB = __shfl_sync(0xffffffffu, vb, j);
			int sb = base + j - sb0;                      // local sub-block index
			int go = 1;
			if (lane == 0) {
				if (sb >= D && !mbar_wait_or_fail(&empty[s], ph, vfailed)) go = 0;
				if (*vfailed) go = 0;
				if (go) {
					unsigned bb = (unsigned)(B1 - B0);
					unsigned char *dst = stages + (unsigned)s * sbytes;
					fence_proxy_async();
					mbar_expect_tx(&full[s], bb + (unsigned)VB);
					bulk_g2s(dst, a.prog + B0, bb, &full[s]);
					if (VB) bulk_g2s(dst + (slice_at_bvo ? (unsigned)a.bvo : bb), in + P0, (unsigned)VB, &full[s]);
					*(volatile int *)issued = sb + 1;
				}
			}
			go = __shfl_sync(0xffffffffu, go, 0);
			if (!go) { stop = true; break; }
			if (++s == D) { s = 0; if (sb >= D) ph ^= 1u; else if (sb == D - 1) ph = 0; }
		}
	}
	if (lane == 0) {
		__threadfence_block();                            // `issued' is final before `pdone'
		*(volatile int *)pdone = 1;
	}
}

// After a consumer failed (one thread): record the timeout, let the producer
// stop, then wait (bounded) for the copies it issued beyond the `done' stages
// this thread consumed, so no copy lands in shared memory after the exit.
__device__ __forceinline__ void sweep_drain(const SweepArgs &a, unsigned long long *full, int D, int done,
                                            int *issued, int *pdone)
{
	fg_set_err(a.err, FEMGPU_E_TIMEOUT);
	for (int i = 0; i < SW_WAIT_LIMIT && !*(volatile int *)pdone; i++) __nanosleep(64);
	__threadfence_block();
	int last = *(volatile int *)issued;
	for (int q = done; q < last; q++) (void)mbar_wait(&full[q % D], (unsigned)((q / D) & 1));
}

// CW consumer warps (warps 0..CW-1) and one producer warp (warp CW).
template <typename T, bool UPPER, int CW, bool FMA>
__global__ void __launch_bounds__((CW + 1) * 32, 1)
k_sweep(SweepArgs a, const T *__restrict__ in, T *out)
{
	if (a.active && !*a.active) return;
	extern __shared__ __align__(128) unsigned char sm[];
	const unsigned ring_b = (unsigned)al16((SW_RING + 1) * sizeof(T));
	T *ring = (T *)sm;
	unsigned long long *full = (unsigned long long *)(sm + ring_b);
	unsigned long long *empty = full + SW_MAXD;
	unsigned char *stages = sm + ((ring_b + SW_BAR_BYTES + 127) & ~127u);
	__shared__ int failed, issued, pdone;
	volatile int *vfailed = &failed;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, D = a.D;
	const unsigned sbytes = (unsigned)a.stage_bytes;
	// this thread block's run of sub-blocks and levels
	const int sb0 = a.chunk_sb ? a.chunk_sb[blockIdx.x] : 0, sb1 = a.chunk_sb ? a.chunk_sb[blockIdx.x + 1] : a.nsb;
	const int l0 = a.chunk_lev ? a.chunk_lev[blockIdx.x] : 0, l1 = a.chunk_lev ? a.chunk_lev[blockIdx.x + 1] : a.nlev;

	if (tid == 0) {
		failed = 0; issued = 0; pdone = 0;
		ring[SW_RING] = T(0);
		for (int s = 0; s < D; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
		fence_mbar_init();
	}
	__syncthreads();

	if (warp == CW) {                                     // ---- producer warp
		sweep_producer(a, in, stages, sbytes, full, empty, D, sb0, sb1, lane, vfailed, &issued, &pdone, false);
		return;
	}

	const int ctid = tid;                                 // ---- consumer warps
	int sb = 0, s = 0;
	unsigned ph = 0;                                      // phase of full[s] to wait for
	for (int l = l0; l < l1; l++) {
		int nsub = 1, j = 0, s0 = s;
		for (; j < nsub; j++) {
			bool ok = mbar_wait_or_fail(&full[s], ph, vfailed);
			if (!ok) { *vfailed = 1; break; }
			const unsigned char *st = stages + (unsigned)s * sbytes;
			const LevHdr h = *(const LevHdr *)st;
			if (j == 0) nsub = h.nsub;
			const int *dep = (const int *)(st + SW_HDR);
			const int *outp = dep + h.w * h.cp;
			const T *val = (const T *)(st + h.voff);
			const T *dinv = val + h.w * h.cp;
			const T *bv = (const T *)(st + h.boff);
			if (!h.hasfar) {
				// every dependency is in the ring
				for (int r = ctid; r < h.c; r += CW * 32) {
					T x = bv[r];
					for (int k = 0; k < h.w; k++)
						x = fmsub<T, FMA>(x, ring[(unsigned)dep[k * h.cp + r] & ~SW_NEAR], val[k * h.cp + r]);
					if (UPPER) x = mul(x, dinv[r]);
					ring[(h.start + r) & (SW_RING - 1)] = x;
					out[outp[r]] = x;
				}
			} else {
				for (int r = ctid; r < h.c; r += CW * 32) {
					T x = bv[r];
					for (int k = 0; k < h.w; k++) {
						unsigned d = (unsigned)dep[k * h.cp + r];
						T xd = (d & SW_NEAR) ? ring[d & ~SW_NEAR] : __ldcg(&out[d]);
						x = fmsub<T, FMA>(x, xd, val[k * h.cp + r]);
					}
					if (UPPER) x = mul(x, dinv[r]);
					ring[(h.start + r) & (SW_RING - 1)] = x;
					out[outp[r]] = x;
				}
			}
			if (++s == D) { s = 0; ph ^= 1u; }
		}
		consumer_sync<CW>();
		// every consumer is done with the level's stages: release them
		if (ctid == 0) {
			int q = s0;
			for (int c = 0; c < j; c++) { mbar_arrive(&empty[q]); if (++q == D) q = 0; }
		}
		sb += j;
		if (*vfailed) break;
	}
	if (*vfailed && ctid == 0) sweep_drain(a, full, D, sb, &issued, &pdone);
}

// ------------------------------------------------ record layout (fixed width)
// When every row of a sweep has at most 16 dependencies, each sub-block is a
// 16-byte header {rows, sub-blocks of the level, level-order position of the
// first row, far flag} followed by one record per row: W dependency codes and
// the output slot (ints, padded to 16 bytes), then W factor values and, in
// the backward sweep, the inverted pivot (padded to 16 bytes).  Rows with
// fewer dependencies are padded with the zero ring slot and a zero value,
// after their real terms, so the order of the real operations is unchanged.
// A record is an odd number of 16-byte words (a quarter warp's 16-byte loads
// then fall in distinct banks), and the input slice sits at the same offset
// of every stage: a consumer thread issues all loads of its row before the
// header arrives, which shortens the per-level chain of dependent loads.
__host__ __device__ constexpr int rec_ib(int w) { return ((w + 1) * 4 + 15) & ~15; }
__host__ __device__ constexpr int rec_vb(int w, bool upper, int ts) { return ((w + (upper ? 1 : 0)) * ts + 15) & ~15; }
__host__ __device__ constexpr int rec_bytes(int w, bool upper, int ts)
{
	return (((rec_ib(w) + rec_vb(w, upper, ts)) / 16) & 1) ? rec_ib(w) + rec_vb(w, upper, ts)
	                                                        : rec_ib(w) + rec_vb(w, upper, ts) + 16;
}
#define SW2_CW FG_SW2_CW              // consumer warps of the record-layout sweep (SW_SUB rows)
#define NEED_STRIDE (((SW2_CW) + 15) / 16 * 16)   // bytes of a warp's need table

template <typename T, bool UPPER, bool FMA, int W>
__global__ void __launch_bounds__((SW2_CW + 1) * 32, 1)
k_sweep_rec(SweepArgs a, const T *__restrict__ in, T *out)
{
	constexpr int CW = SW2_CW;
	constexpr int IB = rec_ib(W), VB = rec_vb(W, UPPER, (int)sizeof(T)), RB = rec_bytes(W, UPPER, (int)sizeof(T));
	static_assert(SW_SUB == CW * 32, "one row per consumer thread and sub-block");
	if (a.active && !*a.active) return;
	extern __shared__ __align__(128) unsigned char sm[];
	const unsigned ring_b = (unsigned)al16((SW_RING + 1) * sizeof(T));
	T *ring = (T *)sm;
	unsigned long long *full = (unsigned long long *)(sm + ring_b);
	unsigned long long *empty = full + SW_MAXD;
	unsigned char *stages = sm + ((ring_b + SW_BAR_BYTES + 127) & ~127u);
	__shared__ int failed, issued, pdone;
	volatile int *vfailed = &failed;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, D = a.D;
	const unsigned sbytes = (unsigned)a.stage_bytes;
	const int sb0 = a.chunk_sb ? a.chunk_sb[blockIdx.x] : 0, sb1 = a.chunk_sb ? a.chunk_sb[blockIdx.x + 1] : a.nsb;
	const int l0 = a.chunk_lev ? a.chunk_lev[blockIdx.x] : 0, l1 = a.chunk_lev ? a.chunk_lev[blockIdx.x + 1] : a.nlev;

	if (tid == 0) {
		failed = 0; issued = 0; pdone = 0;
		ring[SW_RING] = T(0);
		for (int s = 0; s < D; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
		fence_mbar_init();
	}
	__syncthreads();

	if (warp == CW) {                                     // ---- producer warp
		sweep_producer(a, in, stages, sbytes, full, empty, D, sb0, sb1, lane, vfailed, &issued, &pdone, true);
		return;
	}

	const int ctid = tid;                                 // ---- consumer warps
	// the record this thread reads in every stage (clamped into the staged rows;
	// rows past a sub-block's count are read but not used)
	const unsigned roff = 16u + (unsigned)(ctid < a.cmax ? ctid : a.cmax - 1) * RB;
	const unsigned boff = (unsigned)a.bvo + (unsigned)(ctid < a.cmax ? ctid : a.cmax - 1) * sizeof(T);
	int sb = 0, s = 0;
	unsigned ph = 0;
	for (int l = l0; l < l1; l++) {
		int nsub = 1, j = 0, s0 = s;
		for (; j < nsub; j++) {
			bool ok = mbar_wait_or_fail(&full[s], ph, vfailed);
			if (!ok) { *vfailed = 1; break; }
			const unsigned char *st = stages + (unsigned)s * sbytes;
			union { int4 q[IB / 16]; int i[IB / 4]; } ci;
			union { int4 q[VB / 16]; T v[VB / sizeof(T)]; } cv;
#pragma unroll
			for (int q = 0; q < IB / 16; q++) ci.q[q] = ((const int4 *)(st + roff))[q];
#pragma unroll
			for (int q = 0; q < VB / 16; q++) cv.q[q] = ((const int4 *)(st + roff + IB))[q];
			T x = *(const T *)(st + boff);
			const int4 h = *(const int4 *)st;         // rows, sub-blocks, start, far flag
			if (j == 0) nsub = h.y;
			T d[W];
#pragma unroll
			for (int k = 0; k < W; k++) {
				unsigned c = (unsigned)ci.i[k] & ~SW_NEAR;
				d[k] = ring[c < SW_RING ? c : SW_RING];
			}
			if (ctid < h.x) {
				if (h.w) {
#pragma unroll
					for (int k = 0; k < W; k++)
						if (!((unsigned)ci.i[k] & SW_NEAR)) d[k] = __ldcg(&out[ci.i[k]]);
				}
#pragma unroll
				for (int k = 0; k < W; k++) x = fmsub<T, FMA>(x, d[k], cv.v[k]);
				if (UPPER) x = mul(x, cv.v[W]);
				ring[(h.z + ctid) & (SW_RING - 1)] = x;
				out[ci.i[W]] = x;
			}
			if (++s == D) { s = 0; ph ^= 1u; }
		}
		consumer_sync<CW>();
		if (ctid == 0) {
			int q = s0;
			for (int c = 0; c < j; c++) { mbar_arrive(&empty[q]); if (++q == D) q = 0; }
		}
		sb += j;
		if (*vfailed) break;
	}
	if (*vfailed && ctid == 0) sweep_drain(a, full, D, sb, &issued, &pdone);
}

// ------------------------------------------- dataflow sweep (record layout)
// The same records, without a barrier per level: every consumer warp
// publishes the last level it has finished (prog[warp], shared memory) and,
// before computing a sub-block, waits only for the warps whose rows its own
// rows read (a table of 16 bytes per warp in the sub-block header: for each
// producer warp the smallest level distance of a dependency it supplies, 255
// when it supplies none within S + 1 levels) and for every warp to have
// finished level l - S - 1 (S = the program's skew).  The second wait bounds
// how far warps drift apart, so a ring slot is rewritten only after every
// reader of its old value is done: the program reads from the ring only
// dependencies within SW_RING - S * (widest level) positions of their level's
// end.  A warp publishes a level with a release store right after its ring
// writes and only then stores the level's outputs to global memory, so no
// level waits for its own global stores; a dependency read back from global
// memory therefore waits for its producer's next level (whose release covers
// those stores), and the program keeps such dependencies at least two levels
// back.  A warp releases a stage (mbarrier of CW arrivals) as soon as its
// rows are in registers.  Header: {rows, sub-blocks of the level, first
// position, far flag}, then CW need tables of 16 bytes, then the records.
#define DF_HDR (16 + SW2_CW * NEED_STRIDE)

template <typename T, bool UPPER, bool FMA, int W>
__global__ void __launch_bounds__((SW2_CW + 1) * 32, 1)
k_sweep_df(SweepArgs a, const T *__restrict__ in, T *out)
{
	constexpr int CW = SW2_CW;
	constexpr int IB = rec_ib(W), VB = rec_vb(W, UPPER, (int)sizeof(T)), RB = rec_bytes(W, UPPER, (int)sizeof(T));
	static_assert(SW_SUB == CW * 32, "one row per consumer thread and sub-block");
	static_assert(CW <= NEED_STRIDE && CW <= 32, "one need byte per consumer warp in a warp's table");
	if (a.active && !*a.active) return;
	extern __shared__ __align__(128) unsigned char sm[];
	const unsigned ring_b = (unsigned)al16((SW_RING + 1) * sizeof(T));
	T *ring = (T *)sm;
	unsigned long long *full = (unsigned long long *)(sm + ring_b);
	unsigned long long *empty = full + SW_MAXD;
	unsigned char *stages = sm + ((ring_b + SW_BAR_BYTES + 127) & ~127u);
	__shared__ int failed, issued, pdone;
	__shared__ int prog[CW];
	volatile int *vfailed = &failed;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, D = a.D;
	const unsigned sbytes = (unsigned)a.stage_bytes;
	const int sb0 = a.chunk_sb ? a.chunk_sb[blockIdx.x] : 0, sb1 = a.chunk_sb ? a.chunk_sb[blockIdx.x + 1] : a.nsb;
	const int l0 = a.chunk_lev ? a.chunk_lev[blockIdx.x] : 0, l1 = a.chunk_lev ? a.chunk_lev[blockIdx.x + 1] : a.nlev;

	if (tid == 0) {
		failed = 0; issued = 0; pdone = 0;
		ring[SW_RING] = T(0);
		for (int s = 0; s < D; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], CW); }
		fence_mbar_init();
	}
	if (tid < CW) prog[tid] = -1;
	__syncthreads();

	if (warp == CW) {                                     // ---- producer warp
		sweep_producer(a, in, stages, sbytes, full, empty, D, sb0, sb1, lane, vfailed, &issued, &pdone, true);
		return;
	}

	const int ctid = tid;                                 // ---- consumer warps
	const unsigned roff = (unsigned)DF_HDR + (unsigned)(ctid < a.cmax ? ctid : a.cmax - 1) * RB;
	const unsigned boff = (unsigned)a.bvo + (unsigned)(ctid < a.cmax ? ctid : a.cmax - 1) * sizeof(T);
	int s = 0, waited = 0;
	unsigned ph = 0;
	bool fail = false;
	T ydef = T(0);                                        // an output not yet stored to global memory
	int odef = -1;
	for (int l = l0; l < l1 && !fail; l++) {
		const int ll = l - l0;
		int nsub = 1;
		for (int j = 0; j < nsub; j++) {
			if (!mbar_wait_or_fail(&full[s], ph, vfailed)) { *vfailed = 1; fail = true; break; }
			waited++;
			const unsigned char *st = stages + (unsigned)s * sbytes;
			union { int4 q[IB / 16]; int i[IB / 4]; } ci;
			union { int4 q[VB / 16]; T v[VB / sizeof(T)]; } cv;
#pragma unroll
			for (int k = 0; k < IB / 16; k++) ci.q[k] = ((const int4 *)(st + roff))[k];
#pragma unroll
			for (int k = 0; k < VB / 16; k++) cv.q[k] = ((const int4 *)(st + roff + IB))[k];
			const T x0 = *(const T *)(st + boff);
			const int4 h = *(const int4 *)st;
			const int need = lane < CW ? (int)st[16 + warp * NEED_STRIDE + lane] : 255;
			if (j == 0) nsub = h.y;
			__syncwarp();
			if (lane == 0) mbar_arrive(&empty[s]);        // this warp's rows are in registers
			if (++s == D) { s = 0; ph ^= 1u; }
			if (32 * warp >= h.x) continue;               // no rows of this warp here
			// producers of this warp's dependencies, and every warp within the skew
			const int want = ll - (need == 255 ? a.skew + 1 : need);
			bool ready = false;
			for (int it = 0; it < a.wait; it++) {
				const bool mine = lane >= CW || lane == warp || ld_acquire_cta(&prog[lane]) >= want;
				if (__all_sync(0xffffffffu, mine)) { ready = true; break; }
				if (__any_sync(0xffffffffu, *vfailed != 0)) break;
			}
			if (!ready) { *vfailed = 1; fail = true; break; }
			__syncwarp();                                 // the lanes' acquires order every lane's reads
			T d[W];
#pragma unroll
			for (int k = 0; k < W; k++) {
				unsigned c = (unsigned)ci.i[k] & ~SW_NEAR;
				d[k] = ring[c < SW_RING ? c : SW_RING];
			}
			if (ctid < h.x) {
				if (h.w) {
#pragma unroll
					for (int k = 0; k < W; k++)
						if (!((unsigned)ci.i[k] & SW_NEAR)) d[k] = __ldcg(&out[ci.i[k]]);
				}
				T y = x0;
#pragma unroll
				for (int k = 0; k < W; k++) y = fmsub<T, FMA>(y, d[k], cv.v[k]);
				if (UPPER) y = mul(y, cv.v[W]);
				ring[(h.z + ctid) & (SW_RING - 1)] = y;
				if (odef >= 0) out[odef] = ydef;          // an earlier sub-block of this level
				ydef = y;
				odef = ci.i[W];
			}
		}
		if (fail) break;
		__syncwarp();
		if (lane == 0) st_release_cta(&prog[warp], ll);
		if (odef >= 0) { out[odef] = ydef; odef = -1; }
	}
	consumer_sync<CW>();
	if (*vfailed && ctid == 0) sweep_drain(a, full, D, waited, &issued, &pdone);
}

// ------------------------------------------------ chain-scan sweep (records)
// After SYMRCM the rows of a matrix block form fronts, and along a front every
// row depends on its predecessor in the sweep order: y_i = a_i + b_i y_pred,
// with a_i the row's other terms (backward: times the inverted pivot) and b_i
// its coupling to the predecessor -- a first-order linear recurrence.  The
// program groups up to 32 chained rows into a segment, gives segments (not
// rows) dependency levels, and packs each level's segments into 32-slot
// chunks, one per warp (a segment never straddles two chunks; unused slots are
// padding).  A warp computes a_i for its 32 slots from earlier levels, then
// solves its segments' recurrences with a Kogge-Stone scan over the lanes:
// five steps a_t += M_k,t a_{t-2^k}, the multipliers (products of b along the
// segment, zero across a segment start) precompiled from the factor by
// k_chain_mult.  At 2048x1024 with 16 blocks the deepest block falls from
// 1340 row levels to 349 segment levels.  The scan reassociates the
// recurrence, so results agree with the row-by-row sweeps to rounding, not bit
// for bit: it serves the fused-arithmetic (FGMRES) and FP32 sweeps only.
// Records: W dependency codes (the predecessor excluded) and the output slot
// (-1: padding), then W values, the inverted pivot (backward) and M_0..M_4.
// Staging, progress flags, need tables and bounded waits are k_sweep_df's.
__host__ __device__ constexpr int rec_vb_cs(int w, bool upper, int ts) { return ((w + (upper ? 1 : 0) + 5) * ts + 15) & ~15; }
__host__ __device__ constexpr int rec_bytes_cs(int w, bool upper, int ts)
{
	return (((rec_ib(w) + rec_vb_cs(w, upper, ts)) / 16) & 1) ? rec_ib(w) + rec_vb_cs(w, upper, ts)
	                                                           : rec_ib(w) + rec_vb_cs(w, upper, ts) + 16;
}

template <typename T> __device__ __forceinline__ T fma_t(T a, T b, T c);
template <> __device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ dsf fma_t(dsf a, dsf b, dsf c) { return ds_fma(a, b, c); }

// One chain-scan sweep of this thread block's matrix block: the staging,
// dataflow and scan of k_sweep_cs, on the barriers full/empty (D of them);
// every thread returns after a block barrier, true when a wait gave up.
template <typename T, bool UPPER, int W>
__device__ __forceinline__ bool cs_sweep(const SweepArgs &a, const T *__restrict__ in, T *out, unsigned char *sm,
                                         unsigned long long *full, unsigned long long *empty, int *failed,
                                         int *issued, int *pdone, int *prog)
{
	constexpr int CW = SW2_CW;
	constexpr int IB = rec_ib(W), VB = rec_vb_cs(W, UPPER, (int)sizeof(T)), RB = rec_bytes_cs(W, UPPER, (int)sizeof(T));
	constexpr int MO = W + (UPPER ? 1 : 0);              // first scan multiplier
	static_assert(SW_SUB == CW * 32, "one slot per consumer thread and sub-block");
	const unsigned ring_b = (unsigned)al16((SW_RING + 1) * sizeof(T));
	T *ring = (T *)sm;
	unsigned char *stages = sm + ((ring_b + SW_BAR_BYTES + 127) & ~127u);
	volatile int *vfailed = failed;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, D = a.D;
	const unsigned sbytes = (unsigned)a.stage_bytes;
	const int sb0 = a.chunk_sb ? a.chunk_sb[blockIdx.x] : 0, sb1 = a.chunk_sb ? a.chunk_sb[blockIdx.x + 1] : a.nsb;
	const int l0 = a.chunk_lev ? a.chunk_lev[blockIdx.x] : 0, l1 = a.chunk_lev ? a.chunk_lev[blockIdx.x + 1] : a.nlev;

	if (tid == 0) {
		*failed = 0; *issued = 0; *pdone = 0;
		ring[SW_RING] = zero_t<T>();
		for (int s = 0; s < D; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], CW); }
		fence_mbar_init();
	}
	if (tid < CW) prog[tid] = -1;
	__syncthreads();

	if (warp == CW) {                                     // ---- producer warp
		sweep_producer(a, in, stages, sbytes, full, empty, D, sb0, sb1, lane, vfailed, issued, pdone, true);
	} else {                                              // ---- consumer warps
		const int ctid = tid;
		const unsigned roff = (unsigned)DF_HDR + (unsigned)(ctid < a.cmax ? ctid : a.cmax - 1) * RB;
		const unsigned boff = (unsigned)a.bvo + (unsigned)(ctid < a.cmax ? ctid : a.cmax - 1) * sizeof(T);
		int s = 0, waited = 0;
		unsigned ph = 0;
		bool fail = false;
		T ydef = zero_t<T>();                             // an output not yet stored to global memory
		int odef = -1;
		for (int l = l0; l < l1 && !fail; l++) {
			const int ll = l - l0;
			int nsub = 1;
			for (int j = 0; j < nsub; j++) {
				if (!mbar_wait_or_fail(&full[s], ph, vfailed)) { *vfailed = 1; fail = true; break; }
				waited++;
				const unsigned char *st = stages + (unsigned)s * sbytes;
				union { int4 q[IB / 16]; int i[IB / 4]; } ci;
				union { int4 q[VB / 16]; T v[VB / sizeof(T)]; } cv;
#pragma unroll
				for (int k = 0; k < IB / 16; k++) ci.q[k] = ((const int4 *)(st + roff))[k];
#pragma unroll
				for (int k = 0; k < VB / 16; k++) cv.q[k] = ((const int4 *)(st + roff + IB))[k];
				const T x0 = *(const T *)(st + boff);
				const int4 h = *(const int4 *)st;
				const int need = lane < CW ? (int)st[16 + warp * NEED_STRIDE + lane] : 255;
				if (j == 0) nsub = h.y;
				__syncwarp();
				if (lane == 0) mbar_arrive(&empty[s]);    // this warp's slots are in registers
				if (++s == D) { s = 0; ph ^= 1u; }
				if (32 * warp >= h.x) continue;           // no chunk of this warp here (uniform)
				const int want = ll - (need == 255 ? a.skew + 1 : need);
				bool ready = false;
				for (int it = 0; it < a.wait; it++) {
					const bool mine = lane >= CW || lane == warp || ld_acquire_cta(&prog[lane]) >= want;
					if (__all_sync(0xffffffffu, mine)) { ready = true; break; }
					if (__any_sync(0xffffffffu, *vfailed != 0)) break;
				}
				if (!ready) { *vfailed = 1; fail = true; break; }
				__syncwarp();
				T d[W];
#pragma unroll
				for (int k = 0; k < W; k++) {
					unsigned c = (unsigned)ci.i[k] & ~SW_NEAR;
					d[k] = ring[c < SW_RING ? c : SW_RING];
				}
				if (h.w) {
#pragma unroll
					for (int k = 0; k < W; k++)
						if (!((unsigned)ci.i[k] & SW_NEAR)) d[k] = ld_cg(&out[ci.i[k]]);
				}
				T y = x0;
#pragma unroll
				for (int k = 0; k < W; k++) y = fmsub<T, true>(y, d[k], cv.v[k]);
				if (UPPER) y = mul(y, cv.v[W]);
				// the segments' recurrences across the warp's lanes
#pragma unroll
				for (int k = 0; k < 5; k++) {
					const T up = shfl_up_t(y, 1 << k);
					if (lane >= (1 << k)) y = fma_t(cv.v[MO + k], up, y);
				}
				ring[(h.z + ctid) & (SW_RING - 1)] = y;
				if (odef >= 0) out[odef] = ydef;          // an earlier sub-block of this level
				ydef = y;
				odef = ci.i[W];
			}
			if (fail) break;
			__syncwarp();
			if (lane == 0) st_release_cta(&prog[warp], ll);
			if (odef >= 0) { out[odef] = ydef; odef = -1; }
		}
		consumer_sync<CW>();
		if (*vfailed && ctid == 0) sweep_drain(a, full, D, waited, issued, pdone);
	}
	__syncthreads();
	return *vfailed != 0;
}

template <typename T, bool UPPER, int W>
__global__ void __launch_bounds__((SW2_CW + 1) * 32, 1)
k_sweep_cs(SweepArgs a, const T *__restrict__ in, T *out)
{
	if (a.active && !*a.active) return;
	extern __shared__ __align__(128) unsigned char sm[];
	const unsigned ring_b = (unsigned)al16((SW_RING + 1) * sizeof(T));
	unsigned long long *full = (unsigned long long *)(sm + ring_b);
	__shared__ int failed, issued, pdone;
	__shared__ int prog[SW2_CW];
	(void)cs_sweep<T, UPPER, W>(a, in, out, sm, full, full + SW_MAXD, &failed, &issued, &pdone, prog);
}

// Both sweeps of one preconditioner application in one launch: each thread
// block sweeps its matrix block forward (in -> y) and then backward (y ->
// out), keeping its SM between the two (block ILU(0): a block's backward
// sweep reads only its own forward results).  The consumers' global stores
// of y are ordered before the producer's bulk copies of y by an async-proxy
// fence and the block barrier; the backward sweep runs on barriers of its
// own.  Dynamic shared memory: the larger of the two sweeps' layouts.
template <typename T, int WL, int WU>
__global__ void __launch_bounds__((SW2_CW + 1) * 32, 1)
k_sweep_cs_fb(SweepArgs al, SweepArgs au, const T *__restrict__ in, T *y, T *out)
{
	if (al.active && !*al.active) return;
	extern __shared__ __align__(128) unsigned char sm[];
	const unsigned ring_b = (unsigned)al16((SW_RING + 1) * sizeof(T));
	unsigned long long *full = (unsigned long long *)(sm + ring_b);
	__shared__ unsigned long long bar2[2 * SW_MAXD];
	__shared__ int failed, issued, pdone;
	__shared__ int prog[SW2_CW];
	if (cs_sweep<T, false, WL>(al, in, y, sm, full, full + SW_MAXD, &failed, &issued, &pdone, prog)) return;
	asm volatile("fence.proxy.async.global;" ::: "memory");
	__syncthreads();
	(void)cs_sweep<T, true, WU>(au, y, out, sm, bar2, bar2 + SW_MAXD, &failed, &issued, &pdone, prog);
}

// Scan multipliers of a chain-scan program from the factor, one warp per
// 32-slot chunk: b = -L(row, pred) forward, -Dinv[row] U(row, pred) backward
// (0 at a segment start and in padding); M_0 = b and, as the scan composes
// the recurrences, M_{k+1,t} = M_k,t M_k,t-2^k for t >= 2^k (else M_k,t).
template <typename T, bool UPPER>
__global__ void k_chain_mult(unsigned char *prog, const long long *voff, const int *src, const int *row, int nslot,
                             const double *LU, const double *Dinv)
{
	const int lane = threadIdx.x & 31;
	const int w0 = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
	const int nw = (int)((gridDim.x * (unsigned)blockDim.x) >> 5);
	for (int c = w0; c * 32 < nslot; c += nw) {          // uniform per warp
		const int i = c * 32 + lane;
		const int sr = i < nslot ? src[i] : -1;
		double m = 0.0;
		if (sr >= 0) m = UPPER ? -(Dinv[row[i]] * LU[sr]) : -LU[sr];
		double M[5];
		M[0] = m;
#pragma unroll
		for (int k = 0; k < 4; k++) {
			const double up = __shfl_up_sync(0xffffffffu, M[k], 1 << k);
			M[k + 1] = lane >= (1 << k) ? M[k] * up : M[k];
		}
		const long long o = i < nslot ? voff[i] : -1;
		if (o >= 0) {
			T *dst = (T *)(prog + o);
#pragma unroll
			for (int k = 0; k < 5; k++) dst[k] = from_d<T>(M[k]);
		}
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

// The same gather into double-single values, and back from double-single
// (the backward sweep's natural-order output) to FP64.
__global__ void k_perm_in_ds(const double *__restrict__ p, const int *__restrict__ rows,
                             const int *__restrict__ ppos, int n, dsf *in)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		in[ppos[i]] = ds_from(p[rows[i]]);
}

__global__ void k_perm_in_dsds(const dsf *__restrict__ p, const int *__restrict__ rows,
                               const int *__restrict__ ppos, int n, dsf *in, const int *active)
{
	if (active && !*active) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		in[ppos[i]] = p[rows[i]];
}

// dpos[rows[i]] = ppos[i]: where the gather of the double-single apply puts
// natural row r, for a product that writes the gathered input itself.
__global__ void k_inv_gather(const int *__restrict__ rows, const int *__restrict__ ppos, int n, int *dpos)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dpos[rows[i]] = ppos[i];
}

__global__ void k_ds_to_double(const dsf *__restrict__ x, int n, double *z, const int *active)
{
	if (active && !*active) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const dsf v = x[i];
		z[i] = (double)v.hi + (double)v.lo;
	}
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
		*(T *)(prog + val_off[i]) = from_d<T>(v);
	}
}

// ---------------------------------------------------------- factor ------
// IKJ ILU(0) in level order in one block: rows of a level in parallel, one
// __syncthreads per level; U parts and pivots of earlier levels were written
// by this block before a barrier, so plain loads see them.  The elimination
// structure of each row is precompiled (fac_prog): [dpos, ngroups] then per
// lower entry, in ascending column order, [q, jrow, cnt, (dst, src) x cnt]
// -- dst the position in row r updated by U(jrow, src) (-1: the pivot) --
// so a row needs no pattern searches, only independent loads.
#define FAC_CAP 32
__global__ void __launch_bounds__(FAC_THREADS, 1)
k_ilu0_factor_cta(const int *__restrict__ IA, const double *__restrict__ AA,
                  const int *__restrict__ rows, const int *__restrict__ lev_start, int nlev,
                  const int *__restrict__ chunk_lev, const int *__restrict__ fac_ptr,
                  const int *__restrict__ fac_prog, double *LU, double *Dinv, int *err)
{
	const int l0 = chunk_lev ? chunk_lev[blockIdx.x] : 0, l1 = chunk_lev ? chunk_lev[blockIdx.x + 1] : nlev;
	for (int l = l0; l < l1; l++) {
		int b = lev_start[l], e = lev_start[l + 1];
		for (int p = b + threadIdx.x; p < e; p += FAC_THREADS) {
			int r = rows[p];
			int rb = IA[r], len = IA[r + 1] - rb;
			double vals[FAC_CAP];
			for (int q = 0; q < len; q++) vals[q] = AA[rb + q];
			const int *pr = fac_prog + fac_ptr[p];
			int dpos = pr[0], ng = pr[1];
			pr += 2;
			double d = vals[dpos];
			for (int g = 0; g < ng; g++) {
				int q = pr[0], jrow = pr[1], cnt = pr[2];
				pr += 3;
				double lq = __dmul_rn(vals[q], Dinv[jrow]);
				vals[q] = lq;
				for (int c = 0; c < cnt; c++, pr += 2) {
					double prod = __dmul_rn(lq, LU[pr[1]]);
					if (pr[0] < 0) d = __dsub_rn(d, prod);
					else vals[pr[0]] = __dsub_rn(vals[pr[0]], prod);
				}
			}
			for (int q = 0; q < len; q++) LU[rb + q] = (q == dpos) ? d : vals[q];
			if (d == 0.0) { fg_set_err(err, FEMGPU_E_ZERO_PIVOT); Dinv[r] = 0.0; }
			else Dinv[r] = 1.0 / d;
		}
		__syncthreads();
	}
}

// The same factorisation on a thread-block cluster: each level's rows are
// split over the cluster's CTAs (a single SM's FP64 pipe would otherwise
// bound it), with one cluster barrier per level.  A row's loads come in three
// rounds -- its header; its matrix values and elimination program; every
// operand from earlier levels (pivots and U entries, read from L2: other CTAs
// wrote them) -- and the first two do not depend on the factorisation, so
// for each thread's first row of the next level they are issued during the
// current level (header into registers at its start, values and program by
// cp.async into the other half of a double buffer before the barrier).  After
// a barrier only the operand round and the arithmetic remain.  The
// arithmetic is the reference's, in its order.
#define FAC2_T 64                     // threads per CTA
#define FAC2_MAXP 64                  // program ints per row
#define FAC2_MAXOPS 32                // operands per row
#define FAC2_BUF (FAC2_T * ((FAC_CAP + 1) * 8 + FAC2_MAXP * 4))
#define FAC2_SMEM (FAC2_T * FAC2_MAXOPS * 8 + 2 * FAC2_BUF)

__device__ __forceinline__ void cluster_barrier()
{
	asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
	asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank()
{
	unsigned r;
	asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
	return r;
}

__device__ __forceinline__ unsigned cluster_size()
{
	unsigned r;
	asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
	return r;
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" :: "r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__global__ void __launch_bounds__(FAC2_T)
k_ilu0_factor_cluster(const double *__restrict__ AA, const int *__restrict__ rows,
                      const int *__restrict__ lev_start, int nlev, const int *__restrict__ chunk_lev,
                      const int4 *__restrict__ hdr, const int *__restrict__ prog, double *LU, double *Dinv,
                      int *err)
{
	extern __shared__ __align__(16) unsigned char fsm[];
	// per-thread scratch, element i of thread t at [i * FAC2_T + t] (no bank conflicts)
	double *so = (double *)fsm + threadIdx.x;
	unsigned char *bufs = fsm + FAC2_T * FAC2_MAXOPS * 8;
#define SO(i) so[(i) * FAC2_T]
#define SV(B, i) ((double *)(bufs + (B) * FAC2_BUF))[(i) * FAC2_T + threadIdx.x]
#define SP(B, i) ((int *)(bufs + (B) * FAC2_BUF + FAC2_T * (FAC_CAP + 1) * 8))[(i) * FAC2_T + threadIdx.x]
	const int C = (int)cluster_size(), rank = (int)cluster_rank(), tid = (int)threadIdx.x;
	// block ILU(0): cluster k factorises matrix block k (its run of levels)
	const int ck = (int)(blockIdx.x / (unsigned)C);
	const int L0 = chunk_lev ? chunk_lev[ck] : 0, L1 = chunk_lev ? chunk_lev[ck + 1] : nlev;
	// level bounds: [b, e) this level, e1 the next level's end, e2 the one after
	int b = lev_start[L0], e = L1 > L0 ? lev_start[L0 + 1] : b, e1 = L1 > L0 + 1 ? lev_start[L0 + 2] : e;
	int cur = 0, have = 0;                   // buffer of the prefetched first row; its validity
	int4 ph = make_int4(0, 0, 0, 0);
	int pr_ = 0;
	for (int l = L0; l < L1; l++) {
		int e2 = (l + 3 <= L1) ? lev_start[l + 3] : e1;
		int per = (e - b + C - 1) / C, p0 = b + rank * per, p1 = min(e, p0 + per);
		// round 1 of the next level's first row, into registers
		int nper = (e1 - e + C - 1) / C, np0 = e + rank * nper, np1 = min(e1, np0 + nper);
		int np = np0 + tid;
		bool nhave = (l + 1 < L1) && np < np1;
		int4 nh = make_int4(0, 0, 0, 0);
		int nr = 0;
		if (nhave) { nh = hdr[np]; nr = rows[np]; }
		for (int p = p0 + tid; p < p1; p += FAC2_T) {
			int4 h;
			int r;
			const int B = cur;
			if (p == p0 + tid && have) {
				h = ph; r = pr_;
				cp_async_wait_all();
			} else {
				h = hdr[p]; r = rows[p];
				const int len0 = h.w & 255;
				for (int q0 = 0; q0 < len0; q0 += 8) {
					double t[8];
#pragma unroll
					for (int u = 0; u < 8; u++) t[u] = (q0 + u < len0) ? AA[h.x + q0 + u] : 0.0;
#pragma unroll
					for (int u = 0; u < 8; u++) if (q0 + u < len0) SV(B, q0 + u) = t[u];
				}
				for (int i0 = 0; i0 < h.z; i0 += 8) {
					int t[8];
#pragma unroll
					for (int u = 0; u < 8; u++) t[u] = (i0 + u < h.z) ? prog[h.y + i0 + u] : 0;
#pragma unroll
					for (int u = 0; u < 8; u++) if (i0 + u < h.z) SP(B, i0 + u) = t[u];
				}
			}
			const int rb = h.x, len = h.w & 255, dpos = (h.w >> 8) & 255, ng = h.w >> 16;
			// round 3: pivots (code < 0: -1-row) and U entries of earlier levels
			const int nops = SP(B, 0);
			for (int i0 = 0; i0 < nops; i0 += 8) {
				double t[8];
#pragma unroll
				for (int u = 0; u < 8; u++) {
					int a = (i0 + u < nops) ? SP(B, 1 + i0 + u) : 0;
					t[u] = (i0 + u < nops) ? __ldcg(a >= 0 ? LU + a : Dinv + (-1 - a)) : 0.0;
				}
#pragma unroll
				for (int u = 0; u < 8; u++) if (i0 + u < nops) SO(i0 + u) = t[u];
			}
			// the elimination (ILUp_precond_setup.c:119-139), in the reference's order
			double d = SV(B, dpos);
			int gp = 1 + nops, oi = 0;
			for (int gi = 0; gi < ng; gi++) {
				int q = SP(B, gp), cnt = SP(B, gp + 1);
				double lq = __dmul_rn(SV(B, q), SO(oi));
				oi++;
				SV(B, q) = lq;
				for (int c = 0; c < cnt; c++) {
					double prod = __dmul_rn(lq, SO(oi));
					oi++;
					int dst = SP(B, gp + 2 + c);
					if (dst < 0) d = __dsub_rn(d, prod);
					else SV(B, dst) = __dsub_rn(SV(B, dst), prod);
				}
				gp += 2 + cnt;
			}
			for (int q = 0; q < len; q++) LU[rb + q] = (q == dpos) ? d : SV(B, q);
			if (d == 0.0) { fg_set_err(err, FEMGPU_E_ZERO_PIVOT); Dinv[r] = 0.0; }
			else Dinv[r] = 1.0 / d;
		}
		// round 2 of the next level's first row: cp.async into the other buffer
		if (nhave) {
			const int B = cur ^ 1, len = nh.w & 255;
			for (int q = 0; q < len; q++) cp_async8(&SV(B, q), AA + nh.x + q);
			for (int i = 0; i < nh.z; i++) cp_async4(&SP(B, i), prog + nh.y + i);
			cp_async_commit();
			cur = B;
		}
		have = nhave;
		ph = nh;
		pr_ = nr;
		__syncwarp();
		cluster_barrier();
		b = e;
		e = e1;
		e1 = e2;
	}
	cp_async_wait_all();
#undef SO
#undef SV
#undef SP
}

// ------------------------------------------------------- host: programs
struct HostLevels {
	int nlev;
	std::vector<int> start, pstart, rows, pos, ppos;   // pos/ppos indexed by row
};

// Matrix block of a row: P contiguous runs of the numbering (P = 0: one).
struct Blocks {
	int P = 0;
	std::vector<int> id;                                  // block of each row (P > 0)
	int of(int r) const { return P ? id[r] : 0; }
	bool same(int r, int c) const { return !P || id[r] == id[c]; }
};

// Block ILU(0) cuts: P contiguous runs of the numbering; couplings between
// runs are dropped.  A sweep costs one barrier per level and its P thread
// blocks run side by side, so the deepest run (levels counted with the
// couplings dropped) sets its time, while where the cuts fall sets how many
// FGMRES iterations the weaker preconditioner costs.  After SYMRCM every front
// is a dependency chain about as long as the front is wide, so equal row
// counts leave the middle runs deepest.  FEMGPU_ILU_BLOCK_CUT selects:
//   levels (default)  run b starts at the first row where the running maximum
//                     of the full factor's forward level reaches
//                     ceil(b * levels / P): equal spans of fronts;
//   depth             the smallest budget T for which the greedy scan (open a
//                     new run at the row whose level would reach T) makes at
//                     most P runs (bisection), the runs with the most rows then
//                     halved until there are P: the shallowest deepest run;
//   rows              row r in run floor(r * P / n).
// Measured at 2048x1024 with FGMRES(80) to 1e-8 (ms per Picard step, ILU
// application, iterations): rows P=8 148 / 1.90 ms / 56-59; levels P=16
// 125 / 1.47 ms / 57-59; depth P=16 136 / 1.38 ms / 65-67, P=12 134 / 1.50
// ms / 60-63.
static std::vector<int> greedy_runs(const int *IA, const int *JA, int n, int T, std::vector<int> &lev)
{
	std::vector<int> first(1, 0);
	int start = 0;
	for (int i = 0; i < n; i++) {
		int L = 0;
		for (int k = IA[i]; k < IA[i + 1] && JA[k] < i; k++)
			if (JA[k] >= start) L = std::max(L, lev[JA[k]] + 1);
		if (L >= T) { start = i; L = 0; first.push_back(i); }
		lev[i] = L;
	}
	first.push_back(n);
	return first;
}

static Blocks make_blocks(const int *IA, const int *JA, int n, int P, std::vector<int> *first_out)
{
	Blocks B;
	if (P <= 1 || n <= 1) { if (first_out) *first_out = { 0, n }; return B; }
	P = std::min(P, n);
	std::vector<int> cut;
	const char *e = getenv("FEMGPU_ILU_BLOCK_CUT");
	if (e && !strcmp(e, "rows")) {
		cut.assign(P + 1, n);
		for (int b = 0; b < P; b++) cut[b] = (int)(((long long)b * n + P - 1) / P);
	} else if (!e || strcmp(e, "depth")) {
		std::vector<int> lev(n, 0), run(n, 0);
		int top = 0;
		for (int i = 0; i < n; i++) {
			int L = 0;
			for (int k = IA[i]; k < IA[i + 1] && JA[k] < i; k++) L = std::max(L, lev[JA[k]] + 1);
			lev[i] = L;
			top = std::max(top, L);
			run[i] = top;
		}
		const long long nl = (long long)top + 1;
		cut.assign(P + 1, n);
		cut[0] = 0;
		for (int b = 1, i = 0; b < P; b++) {
			const long long fl = (nl * b + P - 1) / P;
			while (i < n && run[i] < fl) i++;
			cut[b] = i;
		}
		for (int b = 1; b < P; b++) cut[b] = std::max(cut[b], cut[b - 1] + 1);     // no empty run
		for (int b = P - 1; b >= 1; b--) cut[b] = std::min(cut[b], cut[b + 1] - 1);
	} else {
		std::vector<int> lev(n, 0);
		int lo = 1, hi = n;                       // T = n always gives one run
		while (lo < hi) {
			int T = lo + (hi - lo) / 2;
			if ((int)greedy_runs(IA, JA, n, T, lev).size() - 1 <= P) hi = T;
			else lo = T + 1;
		}
		cut = greedy_runs(IA, JA, n, lo, lev);
		while ((int)cut.size() - 1 < P) {          // halve the run with the most rows
			int bb = 0;
			for (int b = 1; b + 1 < (int)cut.size(); b++)
				if (cut[b + 1] - cut[b] > cut[bb + 1] - cut[bb]) bb = b;
			cut.insert(cut.begin() + bb + 1, cut[bb] + (cut[bb + 1] - cut[bb]) / 2);
		}
	}
	B.P = P;
	B.id.assign(n, 0);
	for (int b = 0; b < P; b++)
		for (int r = cut[b]; r < cut[b + 1]; r++) B.id[r] = b;
	if (first_out) *first_out = cut;
	return B;
}

// Dependency levels of the forward (lower) or backward sweep; with blocks,
// levels are numbered block by block (block b's levels follow block b-1's),
// and clev [P+1] receives each block's first level.
static HostLevels host_levels(const int *IA, const int *JA, int n, bool lower, const Blocks &B,
                              std::vector<int> *clev = nullptr)
{
	HostLevels H;
	std::vector<int> lev(n, 0);
	int P = B.P ? B.P : 1;
	std::vector<int> bl(P, 0);                 // levels of each block
	if (lower) {
		for (int i = 0; i < n; i++) {
			int L = 0;
			for (int k = IA[i]; k < IA[i + 1] && JA[k] < i; k++)
				if (B.same(i, JA[k])) L = std::max(L, lev[JA[k]] + 1);
			lev[i] = L; bl[B.of(i)] = std::max(bl[B.of(i)], L + 1);
		}
	} else {
		for (int i = n - 1; i >= 0; i--) {
			int L = 0;
			for (int k = IA[i]; k < IA[i + 1]; k++) if (JA[k] > i && B.same(i, JA[k])) L = std::max(L, lev[JA[k]] + 1);
			lev[i] = L; bl[B.of(i)] = std::max(bl[B.of(i)], L + 1);
		}
	}
	std::vector<int> boff(P + 1, 0);
	for (int b = 0; b < P; b++) boff[b + 1] = boff[b] + bl[b];
	for (int i = 0; i < n; i++) lev[i] += boff[B.of(i)];
	if (clev) *clev = boff;
	int nlev = boff[P];
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

// Width of the record layout for a sweep whose widest row has w dependencies
// (0: the ELL sub-block layout, used above 16 or when FEMGPU_SWEEP_LAYOUT=ell).
static int rec_width(int w)
{
	const char *e = getenv("FEMGPU_SWEEP_LAYOUT");
	if (e && !strcmp(e, "ell")) return 0;
	static const int widths[] = { 2, 3, 4, 6, 8, 12, 16 };
	for (int v : widths) if (w <= v) return v;
	return 0;
}

// Dependencies at most this many level-order positions before the end of
// their row's level are read from the shared-memory ring, older ones from
// global memory.  FEMGPU_SWEEP_NEAR lowers the limit (1..SW_RING) so that
// small systems exercise the global-memory path too.
static int sweep_near_limit(void)
{
	const char *e = getenv("FEMGPU_SWEEP_NEAR");
	int v = e ? atoi(e) : SW_RING;
	return (v >= 1 && v <= SW_RING) ? v : SW_RING;
}

// Record-layout sweeps run as dataflow (k_sweep_df) unless
// FEMGPU_SWEEP_SYNC=barrier asks for one barrier per level (k_sweep_rec).  At
// 2048x1024 with 16 blocks: 1.36 ms per FP64 application against 1.47.
static bool sweep_dataflow(void)
{
	const char *e = getenv("FEMGPU_SWEEP_SYNC");
	return !(e && !strcmp(e, "barrier"));
}

// Chain-scan programs for the fused and FP32 sweeps (FEMGPU_SWEEP_CHAIN=0
// keeps the row-by-row programs for them too).
static bool sweep_chain(void)
{
	const char *e = getenv("FEMGPU_SWEEP_CHAIN");
	return !(e && !strcmp(e, "0"));
}

// Double-single chain sweeps for the fused FP64 (FGMRES) applications
// (FEMGPU_SWEEP_DS=0: FP64 chain sweeps).
static bool sweep_ds(void)
{
	const char *e = getenv("FEMGPU_SWEEP_DS");
	return !(e && !strcmp(e, "0"));
}

// Levels a dataflow warp may run ahead of the slowest one (FEMGPU_SWEEP_SKEW,
// 1..64; default 4).
static int sweep_skew(void)
{
	const char *e = getenv("FEMGPU_SWEEP_SKEW");
	int v = e ? atoi(e) : 4;
	return (v >= 1 && v <= 64) ? v : 4;
}

// One sweep program.  Forward (lower): L part, outputs to the backward
// sweep's padded level order (target = the U levels' ppos).  Backward: U part
// and pivots, outputs in natural order.
template <typename T, bool UPPER>
static int build_prog(const int *IA, const int *JA, int n, const HostLevels &H, const HostLevels *target,
                      const Blocks &B, const std::vector<int> &clev, fg_sweep &sw)
{
	const bool lower = !UPPER;
	const long long tsize = sizeof(T);
	int near_lim = sweep_near_limit();
	int nlev = H.nlev;
	// sub-blocks: (level, first row within the level, rows, width)
	struct Sub { int l, j0, c, w; };
	std::vector<Sub> subs;
	subs.reserve(nlev + 16);
	for (int l = 0; l < nlev; l++) {
		int c = H.start[l + 1] - H.start[l];
		for (int j0 = 0; j0 < c; j0 += SW_SUB) {
			int cc = std::min(SW_SUB, c - j0), w = 0;
			for (int p = H.start[l] + j0; p < H.start[l] + j0 + cc; p++) {
				int r = H.rows[p], cnt = 0;
				for (int k = IA[r]; k < IA[r + 1]; k++)
					if ((lower ? JA[k] < r : JA[k] > r) && B.same(r, JA[k])) cnt++;
				w = std::max(w, cnt);
			}
			subs.push_back({ l, j0, cc, w });
		}
	}
	int nsb = (int)subs.size();
	int wmax = 0, cmax = 1, lmax = 1;
	for (const Sub &S : subs) { wmax = std::max(wmax, S.w); cmax = std::max(cmax, S.c); }
	for (int l = 0; l < nlev; l++) lmax = std::max(lmax, H.start[l + 1] - H.start[l]);
	int rw = rec_width(wmax);                                         // 0: ELL sub-blocks
	if (rw) {
		// wide records must still leave room for two stages of the widest sub-block
		const long long fixed = (al16((SW_RING + 1) * tsize) + SW_BAR_BYTES + 127) & ~127LL;
		const long long stage = DF_HDR + (long long)cmax * rec_bytes(rw, UPPER, (int)tsize) +
		                        al16((long long)((cmax + 3) & ~3) * tsize);
		if (fixed + 2 * ((stage + 127) & ~127LL) > SW_SMEM_CAP) rw = 0;
	}
	const long long RB = rw ? rec_bytes(rw, UPPER, (int)tsize) : 0;
	// dataflow: the ring holds only what no warp up to the skew behind can still overwrite
	const int skew = sweep_skew();
	bool df = rw && sweep_dataflow() && SW_RING - skew * lmax >= 2 * lmax;
	if (df) near_lim = std::min(near_lim, SW_RING - skew * lmax);
	if (df && near_lim < 2 * lmax) df = false;      // a far dependency must be two levels back
	const long long hdrb = df ? DF_HDR : 16;
	std::vector<int> lev_of(df ? n : 0);
	if (df)
		for (int l = 0; l < nlev; l++)
			for (int q = H.start[l]; q < H.start[l + 1]; q++) lev_of[q] = l;
	std::vector<long long> off(nsb + 1, 0);
	std::vector<int> sb_in(nsb), sb_inb(nsb);
	long long maxblk = 0, bvo = 0, maxin = 0;
	for (int i = 0; i < nsb; i++) {
		int cp = (subs[i].c + 3) & ~3;
		long long bb = rw ? hdrb + (long long)subs[i].c * RB : blk_bytes<T, UPPER>(subs[i].w, cp);
		off[i + 1] = off[i] + bb;
		sb_in[i] = H.pstart[subs[i].l] + subs[i].j0;                 // j0 is a multiple of 4
		sb_inb[i] = (int)al16((long long)cp * tsize);
		maxblk = std::max(maxblk, bb + sb_inb[i]);
		bvo = std::max(bvo, bb);
		maxin = std::max(maxin, (long long)sb_inb[i]);
	}
	if (rw) maxblk = bvo + maxin;                                     // input slice at a fixed offset
	std::vector<unsigned char> prog((size_t)off[nsb] + 16, 0);
	std::vector<long long> val_off;
	std::vector<int> val_src;
	val_off.reserve((size_t)IA[n] + n);
	val_src.reserve((size_t)IA[n] + n);
	for (int i = 0; i < nsb; i++) {
		const Sub &S = subs[i];
		int l = S.l, c = S.c, w = S.w, cp = (c + 3) & ~3, start = H.start[l] + S.j0;
		int end = H.start[l + 1];
		int nsub = (H.start[l + 1] - H.start[l] + SW_SUB - 1) / SW_SUB;
		unsigned char *b = prog.data() + off[i];
		int hasfar = 0;
		for (int j = 0; j < c; j++) {
			int r = H.rows[start + j];
			for (int q = IA[r]; q < IA[r + 1]; q++) {
				int col = JA[q];
				if ((lower ? col < r : col > r) && B.same(r, col) && end - H.pos[col] > near_lim) hasfar = 1;
			}
		}
		if (rw) {
			const int hh[4] = { c, nsub, start, hasfar };
			memcpy(b, hh, sizeof hh);
			if (df) {
				// need[w][pw]: smallest level distance of a dependency of warp w's rows
				// produced by warp pw (255: none within skew + 1 levels)
				unsigned char *need = b + 16;
				memset(need, 255, (size_t)SW2_CW * NEED_STRIDE);
				for (int j = 0; j < c; j++) {
					int r = H.rows[start + j];
					for (int q = IA[r]; q < IA[r + 1]; q++) {
						int col = JA[q];
						if ((lower ? !(col < r) : !(col > r)) || !B.same(r, col)) continue;
						int p = H.pos[col], lp = lev_of[p], dl = l - lp;
						if (end - p > near_lim) dl--;      // read back from global memory: the next level's release
						if (dl > skew + 1) continue;
						int pw = ((p - H.start[lp]) % SW_SUB) / 32;
						unsigned char &e = need[(j / 32) * NEED_STRIDE + pw];
						if (dl < (int)e) e = (unsigned char)dl;
					}
				}
			}
			for (int j = 0; j < c; j++) {
				int *ri = (int *)(b + hdrb + (size_t)j * RB), r = H.rows[start + j], k = 0;
				long long vo = off[i] + hdrb + (long long)j * RB + rec_ib(rw);
				for (int q = 0; q < rw; q++) ri[q] = (int)(SW_NEAR | SW_RING);   // the zero slot
				ri[rw] = lower ? target->ppos[r] : r;
				for (int q = IA[r]; q < IA[r + 1]; q++) {
					int col = JA[q];
					if ((lower ? !(col < r) : !(col > r)) || !B.same(r, col)) continue;
					int p = H.pos[col];
					ri[k] = (int)((end - p <= near_lim) ? (SW_NEAR | (unsigned)(p & (SW_RING - 1)))
					                                   : (unsigned)(lower ? target->ppos[col] : col));
					val_off.push_back(vo + k * tsize);
					val_src.push_back(q);
					k++;
				}
				for (; k < rw; k++) { val_off.push_back(vo + k * tsize); val_src.push_back(-1); }
				if (!lower) { val_off.push_back(vo + rw * tsize); val_src.push_back(-2 - r); }
			}
			continue;
		}
		LevHdr h = { c, w, start, cp, nsub, hasfar, (int)al16(SW_HDR + (long long)(w + 1) * cp * 4),
		             (int)blk_bytes<T, UPPER>(w, cp) };
		memcpy(b, &h, sizeof h);
		int *dep = (int *)(b + SW_HDR), *outp = dep + (size_t)w * cp;
		long long voff = al16(SW_HDR + (long long)(w + 1) * cp * 4);
		for (int k = 0; k < w * cp; k++) dep[k] = (int)(SW_NEAR | SW_RING);       // the zero slot
		for (int j = 0; j < c; j++) {
			int r = H.rows[start + j], k = 0;
			outp[j] = lower ? target->ppos[r] : r;
			for (int q = IA[r]; q < IA[r + 1]; q++) {
				int col = JA[q];
				if ((lower ? !(col < r) : !(col > r)) || !B.same(r, col)) continue;
				int p = H.pos[col];
				unsigned code = (end - p <= near_lim) ? (SW_NEAR | (unsigned)(p & (SW_RING - 1)))
				                                     : (unsigned)(lower ? target->ppos[col] : col);
				dep[(size_t)k * cp + j] = (int)code;
				val_off.push_back(off[i] + voff + ((long long)k * cp + j) * tsize);
				val_src.push_back(q);
				k++;
			}
			for (; k < w; k++) {
				val_off.push_back(off[i] + voff + ((long long)k * cp + j) * tsize);
				val_src.push_back(-1);
			}
			if (!lower) {
				val_off.push_back(off[i] + voff + ((long long)w * cp + j) * tsize);
				val_src.push_back(-2 - r);
			}
		}
	}
	// first sub-block of each matrix block (its first level's first sub-block)
	std::vector<int> csb(clev.size(), nsb);
	for (size_t b = 0, i = 0; b < clev.size(); b++) {
		while (i < (size_t)nsb && subs[i].l < clev[b]) i++;
		csb[b] = (int)i;
	}
	sw.nchunk = (int)clev.size() - 1;
	sw.rw = rw;
	sw.df = df;
	sw.skew = skew;
	sw.bvo = (int)bvo;
	sw.cmax = cmax;
	sw.nlev = nlev;
	sw.nsb = nsb;
	sw.bytes = off[nsb];
	sw.maxblk = maxblk;
	sw.nval = (long long)val_off.size();
	sw.npad = H.pstart[nlev];
	int rc;
	FG_TRY(cudaMalloc((void **)&sw.prog, prog.size()));
	FG_TRY(cudaMemcpy(sw.prog, prog.data(), prog.size(), cudaMemcpyHostToDevice));
	if ((rc = up_vec(&sw.blk_off, off))) return rc;
	if ((rc = up_vec(&sw.sb_in, sb_in))) return rc;
	if ((rc = up_vec(&sw.sb_inb, sb_inb))) return rc;
	if ((rc = up_vec(&sw.lev_start, H.start))) return rc;
	if ((rc = up_vec(&sw.rows, H.rows))) return rc;
	std::vector<int> ppos_by_pos(n);
	for (int p = 0; p < n; p++) ppos_by_pos[p] = H.ppos[H.rows[p]];
	if ((rc = up_vec(&sw.ppos, ppos_by_pos))) return rc;
	if ((rc = up_vec(&sw.val_off, val_off))) return rc;
	if ((rc = up_vec(&sw.val_src, val_src))) return rc;
	if ((rc = up_vec(&sw.chunk_sb, csb))) return rc;
	if ((rc = up_vec(&sw.chunk_lev, clev))) return rc;
	return 0;
}

// ------------------------------------------- host: chain-scan programs
// Segments of one sweep (the order of k_sweep_cs): rows in sweep order
// (forward ascending, backward descending) within their matrix block; a row
// joins the current segment when it depends on its sweep predecessor, the
// segment has fewer than 32 rows and the row's other dependencies are all on
// earlier levels than the segment's -- otherwise it starts a new segment,
// whose level is one past its dependencies' (the predecessor among them).
// This cut keeps segments of consecutive fronts aligned, so a block's depth
// is about its fronts plus a front's chunk count, not fronts plus front width.
// Each level's segments are packed, in order, into 32-slot chunks.
struct ChainLevels {
	int nlev = 0, nslot = 0, maxw = 0;
	std::vector<int> lstart;   // [nlev+1] first slot of each level (multiples of 32)
	std::vector<int> slot_row; // [nslot] row in each slot (-1 padding)
	std::vector<int> slot_pred; // [nslot] CSR position of the chain coefficient (-1: segment start, padding)
	std::vector<int> slot;     // [n] slot of each row
	std::vector<int> clev;     // [P+1] first level of each matrix block
	int rowlev_max = 0;        // deepest block in row levels (for the choice of program)
};

static ChainLevels host_chain_levels(const int *IA, const int *JA, int n, bool lower, const Blocks &B)
{
	ChainLevels H;
	const int P = B.P ? B.P : 1;
	std::vector<int> seg_of(n), seg_lev, seg_blk, seg_first, seg_pred_pos(n, -1), rowlev(n, 0);
	std::vector<int> bl(P, 0), blrow(P, 0);
	int cur = -1, run = 0;
	for (int s = 0; s < n; s++) {
		const int i = lower ? s : n - 1 - s, pred = lower ? i - 1 : i + 1, b = B.of(i);
		int elev = 0, ppos = -1, rl = 0, nd = 0;
		for (int k = IA[i]; k < IA[i + 1]; k++) {
			const int c = JA[k];
			if (!(lower ? c < i : c > i) || !B.same(i, c)) continue;
			rl = std::max(rl, rowlev[c] + 1);
			if (c == pred) { ppos = k; continue; }
			elev = std::max(elev, seg_lev[seg_of[c]] + 1);
			nd++;
		}
		rowlev[i] = rl;
		blrow[b] = std::max(blrow[b], rl + 1);
		bool chain = ppos >= 0 && cur >= 0 && seg_blk[cur] == b && run < 32 && elev <= seg_lev[cur] &&
		             seg_of[pred] == cur;
		if (chain) {
			seg_of[i] = cur;
			seg_pred_pos[i] = ppos;
			run++;
		} else {
			if (ppos >= 0) { elev = std::max(elev, seg_lev[seg_of[pred]] + 1); nd++; }
			seg_lev.push_back(elev);
			seg_blk.push_back(b);
			seg_first.push_back(i);
			cur = (int)seg_lev.size() - 1;
			seg_of[i] = cur;
			run = 1;
			bl[b] = std::max(bl[b], elev + 1);
		}
		H.maxw = std::max(H.maxw, nd);
	}
	for (int b = 0; b < P; b++) H.rowlev_max = std::max(H.rowlev_max, blrow[b]);
	std::vector<int> boff(P + 1, 0);
	for (int b = 0; b < P; b++) boff[b + 1] = boff[b] + bl[b];
	H.clev = boff;
	H.nlev = boff[P];
	const int nseg = (int)seg_lev.size();
	// segments by global level, in creation order; their rows in sweep order
	std::vector<int> lcount(H.nlev + 1, 0), seg_len(nseg, 0), order(nseg);
	for (int g = 0; g < nseg; g++) lcount[seg_lev[g] + boff[seg_blk[g]] + 1]++;
	for (int l = 0; l < H.nlev; l++) lcount[l + 1] += lcount[l];
	{
		std::vector<int> fill(lcount.begin(), lcount.end() - 1);
		for (int g = 0; g < nseg; g++) order[fill[seg_lev[g] + boff[seg_blk[g]]]++] = g;
	}
	for (int i = 0; i < n; i++) seg_len[seg_of[i]]++;
	std::vector<int> seg_slot(nseg);
	H.lstart.assign(H.nlev + 1, 0);
	int slot = 0;
	for (int l = 0; l < H.nlev; l++) {
		H.lstart[l] = slot;
		int used = 32;                                    // lanes used in the current chunk
		for (int q = lcount[l]; q < lcount[l + 1]; q++) {
			const int g = order[q];
			if (used + seg_len[g] > 32) { if (used < 32) slot += 32 - used; used = 0; }
			seg_slot[g] = slot;
			slot += seg_len[g];
			used += seg_len[g];
		}
		if (used < 32) slot += 32 - used;
	}
	H.lstart[H.nlev] = slot;
	H.nslot = slot;
	H.slot_row.assign(slot, -1);
	H.slot_pred.assign(slot, -1);
	H.slot.assign(n, 0);
	std::vector<int> next(seg_slot);
	for (int s = 0; s < n; s++) {
		const int i = lower ? s : n - 1 - s, g = seg_of[i], sl = next[g]++;
		H.slot[i] = sl;
		H.slot_row[sl] = i;
		H.slot_pred[sl] = seg_pred_pos[i];
	}
	return H;
}

// The chain-scan program of one sweep (k_sweep_cs): sub-blocks of up to
// SW_SUB slots of one level, the k_sweep_df header and need tables, one record
// per slot, the input slice at a fixed stage offset.  Forward: L part, outputs
// to the backward program's slots; backward: U part and pivots, outputs in
// natural order.  Returns FEMGPU_E_MESH when the ring cannot hold the widest
// level (the caller keeps the row-by-row programs then).
template <typename T, bool UPPER>
static int build_prog_chain(const int *IA, const int *JA, int n, const ChainLevels &H, const ChainLevels *target,
                            const Blocks &B, fg_sweep &sw)
{
	const bool lower = !UPPER;
	const long long tsize = sizeof(T);
	const int nlev = H.nlev;
	int rw = rec_width(std::max(H.maxw, 1));
	if (!rw) return FEMGPU_E_MESH;
	const long long RB = rec_bytes_cs(rw, UPPER, (int)tsize), IBy = rec_ib(rw);
	int lmax = 32;
	for (int l = 0; l < nlev; l++) lmax = std::max(lmax, H.lstart[l + 1] - H.lstart[l]);
	int skew = std::min(sweep_skew(), 4);
	while (skew > 1 && SW_RING - skew * lmax < 2 * lmax) skew--;
	if (SW_RING - skew * lmax < 2 * lmax) return FEMGPU_E_MESH;
	// a dependency read back from global memory must be two levels back: a
	// lowered reach (FEMGPU_SWEEP_NEAR) stops at two of the widest levels
	const int near_lim = std::max(std::min(sweep_near_limit(), SW_RING - skew * lmax), 2 * lmax);
	struct Sub { int l, j0, c; };
	std::vector<Sub> subs;
	for (int l = 0; l < nlev; l++) {
		const int c = H.lstart[l + 1] - H.lstart[l];
		for (int j0 = 0; j0 < c; j0 += SW_SUB) subs.push_back({ l, j0, std::min(SW_SUB, c - j0) });
	}
	const int nsb = (int)subs.size();
	int cmax = 32;
	for (const Sub &S : subs) cmax = std::max(cmax, S.c);
	const long long fixed = (al16((SW_RING + 1) * tsize) + SW_BAR_BYTES + 127) & ~127LL;
	const long long stage = DF_HDR + (long long)cmax * RB + al16((long long)cmax * tsize);
	if (fixed + 2 * ((stage + 127) & ~127LL) > SW_SMEM_CAP) return FEMGPU_E_MESH;
	std::vector<int> lev_of(H.nslot);
	for (int l = 0; l < nlev; l++)
		for (int q = H.lstart[l]; q < H.lstart[l + 1]; q++) lev_of[q] = l;
	std::vector<long long> off(nsb + 1, 0);
	std::vector<int> sb_in(nsb), sb_inb(nsb);
	long long bvo = 0, maxin = 0;
	for (int i = 0; i < nsb; i++) {
		const long long bb = DF_HDR + (long long)subs[i].c * RB;
		off[i + 1] = off[i] + bb;
		sb_in[i] = H.lstart[subs[i].l] + subs[i].j0;
		sb_inb[i] = (int)al16((long long)subs[i].c * tsize);
		bvo = std::max(bvo, bb);
		maxin = std::max(maxin, (long long)sb_inb[i]);
	}
	std::vector<unsigned char> prog((size_t)off[nsb] + 16, 0);
	std::vector<long long> val_off, cs_voff(H.nslot, -1);
	std::vector<int> val_src, cs_src(H.nslot, -1), cs_row(H.nslot, 0);
	val_off.reserve((size_t)H.nslot * (rw + 1));
	val_src.reserve((size_t)H.nslot * (rw + 1));
	for (int i = 0; i < nsb; i++) {
		const Sub &S = subs[i];
		const int l = S.l, c = S.c, start = H.lstart[l] + S.j0, end = H.lstart[l + 1];
		const int nsub = (end - H.lstart[l] + SW_SUB - 1) / SW_SUB;
		unsigned char *b = prog.data() + off[i];
		int hasfar = 0;
		for (int j = 0; j < c; j++) {
			const int r = H.slot_row[start + j];
			if (r < 0) continue;
			for (int q = IA[r]; q < IA[r + 1]; q++) {
				const int col = JA[q];
				if ((lower ? col < r : col > r) && B.same(r, col) && q != H.slot_pred[start + j] &&
				    end - H.slot[col] > near_lim) hasfar = 1;
			}
		}
		const int hh[4] = { c, nsub, start, hasfar };
		memcpy(b, hh, sizeof hh);
		unsigned char *need = b + 16;
		memset(need, 255, (size_t)SW2_CW * NEED_STRIDE);
		for (int j = 0; j < c; j++) {
			const int r = H.slot_row[start + j];
			int *ri = (int *)(b + DF_HDR + (size_t)j * RB), k = 0;
			const long long vo = off[i] + DF_HDR + (long long)j * RB + IBy;
			for (int q = 0; q < rw; q++) ri[q] = (int)(SW_NEAR | SW_RING);     // the zero slot
			if (r < 0) {                                                       // padding
				ri[rw] = -1;
				for (int q = 0; q < rw + (UPPER ? 1 : 0); q++) { val_off.push_back(vo + q * tsize); val_src.push_back(-1); }
				continue;
			}
			ri[rw] = lower ? target->slot[r] : r;
			for (int q = IA[r]; q < IA[r + 1]; q++) {
				const int col = JA[q];
				if ((lower ? !(col < r) : !(col > r)) || !B.same(r, col) || q == H.slot_pred[start + j]) continue;
				const int p = H.slot[col], lp = lev_of[p];
				int dl = l - lp;
				const bool nearp = end - p <= near_lim;
				ri[k] = (int)(nearp ? (SW_NEAR | (unsigned)(p & (SW_RING - 1))) : (unsigned)(lower ? target->slot[col] : col));
				if (!nearp) dl--;                     // read back from global memory: the next level's release
				if (dl <= skew + 1) {
					const int pw = ((p - H.lstart[lp]) % SW_SUB) / 32;
					unsigned char &e = need[(j / 32) * NEED_STRIDE + pw];
					if (dl < (int)e) e = (unsigned char)dl;
				}
				val_off.push_back(vo + k * tsize);
				val_src.push_back(q);
				k++;
			}
			for (; k < rw; k++) { val_off.push_back(vo + k * tsize); val_src.push_back(-1); }
			if (!lower) { val_off.push_back(vo + rw * tsize); val_src.push_back(-2 - r); }
			cs_voff[start + j] = vo + (rw + (UPPER ? 1 : 0)) * tsize;
			cs_src[start + j] = H.slot_pred[start + j];
			cs_row[start + j] = r;
		}
		// padding slots: multipliers zero (the refresh writes them too)
		for (int j = 0; j < c; j++)
			if (H.slot_row[start + j] < 0) cs_voff[start + j] = off[i] + DF_HDR + (long long)j * RB + IBy +
			                                                    (rw + (UPPER ? 1 : 0)) * tsize;
	}
	// every index the kernel will follow stays inside its array: dependency
	// codes (ring slots or output positions), output positions, input slices
	{
		const long long nout = lower ? target->nslot : n;
		for (int i = 0; i < nsb; i++) {
			const unsigned char *b = prog.data() + off[i];
			const int c = subs[i].c;
			if (sb_in[i] < 0 || (long long)sb_in[i] + c > H.nslot) return FEMGPU_E_MESH;
			for (int j = 0; j < c; j++) {
				const int *ri = (const int *)(b + DF_HDR + (size_t)j * RB);
				for (int q = 0; q < rw; q++) {
					const unsigned code = (unsigned)ri[q];
					if (code & SW_NEAR) { if ((code & ~SW_NEAR) > SW_RING) return FEMGPU_E_MESH; }
					else if ((long long)code >= nout) return FEMGPU_E_MESH;
				}
				if (ri[rw] < -1 || ri[rw] >= nout) return FEMGPU_E_MESH;
			}
		}
		for (size_t q = 0; q < cs_voff.size(); q++)
			if (cs_voff[q] < 0 || cs_voff[q] + 5 * tsize > off[nsb]) return FEMGPU_E_MESH;
		for (size_t q = 0; q < val_off.size(); q++)
			if (val_off[q] < 0 || val_off[q] + tsize > off[nsb]) return FEMGPU_E_MESH;
	}
	std::vector<int> csb(H.clev.size(), nsb);
	for (size_t bk = 0, i = 0; bk < H.clev.size(); bk++) {
		while (i < (size_t)nsb && subs[i].l < H.clev[bk]) i++;
		csb[bk] = (int)i;
	}
	// real rows in slot order (the gather of the sweep input)
	std::vector<int> rows, ppos;
	rows.reserve(n);
	ppos.reserve(n);
	for (int q = 0; q < H.nslot; q++)
		if (H.slot_row[q] >= 0) { rows.push_back(H.slot_row[q]); ppos.push_back(q); }
	std::vector<int> lev_start(H.lstart);
	sw.nchunk = (int)H.clev.size() - 1;
	sw.rw = rw;
	sw.df = 1;
	sw.cs = 1;
	sw.skew = skew;
	sw.bvo = (int)bvo;
	sw.cmax = cmax;
	sw.nlev = nlev;
	sw.nsb = nsb;
	sw.bytes = off[nsb];
	sw.maxblk = bvo + maxin;
	sw.nval = (long long)val_off.size();
	sw.npad = H.nslot;
	sw.nslot = H.nslot;
	int rc;
	FG_TRY(cudaMalloc((void **)&sw.prog, prog.size()));
	FG_TRY(cudaMemcpy(sw.prog, prog.data(), prog.size(), cudaMemcpyHostToDevice));
	if ((rc = up_vec(&sw.blk_off, off))) return rc;
	if ((rc = up_vec(&sw.sb_in, sb_in))) return rc;
	if ((rc = up_vec(&sw.sb_inb, sb_inb))) return rc;
	if ((rc = up_vec(&sw.lev_start, lev_start))) return rc;
	if ((rc = up_vec(&sw.rows, rows))) return rc;
	if ((rc = up_vec(&sw.ppos, ppos))) return rc;
	if ((rc = up_vec(&sw.val_off, val_off))) return rc;
	if ((rc = up_vec(&sw.val_src, val_src))) return rc;
	if ((rc = up_vec(&sw.chunk_sb, csb))) return rc;
	if ((rc = up_vec(&sw.chunk_lev, H.clev))) return rc;
	if ((rc = up_vec(&sw.cs_voff, cs_voff))) return rc;
	if ((rc = up_vec(&sw.cs_src, cs_src))) return rc;
	if ((rc = up_vec(&sw.cs_row, cs_row))) return rc;
	return 0;
}

// Elimination program of every row, in forward level order (the layout
// k_ilu0_factor_cta reads): the same sequence of updates as
// ILUp_precond_setup.c:119-139, resolved against the pattern once.
static int build_factor_prog(const int *IA, const int *JA, int n, const HostLevels &Lo, const Blocks &B,
                             fg_ilu_sweeps &S)
{
	std::vector<int> ptr(n + 1, 0), prog;
	prog.reserve((size_t)n * 24);
	for (int p = 0; p < n; p++) {
		int r = Lo.rows[p], rb = IA[r], len = IA[r + 1] - rb, dpos = -1, ng = 0;
		if (len > FAC_CAP) return FEMGPU_E_MESH;
		for (int q = 0; q < len; q++) if (JA[rb + q] == r) dpos = q;
		if (dpos < 0) return FEMGPU_E_ZERO_PIVOT;           // no diagonal entry
		ptr[p] = (int)prog.size();
		size_t hdr = prog.size();
		prog.push_back(dpos);
		prog.push_back(0);
		for (int q = 0; q < len && JA[rb + q] < r; q++) {
			int jrow = JA[rb + q], cnt = 0;
			if (!B.same(r, jrow)) continue;              // coupling to another block: dropped
			size_t g = prog.size();
			prog.push_back(q);
			prog.push_back(jrow);
			prog.push_back(0);
			for (int k = IA[jrow]; k < IA[jrow + 1]; k++) {
				int col = JA[k], pos = -1;
				if (col <= jrow || !B.same(r, col)) continue;
				for (int m = 0; m < len; m++) if (JA[rb + m] == col) { pos = m; break; }
				if (pos < 0) continue;
				prog.push_back(col == r ? -1 : pos);
				prog.push_back(k);
				cnt++;
			}
			prog[g + 2] = cnt;
			ng++;
		}
		prog[hdr + 1] = ng;
	}
	ptr[n] = (int)prog.size();
	int rc;
	if ((rc = up_vec(&S.fac_ptr, ptr))) return rc;
	return up_vec(&S.fac_prog, prog);
}

// The elimination program of k_ilu0_factor_cluster: per level-order
// position a header and a row program whose operand addresses come first
// (couplings between matrix blocks dropped, as in build_factor_prog).  fac2_ok = 0 when a row exceeds the kernel's per-row capacity.
static int build_factor_prog2(const int *IA, const int *JA, int n, const HostLevels &Lo, const Blocks &B,
                              fg_ilu_sweeps &S)
{
	std::vector<int> hdr((size_t)n * 4), prog, ops, grp;
	prog.reserve((size_t)n * 28);
	S.fac2_ok = 1;
	for (int p = 0; p < n; p++) {
		int r = Lo.rows[p], rb = IA[r], len = IA[r + 1] - rb, dpos = -1, ng = 0;
		for (int q = 0; q < len; q++) if (JA[rb + q] == r) dpos = q;
		ops.clear();
		grp.clear();
		for (int q = 0; q < len && JA[rb + q] < r; q++) {
			int jrow = JA[rb + q];
			if (!B.same(r, jrow)) continue;              // coupling to another block: dropped
			size_t g = grp.size();
			grp.push_back(q);
			grp.push_back(0);
			ops.push_back(-1 - jrow);
			for (int k = IA[jrow]; k < IA[jrow + 1]; k++) {
				int col = JA[k], pos = -1;
				if (col <= jrow || !B.same(r, col)) continue;
				for (int m = 0; m < len; m++) if (JA[rb + m] == col) { pos = m; break; }
				if (pos < 0) continue;
				grp.push_back(col == r ? -1 : pos);
				ops.push_back(k);
				grp[g + 1]++;
			}
			ng++;
		}
		int plen = 1 + (int)ops.size() + (int)grp.size();
		if (len > FAC_CAP || dpos < 0 || plen > FAC2_MAXP || (int)ops.size() > FAC2_MAXOPS || ng > 32767) {
			S.fac2_ok = 0;
			return 0;
		}
		hdr[4 * (size_t)p] = rb;
		hdr[4 * (size_t)p + 1] = (int)prog.size();
		hdr[4 * (size_t)p + 2] = plen;
		hdr[4 * (size_t)p + 3] = len | (dpos << 8) | (ng << 16);
		prog.push_back((int)ops.size());
		prog.insert(prog.end(), ops.begin(), ops.end());
		prog.insert(prog.end(), grp.begin(), grp.end());
	}
	int rc;
	if ((rc = up_vec(&S.fac2_hdr, hdr))) return rc;
	return up_vec(&S.fac2, prog);
}

// Cluster size for the factorisation of P matrix blocks (one cluster each):
// the largest of 16, 8, 4, 2 CTAs with which P clusters fit on the device at
// once; 0 when none does (the one-block-per-matrix-block kernel runs).
static int factor_cluster_size(int P)
{
	static int init = 0, fits[17];
	if (!init) {
		init = 1;
		if (cudaFuncSetAttribute(k_ilu0_factor_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, FAC2_SMEM) !=
		    cudaSuccess) { cudaGetLastError(); return 0; }
		cudaFuncSetAttribute(k_ilu0_factor_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
		cudaGetLastError();
		for (int c = 16; c >= 1; c /= 2) {
			cudaLaunchConfig_t cfg = {};
			cudaLaunchAttribute at[1];
			at[0].id = cudaLaunchAttributeClusterDimension;
			at[0].val.clusterDim.x = (unsigned)c; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
			cfg.gridDim = dim3((unsigned)c); cfg.blockDim = dim3(FAC2_T); cfg.dynamicSmemBytes = FAC2_SMEM;
			cfg.attrs = at; cfg.numAttrs = 1;
			int ncl = 0;
			if (cudaOccupancyMaxActiveClusters(&ncl, k_ilu0_factor_cluster, &cfg) == cudaSuccess) fits[c] = ncl;
			cudaGetLastError();
		}
	}
	// FEMGPU_FACTOR_CLUSTER caps the cluster size (1 allowed: one CTA per
	// block with the cluster kernel)
	const char *e = getenv("FEMGPU_FACTOR_CLUSTER");
	const int cap = e ? atoi(e) : 16;
	for (int c = 16; c >= (cap == 1 ? 1 : 2); c /= 2)
		if (c <= cap && fits[c] >= P) return c;
	return 0;
}

#define SW_SET(T, U, CW, F) FG_TRY(cudaFuncSetAttribute(k_sweep<T, U, CW, F>, \
	cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP))
#define SW_SET_CW(CW) SW_SET(double, false, CW, false); SW_SET(double, true, CW, false); \
	SW_SET(double, false, CW, true); SW_SET(double, true, CW, true); \
	SW_SET(float, false, CW, false); SW_SET(float, true, CW, false)
#define SR_SET(T, U, F, W) FG_TRY(cudaFuncSetAttribute(k_sweep_rec<T, U, F, W>, \
	cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP))
#define SD_SET(T, U, F, W) FG_TRY(cudaFuncSetAttribute(k_sweep_df<T, U, F, W>, \
	cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP))
#define SC_SET(T, U, W) FG_TRY(cudaFuncSetAttribute(k_sweep_cs<T, U, W>, \
	cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP))
#define SR_SET_W(W) SC_SET(double, false, W); SC_SET(double, true, W); SC_SET(float, false, W); \
	SC_SET(float, true, W); SC_SET(dsf, false, W); SC_SET(dsf, true, W); \
	SR_SET(double, false, false, W); SR_SET(double, true, false, W); \
	SR_SET(double, false, true, W); SR_SET(double, true, true, W); \
	SR_SET(float, false, false, W); SR_SET(float, true, false, W); \
	SD_SET(double, false, false, W); SD_SET(double, true, false, W); \
	SD_SET(double, false, true, W); SD_SET(double, true, true, W); \
	SD_SET(float, false, false, W); SD_SET(float, true, false, W)
#define SF_SET(W) FG_TRY(cudaFuncSetAttribute(k_sweep_cs_fb<dsf, W, W>, \
	cudaFuncAttributeMaxDynamicSharedMemorySize, SW_SMEM_CAP))
static int sweep_attrs(void)
{
	SF_SET(2);
	SF_SET(3);
	SF_SET(4);
	SF_SET(6);
	SF_SET(8);
	SW_SET_CW(4);
	SW_SET_CW(8);
	SW_SET_CW(16);
	SR_SET_W(2);
	SR_SET_W(3);
	SR_SET_W(4);
	SR_SET_W(6);
	SR_SET_W(8);
	SR_SET_W(12);
	SR_SET_W(16);
	return 0;
}

// Consumer warps per sweep (4, 8 or 16; FEMGPU_SWEEP_WARPS overrides).
static int sweep_cw(void)
{
	static int cw = 0;
	if (!cw) {
		const char *e = getenv("FEMGPU_SWEEP_WARPS");
		int v = e ? atoi(e) : 16;
		cw = (v == 4 || v == 8 || v == 16) ? v : 16;
	}
	return cw;
}

// fma: fused multiply-subtract in the FP64 sweeps (the FGMRES solves); the
// separately rounded form reproduces the reference bit for bit.
template <typename T, bool UPPER, bool FMA>
static void launch_df(const SweepArgs &a, int rw, int grid, int bytes, cudaStream_t s, const T *in, T *out)
{
	const int nt = (SW2_CW + 1) * 32;
	switch (rw) {
	case 2: k_sweep_df<T, UPPER, FMA, 2><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 3: k_sweep_df<T, UPPER, FMA, 3><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 4: k_sweep_df<T, UPPER, FMA, 4><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 6: k_sweep_df<T, UPPER, FMA, 6><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 8: k_sweep_df<T, UPPER, FMA, 8><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 12: k_sweep_df<T, UPPER, FMA, 12><<<grid, nt, bytes, s>>>(a, in, out); break;
	default: k_sweep_df<T, UPPER, FMA, 16><<<grid, nt, bytes, s>>>(a, in, out); break;
	}
}

template <typename T, bool UPPER>
static void launch_cs(const SweepArgs &a, int rw, int grid, int bytes, cudaStream_t s, const T *in, T *out)
{
	const int nt = (SW2_CW + 1) * 32;
	switch (rw) {
	case 2: k_sweep_cs<T, UPPER, 2><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 3: k_sweep_cs<T, UPPER, 3><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 4: k_sweep_cs<T, UPPER, 4><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 6: k_sweep_cs<T, UPPER, 6><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 8: k_sweep_cs<T, UPPER, 8><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 12: k_sweep_cs<T, UPPER, 12><<<grid, nt, bytes, s>>>(a, in, out); break;
	default: k_sweep_cs<T, UPPER, 16><<<grid, nt, bytes, s>>>(a, in, out); break;
	}
}

// Both double-single sweeps in one launch (k_sweep_cs_fb) when the two
// programs have the same record width (one of 2, 3, 4, 6, 8) and blocks;
// false: the caller launches them one by one.
static bool launch_cs_fb(const SweepArgs &al, const SweepArgs &au, int rw, int grid, int bytes, cudaStream_t s,
                         const dsf *in, dsf *y, dsf *out)
{
	const int nt = (SW2_CW + 1) * 32;
	switch (rw) {
	case 2: k_sweep_cs_fb<dsf, 2, 2><<<grid, nt, bytes, s>>>(al, au, in, y, out); return true;
	case 3: k_sweep_cs_fb<dsf, 3, 3><<<grid, nt, bytes, s>>>(al, au, in, y, out); return true;
	case 4: k_sweep_cs_fb<dsf, 4, 4><<<grid, nt, bytes, s>>>(al, au, in, y, out); return true;
	case 6: k_sweep_cs_fb<dsf, 6, 6><<<grid, nt, bytes, s>>>(al, au, in, y, out); return true;
	case 8: k_sweep_cs_fb<dsf, 8, 8><<<grid, nt, bytes, s>>>(al, au, in, y, out); return true;
	default: return false;
	}
}

template <typename T, bool UPPER, bool FMA>
static void launch_rec(const SweepArgs &a, int rw, int grid, int bytes, cudaStream_t s, const T *in, T *out)
{
	const int nt = (SW2_CW + 1) * 32;
	switch (rw) {
	case 2: k_sweep_rec<T, UPPER, FMA, 2><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 3: k_sweep_rec<T, UPPER, FMA, 3><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 4: k_sweep_rec<T, UPPER, FMA, 4><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 6: k_sweep_rec<T, UPPER, FMA, 6><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 8: k_sweep_rec<T, UPPER, FMA, 8><<<grid, nt, bytes, s>>>(a, in, out); break;
	case 12: k_sweep_rec<T, UPPER, FMA, 12><<<grid, nt, bytes, s>>>(a, in, out); break;
	default: k_sweep_rec<T, UPPER, FMA, 16><<<grid, nt, bytes, s>>>(a, in, out); break;
	}
}

template <typename T, bool UPPER>
static void launch_sweep(const SweepArgs &a, int rw, int df, int grid, int bytes, cudaStream_t s, const T *in,
                         T *out, bool fma, int cs = 0)
{
	if (cs) {
		launch_cs<T, UPPER>(a, rw, grid, bytes, s, in, out);
		return;
	}
	if (rw && df) {
		if (fma && sizeof(T) == 8) launch_df<T, UPPER, true>(a, rw, grid, bytes, s, in, out);
		else launch_df<T, UPPER, false>(a, rw, grid, bytes, s, in, out);
		return;
	}
	if (rw) {
		if (fma && sizeof(T) == 8) launch_rec<T, UPPER, true>(a, rw, grid, bytes, s, in, out);
		else launch_rec<T, UPPER, false>(a, rw, grid, bytes, s, in, out);
		return;
	}
	int cw = sweep_cw();
	if (fma && sizeof(T) == 8) {
		if (cw == 4) k_sweep<T, UPPER, 4, true><<<grid, 160, bytes, s>>>(a, in, out);
		else if (cw == 8) k_sweep<T, UPPER, 8, true><<<grid, 288, bytes, s>>>(a, in, out);
		else k_sweep<T, UPPER, 16, true><<<grid, 544, bytes, s>>>(a, in, out);
	} else {
		if (cw == 4) k_sweep<T, UPPER, 4, false><<<grid, 160, bytes, s>>>(a, in, out);
		else if (cw == 8) k_sweep<T, UPPER, 8, false><<<grid, 288, bytes, s>>>(a, in, out);
		else k_sweep<T, UPPER, 16, false><<<grid, 544, bytes, s>>>(a, in, out);
	}
}

static int sweep_smem(const fg_sweep &sw, size_t tsize, int *D, int *stage_bytes)
{
	size_t fixed = ((al16((SW_RING + 1) * tsize) + SW_BAR_BYTES + 127) & ~(size_t)127);
	size_t sb = (size_t)((sw.maxblk + 127) & ~127LL);
	if (fixed + 2 * sb > SW_SMEM_CAP) return FEMGPU_E_MESH;   // a sub-block too wide to stage
	int d = (int)((SW_SMEM_CAP - fixed) / sb);
	if (d > SW_MAXD) d = SW_MAXD;
	*D = d;
	*stage_bytes = (int)sb;
	return (int)(fixed + (size_t)d * sb);
}

// Host only (no device call): the block ILU(0) cut of a CSR pattern, as
// fg_ilu_prepare computes it.  first receives R + 1 row boundaries, R =
// max(min(P, n), 1); cap is the room in first.  The pattern is checked first
// (IA[0] == 0, IA non-decreasing, every column in 0..n-1, columns ascending in
// each row): the cut's level scan indexes by column and stops at the first
// column at or past the row.
extern "C" int femgpu_ilu_block_cut(int n, const int *IA, const int *JA, int P, int *first, int cap)
{
	if (n <= 0 || !IA || !JA || !first) return FEMGPU_E_ARG;
	const int R = std::max(std::min(P, n), 1);
	if (cap < R + 1) return FEMGPU_E_ARG;
	if (IA[0] != 0) return FEMGPU_E_ARG;
	for (int i = 0; i < n; i++) {
		if (IA[i + 1] < IA[i]) return FEMGPU_E_ARG;
		for (int k = IA[i]; k < IA[i + 1]; k++) {
			if (JA[k] < 0 || JA[k] >= n) return FEMGPU_E_ARG;
			if (k > IA[i] && JA[k] <= JA[k - 1]) return FEMGPU_E_ARG;
		}
	}
	std::vector<int> f;
	(void)make_blocks(IA, JA, n, P, &f);
	if ((int)f.size() > cap) return FEMGPU_E_ARG;
	memcpy(first, f.data(), sizeof(int) * f.size());
	return (int)f.size() - 1;
}

// Host only (no device call): the chain-scan segmentation of one ILU(0)
// sweep of a CSR pattern with P blocks, as fg_ilu_prepare computes it.
extern "C" int femgpu_ilu_chain_segments(int n, const int *IA, const int *JA, int P, int lower, int *info,
                                         int *slot_row, int *slot_pred, int *lstart, int cap_slots, int cap_levels)
{
	if (n <= 0 || !IA || !JA || !info) return FEMGPU_E_ARG;
	if (IA[0] != 0) return FEMGPU_E_ARG;
	for (int i = 0; i < n; i++) {
		if (IA[i + 1] < IA[i]) return FEMGPU_E_ARG;
		for (int k = IA[i]; k < IA[i + 1]; k++)
			if (JA[k] < 0 || JA[k] >= n || (k > IA[i] && JA[k] <= JA[k - 1])) return FEMGPU_E_ARG;
	}
	Blocks B = make_blocks(IA, JA, n, P, nullptr);
	ChainLevels H = host_chain_levels(IA, JA, n, lower != 0, B);
	int deep = 0;
	for (size_t b = 0; b + 1 < H.clev.size(); b++) deep = std::max(deep, H.clev[b + 1] - H.clev[b]);
	info[0] = H.nlev;
	info[1] = deep;
	info[2] = H.rowlev_max;
	info[3] = H.maxw;
	if (slot_row || slot_pred || lstart) {
		if (cap_slots < H.nslot || cap_levels < H.nlev + 1) return FEMGPU_E_ARG;
		if (slot_row) memcpy(slot_row, H.slot_row.data(), sizeof(int) * H.nslot);
		if (slot_pred) memcpy(slot_pred, H.slot_pred.data(), sizeof(int) * H.nslot);
		if (lstart) memcpy(lstart, H.lstart.data(), sizeof(int) * (H.nlev + 1));
	}
	return H.nslot;
}

extern "C" int fg_ilu_prepare(femgpu_transport *t, const int *hIA, const int *hJA)
{
	int n = t->neq, rc, D, sb;
	fg_ilu_sweeps &S = t->sweeps;
	std::vector<int> first;
	Blocks B = make_blocks(hIA, hJA, n, t->o.ilu_blocks, &first);
	free(S.block_first);
	S.block_first = (int *)malloc(sizeof(int) * first.size());
	if (!S.block_first) return FEMGPU_E_NOMEM;
	memcpy(S.block_first, first.data(), sizeof(int) * first.size());
	S.nblocks = (int)first.size() - 1;
	std::vector<int> clo, cup;
	HostLevels Lo = host_levels(hIA, hJA, n, true, B, &clo), Up = host_levels(hIA, hJA, n, false, B, &cup);
	if ((rc = build_prog<double, true>(hIA, hJA, n, Up, nullptr, B, cup, S.up64))) return rc;
	if ((rc = build_prog<double, false>(hIA, hJA, n, Lo, &Up, B, clo, S.lo64))) return rc;
	if ((rc = build_prog<float, true>(hIA, hJA, n, Up, nullptr, B, cup, S.up32))) return rc;
	if ((rc = build_prog<float, false>(hIA, hJA, n, Lo, &Up, B, clo, S.lo32))) return rc;
	if ((rc = build_factor_prog(hIA, hJA, n, Lo, B, S))) return rc;
	S.fac2_ok = 0;
	if ((rc = build_factor_prog2(hIA, hJA, n, Lo, B, S))) return rc;
	S.chain = 0;
	S.ds = 0;
	size_t nb = (size_t)std::max(Lo.pstart[Lo.nlev], Up.pstart[Up.nlev]) + 64;
	if (sweep_chain()) {
		ChainLevels CL = host_chain_levels(hIA, hJA, n, true, B), CU = host_chain_levels(hIA, hJA, n, false, B);
		int deepL = 0, deepU = 0;
		for (size_t b = 0; b + 1 < CL.clev.size(); b++) deepL = std::max(deepL, CL.clev[b + 1] - CL.clev[b]);
		for (size_t b = 0; b + 1 < CU.clev.size(); b++) deepU = std::max(deepU, CU.clev[b + 1] - CU.clev[b]);
		// worth it only when the segments remove most of the levels
		if (4 * (deepL + deepU) <= 3 * (CL.rowlev_max + CU.rowlev_max)) {
			int r1 = build_prog_chain<double, true>(hIA, hJA, n, CU, nullptr, B, S.up64c);
			int r2 = r1 ? r1 : build_prog_chain<double, false>(hIA, hJA, n, CL, &CU, B, S.lo64c);
			int r3 = r2 ? r2 : build_prog_chain<float, true>(hIA, hJA, n, CU, nullptr, B, S.up32c);
			int r4 = r3 ? r3 : build_prog_chain<float, false>(hIA, hJA, n, CL, &CU, B, S.lo32c);
			if (r4 && r4 != FEMGPU_E_MESH) return r4;
			S.chain = r4 == 0;
			if (S.chain) {
				nb = std::max(nb, (size_t)std::max(CL.nslot, CU.nslot) + 64);
				const fg_sweep *cs[4] = { &S.lo64c, &S.up64c, &S.lo32c, &S.up32c };
				for (int i = 0; i < 4; i++) {
					rc = sweep_smem(*cs[i], i < 2 ? sizeof(double) : sizeof(float), &D, &sb);
					if (rc < 0) { S.chain = 0; break; }
				}
			}
			if (S.chain && sweep_ds()) {
				// the FP64 programs' bytes (codes and offsets are the same;
				// the refresh rewrites the values as double-single)
				const size_t bl = (size_t)S.lo64c.bytes + 16, bu = (size_t)S.up64c.bytes + 16;
				FG_TRY(cudaMalloc((void **)&S.prog_lo_ds, bl));
				FG_TRY(cudaMalloc((void **)&S.prog_up_ds, bu));
				FG_TRY(cudaMemcpy(S.prog_lo_ds, S.lo64c.prog, bl, cudaMemcpyDeviceToDevice));
				FG_TRY(cudaMemcpy(S.prog_up_ds, S.up64c.prog, bu, cudaMemcpyDeviceToDevice));
				FG_TRY(cudaMalloc((void **)&S.dpos, sizeof(int) * (size_t)n));
				k_inv_gather<<<fg_grid(n), FG_TPB, 0, t->stream>>>(S.lo64c.rows, S.lo64c.ppos, n, S.dpos);
				FG_TRY(cudaGetLastError());
				S.ds = 1;
			}
		}
	}
	FG_TRY(cudaMalloc((void **)&S.bl64, sizeof(double) * nb));
	FG_TRY(cudaMalloc((void **)&S.y64, sizeof(double) * nb));
	FG_TRY(cudaMalloc((void **)&S.bl32, sizeof(float) * nb));
	FG_TRY(cudaMalloc((void **)&S.y32, sizeof(float) * nb));
	FG_TRY(cudaMemset(S.bl64, 0, sizeof(double) * nb));
	FG_TRY(cudaMemset(S.y64, 0, sizeof(double) * nb));
	if (S.ds) {
		FG_TRY(cudaMalloc((void **)&S.o64, sizeof(double) * nb));
		FG_TRY(cudaMemset(S.o64, 0, sizeof(double) * nb));
	}
	FG_TRY(cudaMemset(S.bl32, 0, sizeof(float) * nb));
	FG_TRY(cudaMemset(S.y32, 0, sizeof(float) * nb));
	const fg_sweep *all[4] = { &S.lo64, &S.up64, &S.lo32, &S.up32 };
	for (int i = 0; i < 4; i++) {
		rc = sweep_smem(*all[i], i < 2 ? sizeof(double) : sizeof(float), &D, &sb);
		if (rc < 0) return rc;
	}
	return sweep_attrs();
}

// ILU(p): the matrix's values onto the filled pattern (fill entries zero).
__global__ void k_fill_scatter(const double *__restrict__ A, const int *__restrict__ map, int nnz, double *fA)
{
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) fA[map[k]] = A[k];
}

extern "C" int fg_ilu0_factor(femgpu_transport *t)
{
	cudaStream_t s = t->stream;
	fg_ilu_sweeps &S = t->sweeps;
	int P = S.lo64.nchunk, C = S.fac2_ok ? factor_cluster_size(P) : 0;
	const double *A = t->A;
	const int *IA = t->IA;
	if (S.fill) {
		FG_TRY(cudaMemsetAsync(S.fA, 0, sizeof(double) * ((size_t)S.fnnz + 1), s));
		k_fill_scatter<<<fg_grid(t->nnz), FG_TPB, 0, s>>>(t->A, S.fmap, t->nnz, S.fA);
		A = S.fA;
		IA = S.fIA;
	}
	if (C) {
		cudaLaunchConfig_t cfg = {};
		cudaLaunchAttribute at[1];
		at[0].id = cudaLaunchAttributeClusterDimension;
		at[0].val.clusterDim.x = (unsigned)C; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
		cfg.gridDim = dim3((unsigned)(C * P)); cfg.blockDim = dim3(FAC2_T); cfg.dynamicSmemBytes = FAC2_SMEM;
		cfg.stream = s; cfg.attrs = at; cfg.numAttrs = 1;
		FG_TRY(cudaLaunchKernelEx(&cfg, k_ilu0_factor_cluster, A, (const int *)S.lo64.rows,
		                          (const int *)S.lo64.lev_start, S.lo64.nlev, (const int *)S.lo64.chunk_lev,
		                          (const int4 *)S.fac2_hdr, (const int *)S.fac2, t->ilu.LU, t->ilu.Dinv,
		                          &t->st->err));
	} else {
		k_ilu0_factor_cta<<<S.lo64.nchunk, FAC_THREADS, 0, s>>>(IA, A, S.lo64.rows, S.lo64.lev_start,
		                                                       S.lo64.nlev, S.lo64.chunk_lev, S.fac_ptr,
		                                                       S.fac_prog, t->ilu.LU, t->ilu.Dinv, &t->st->err);
	}
	// the double-single chain programs (the FGMRES sweeps) take the new
	// values now, the others when an application first uses them
	S.stale = S.chain ? 0xFF : 0x0F;
	if (S.ds) {
		const fg_sweep &L = S.lo64c, &U = S.up64c;
		k_refresh<dsf><<<fg_grid(L.nval), FG_TPB, 0, s>>>(S.prog_lo_ds, L.val_off, L.val_src, L.nval, t->ilu.LU,
		                                                  t->ilu.Dinv);
		k_refresh<dsf><<<fg_grid(U.nval), FG_TPB, 0, s>>>(S.prog_up_ds, U.val_off, U.val_src, U.nval, t->ilu.LU,
		                                                  t->ilu.Dinv);
		k_chain_mult<dsf, false><<<fg_grid((long long)L.nslot), FG_TPB, 0, s>>>(S.prog_lo_ds, L.cs_voff, L.cs_src,
		                                                                      L.cs_row, L.nslot, t->ilu.LU,
		                                                                      t->ilu.Dinv);
		k_chain_mult<dsf, true><<<fg_grid((long long)U.nslot), FG_TPB, 0, s>>>(S.prog_up_ds, U.cs_voff, U.cs_src,
		                                                                     U.cs_row, U.nslot, t->ilu.LU,
		                                                                     t->ilu.Dinv);
	}
	return (int)cudaGetLastError();
}

// Program pair i0, i0 + 1 (0: lo64/up64, 2: lo32/up32, 4: lo64c/up64c,
// 6: lo32c/up32c) given the current factor's values (and, for the chain
// programs, their scan multipliers) if the factorisation left it stale; on
// the context's stream, ahead of the application that uses it.
static int refresh_pair(femgpu_transport *t, int i0)
{
	fg_ilu_sweeps &S = t->sweeps;
	cudaStream_t s = t->stream;
	fg_sweep *pr[8] = { &S.lo64, &S.up64, &S.lo32, &S.up32, &S.lo64c, &S.up64c, &S.lo32c, &S.up32c };
	for (int i = i0; i < i0 + 2; i++) {
		if (!(S.stale & (1 << i))) continue;
		const fg_sweep &c = *pr[i];
		const bool f64 = (i & 2) == 0, up = (i & 1) != 0;
		const int g = fg_grid(c.nval);
		if (f64) k_refresh<double><<<g, FG_TPB, 0, s>>>(c.prog, c.val_off, c.val_src, c.nval, t->ilu.LU, t->ilu.Dinv);
		else k_refresh<float><<<g, FG_TPB, 0, s>>>(c.prog, c.val_off, c.val_src, c.nval, t->ilu.LU, t->ilu.Dinv);
		if (i >= 4) {
			const int gc = fg_grid((long long)c.nslot);
			if (f64 && up) k_chain_mult<double, true><<<gc, FG_TPB, 0, s>>>(c.prog, c.cs_voff, c.cs_src, c.cs_row,
			                                                               c.nslot, t->ilu.LU, t->ilu.Dinv);
			else if (f64) k_chain_mult<double, false><<<gc, FG_TPB, 0, s>>>(c.prog, c.cs_voff, c.cs_src, c.cs_row,
			                                                               c.nslot, t->ilu.LU, t->ilu.Dinv);
			else if (up) k_chain_mult<float, true><<<gc, FG_TPB, 0, s>>>(c.prog, c.cs_voff, c.cs_src, c.cs_row,
			                                                            c.nslot, t->ilu.LU, t->ilu.Dinv);
			else k_chain_mult<float, false><<<gc, FG_TPB, 0, s>>>(c.prog, c.cs_voff, c.cs_src, c.cs_row,
			                                                     c.nslot, t->ilu.LU, t->ilu.Dinv);
		}
		S.stale &= ~(1 << i);
	}
	return (int)cudaGetLastError();
}

// The dependency-wait bound of the sweep warps: the context's override
// (sweep_wait1 = bound + 1) or SW_WAIT_LIMIT.  Stage waits and the drain after
// a timeout always keep SW_WAIT_LIMIT, so no bulk copy outlives its block.
static int sweep_wait(const femgpu_transport *t)
{
	return t->sweep_wait1 > 0 ? t->sweep_wait1 - 1 : SW_WAIT_LIMIT;
}

template <typename T, typename TI, typename TO>
static int apply_t(femgpu_transport *t, const fg_sweep &lo, const fg_sweep &up, T *bl, T *y,
                   const TI *p, TO *z, const int *active, bool fma)
{
	cudaStream_t s = t->stream;
	int n = t->neq, D, sb, bytes;
	k_perm_in<T, TI><<<fg_grid(n), FG_TPB, 0, s>>>(p, lo.rows, lo.ppos, n, bl);
	SweepArgs a;
	a.err = &t->st->err;
	a.active = active;
	a.wait = sweep_wait(t);
	bytes = sweep_smem(lo, sizeof(T), &D, &sb);
	if (bytes < 0) return bytes;
	a.prog = lo.prog; a.blk_off = lo.blk_off; a.sb_in = lo.sb_in; a.sb_inb = lo.sb_inb;
	a.nlev = lo.nlev; a.nsb = lo.nsb; a.D = D; a.stage_bytes = sb;
	a.chunk_sb = lo.chunk_sb; a.chunk_lev = lo.chunk_lev; a.bvo = lo.bvo; a.cmax = lo.cmax; a.skew = lo.skew;
	launch_sweep<T, false>(a, lo.rw, lo.df, lo.nchunk, bytes, s, bl, y, fma, lo.cs);
	bytes = sweep_smem(up, sizeof(T), &D, &sb);
	if (bytes < 0) return bytes;
	a.prog = up.prog; a.blk_off = up.blk_off; a.sb_in = up.sb_in; a.sb_inb = up.sb_inb;
	a.nlev = up.nlev; a.nsb = up.nsb; a.D = D; a.stage_bytes = sb;
	a.chunk_sb = up.chunk_sb; a.chunk_lev = up.chunk_lev; a.bvo = up.bvo; a.cmax = up.cmax; a.skew = up.skew;
	launch_sweep<T, true>(a, up.rw, up.df, up.nchunk, bytes, s, y, (T *)z, fma, up.cs);
	return (int)cudaGetLastError();
}

// FGMRES sweeps (fused arithmetic) and FP32 sweeps take the chain-scan
// programs when the factor has them; the reference's left-preconditioned
// GMRES keeps the row-by-row programs, bit-identical to its ILUp_precond.
// The double-single chain sweeps: gather into double-single slots, the
// forward and backward chain-scan programs with double-single values, the
// backward output (natural order, in the gather buffer) back to FP64.
static int sweeps_ds(femgpu_transport *t, const int *active);
static int apply_ds(femgpu_transport *t, const double *p, const dsf *p_ds, double *z, const int *active)
{
	fg_ilu_sweeps &S = t->sweeps;
	const fg_sweep &lo = S.lo64c;
	cudaStream_t s = t->stream;
	const int n = t->neq;
	dsf *bl = (dsf *)S.bl64;
	if (p_ds) k_perm_in_dsds<<<fg_grid(n), FG_TPB, 0, s>>>(p_ds, lo.rows, lo.ppos, n, bl, active);
	else k_perm_in_ds<<<fg_grid(n), FG_TPB, 0, s>>>(p, lo.rows, lo.ppos, n, bl);
	const int rc = sweeps_ds(t, active);
	if (rc) return rc;
	k_ds_to_double<<<fg_grid(n), FG_TPB, 0, s>>>((const dsf *)S.o64, n, z, active);
	return (int)cudaGetLastError();
}

// The two double-single chain sweeps on the gathered input in the gather
// buffer; the backward sweep writes its output, in natural order, to o64 (not
// back into the gather buffer: in the one-launch form a block's backward sweep
// may run while another block's forward sweep still reads its input there).
static int sweeps_ds(femgpu_transport *t, const int *active)
{
	fg_ilu_sweeps &S = t->sweeps;
	const fg_sweep &lo = S.lo64c, &up = S.up64c;
	cudaStream_t s = t->stream;
	int D, sb, bytes;
	dsf *bl = (dsf *)S.bl64, *y = (dsf *)S.y64, *o = (dsf *)S.o64;
	SweepArgs a;
	a.err = &t->st->err;
	a.active = active;
	a.wait = sweep_wait(t);
	bytes = sweep_smem(lo, sizeof(dsf), &D, &sb);
	if (bytes < 0) return bytes;
	a.prog = S.prog_lo_ds; a.blk_off = lo.blk_off; a.sb_in = lo.sb_in; a.sb_inb = lo.sb_inb;
	a.nlev = lo.nlev; a.nsb = lo.nsb; a.D = D; a.stage_bytes = sb;
	a.chunk_sb = lo.chunk_sb; a.chunk_lev = lo.chunk_lev; a.bvo = lo.bvo; a.cmax = lo.cmax; a.skew = lo.skew;
	SweepArgs b = a;
	const int bytes_lo = bytes;
	bytes = sweep_smem(up, sizeof(dsf), &D, &sb);
	if (bytes < 0) return bytes;
	b.prog = S.prog_up_ds; b.blk_off = up.blk_off; b.sb_in = up.sb_in; b.sb_inb = up.sb_inb;
	b.nlev = up.nlev; b.nsb = up.nsb; b.D = D; b.stage_bytes = sb;
	b.chunk_sb = up.chunk_sb; b.chunk_lev = up.chunk_lev; b.bvo = up.bvo; b.cmax = up.cmax; b.skew = up.skew;
	// one launch for both sweeps unless FEMGPU_SWEEP_FB=0
	const char *e = getenv("FEMGPU_SWEEP_FB");
	if (!(e && e[0] == '0') && lo.rw == up.rw && lo.nchunk == up.nchunk &&
	    launch_cs_fb(a, b, lo.rw, lo.nchunk, bytes_lo > bytes ? bytes_lo : bytes, s, bl, y, o))
		return (int)cudaGetLastError();
	launch_cs<dsf, false>(a, lo.rw, lo.nchunk, bytes_lo, s, bl, y);
	launch_cs<dsf, true>(b, up.rw, up.nchunk, bytes, s, y, o);
	return (int)cudaGetLastError();
}

extern "C" int fg_ilu0_sweeps_gathered(femgpu_transport *t, const int *active)
{
	if (!t->sweeps.ds) return FEMGPU_E_ARG;
	return sweeps_ds(t, active);
}

extern "C" int fg_ilu0_apply64(femgpu_transport *t, const double *p, double *z, const int *active)
{
	fg_ilu_sweeps &S = t->sweeps;
	const bool fma = t->o.solver == FEMGPU_FGMRES;
	if (fma && S.ds) return apply_ds(t, p, NULL, z, active);
	const int pair = (fma && S.chain) ? 4 : 0;
	const int rc = refresh_pair(t, pair);
	if (rc) return rc;
	if (pair) return apply_t<double, double, double>(t, S.lo64c, S.up64c, S.bl64, S.y64, p, z, active, true);
	return apply_t<double, double, double>(t, S.lo64, S.up64, S.bl64, S.y64, p, z, active, fma);
}

// The double-single sweeps with a double-single input (the Krylov basis of
// the double-single Arnoldi); available when fg_ilu0_ds_ready says so.
extern "C" int fg_ilu0_ds_ready(const femgpu_transport *t)
{
	return t->sweeps.ds ? 1 : 0;
}

extern "C" int fg_ilu0_apply64_dsin(femgpu_transport *t, const void *p, double *z, const int *active)
{
	if (!t->sweeps.ds) return FEMGPU_E_NOT_BUILT;
	return apply_ds(t, NULL, (const dsf *)p, z, active);
}

extern "C" int fg_ilu0_apply32(femgpu_transport *t, const double *p, float *z, const int *active)
{
	fg_ilu_sweeps &S = t->sweeps;
	const int rc = refresh_pair(t, S.chain ? 6 : 2);
	if (rc) return rc;
	if (S.chain) return apply_t<float, double, float>(t, S.lo32c, S.up32c, S.bl32, S.y32, p, z, active, false);
	return apply_t<float, double, float>(t, S.lo32, S.up32, S.bl32, S.y32, p, z, active, false);
}

extern "C" void fg_ilu_free(femgpu_transport *t)
{
	fg_ilu_sweeps &S = t->sweeps;
	fg_sweep *all[8] = { &S.lo64, &S.up64, &S.lo32, &S.up32, &S.lo64c, &S.up64c, &S.lo32c, &S.up32c };
	for (int i = 0; i < 8; i++) {
		void *p[] = { all[i]->prog, all[i]->blk_off, all[i]->sb_in, all[i]->sb_inb, all[i]->lev_start,
		              all[i]->rows, all[i]->ppos, all[i]->val_off, all[i]->val_src, all[i]->chunk_sb,
		              all[i]->chunk_lev, all[i]->cs_voff, all[i]->cs_src, all[i]->cs_row };
		for (void *q : p) if (q) cudaFree(q);
		memset(all[i], 0, sizeof(fg_sweep));
	}
	S.chain = 0;
	void *v[] = { S.bl64, S.y64, S.o64, S.bl32, S.y32, S.fac_ptr, S.fac_prog, S.fac2_hdr, S.fac2, S.fIA, S.fJA, S.fmap,
	              S.fA };
	for (void *q : v) if (q) cudaFree(q);
	S.bl64 = S.y64 = S.o64 = nullptr;
	S.bl32 = S.y32 = nullptr;
	S.fIA = S.fJA = S.fmap = nullptr;
	S.fA = nullptr;
	S.fill = 0;
	if (S.dpos) cudaFree(S.dpos);
	S.dpos = nullptr;
	if (S.prog_lo_ds) cudaFree(S.prog_lo_ds);
	if (S.prog_up_ds) cudaFree(S.prog_up_ds);
	S.prog_lo_ds = S.prog_up_ds = nullptr;
	S.ds = 0;
	free(S.block_first);
	S.block_first = nullptr;
	S.nblocks = 0;
}
