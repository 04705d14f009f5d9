// V-cycle of the double-pairwise AMG preconditioner
// (00_CommonFiles/Solvers_and_Preconditioners/CSR/AMG/amg_dpa.c:485-506).
//
// Per smoothed level l (even levels; odd levels are only the intermediate of
// the double pairwise step): SOR_relax (amg_solvers.c:3-17) forward nr times,
// residual r = f - A u (amg_util.c:44-48 with mat_vec, amg_matrix.c:276-282),
// restriction twice (dpa_fine2coarse, amg_dpa.c:394-401), zero coarse u; at
// the coarsest level SOR forward nr + reverse nr times; on the way up
// prolongation twice (dpa_coarse2fine_pure then dpa_coarse2fine,
// amg_dpa.c:403-422) and SOR_relax_rev (amg_solvers.c:19-33) nr times.
//
// GB300 mapping.  The Gauss-Seidel sweeps are level scheduled: a row is
// updated after every lower (forward) or higher (reverse) neighbour, so each
// row sees exactly the values the sequential sweep sees and the result is the
// reference's bit for bit (this translation unit is compiled without FMA
// contraction; sums run in CSR order).  Narrow runs of levels go to one
// 1024-thread block that walks them with __syncthreads between levels (the
// sweep is latency bound: one launch per sweep instead of one per level);
// wide levels get a grid each.  The residual and both restrictions are one
// kernel (one thread per level-(l+2) row recomputes its <= 4 fine residual
// rows, r is never stored), and both prolongations are one kernel through
// the composite aggregate map.
#include <cuda_runtime.h>

#include "fg_amg.h"

namespace {

constexpr int kNarrowThreads = 1024;
constexpr int kThreads = 256;

__device__ __forceinline__ bool skip(const int *active) { return active && !*active; }

__device__ __forceinline__ void sor_row(const int *__restrict__ ptr, const int *__restrict__ col,
                                        const double *__restrict__ val, const double *__restrict__ diag,
                                        const double *__restrict__ f, double *u, int i, double omega)
{
	double sum = 0.0;
	for (int k = ptr[i]; k < ptr[i + 1]; k++) {
		int c = col[k];
		if (c != i) sum += val[k] * u[c];
	}
	u[i] += omega * ((f[i] - sum) / diag[i] - u[i]);
}

// levels [l0, l1) of a schedule, `sweeps` times, by one block
__global__ void __launch_bounds__(kNarrowThreads)
k_sor_narrow(const int *__restrict__ ptr, const int *__restrict__ col, const double *__restrict__ val,
             const double *__restrict__ diag, const double *__restrict__ f, double *u,
             const int *__restrict__ rows, const int *__restrict__ lev, int l0, int l1, int sweeps,
             double omega, const int *active)
{
	if (skip(active)) return;
	for (int s = 0; s < sweeps; s++)
		for (int l = l0; l < l1; l++) {
			int b = lev[l], e = lev[l + 1];
			for (int t = b + (int)threadIdx.x; t < e; t += kNarrowThreads)
				sor_row(ptr, col, val, diag, f, u, rows[t], omega);
			__syncthreads();
		}
}

// one wide level
__global__ void k_sor_level(const int *__restrict__ ptr, const int *__restrict__ col,
                            const double *__restrict__ val, const double *__restrict__ diag,
                            const double *__restrict__ f, double *u, const int *__restrict__ rows,
                            int b, int e, double omega, const int *active)
{
	if (skip(active)) return;
	int t = b + (int)(blockIdx.x * blockDim.x + threadIdx.x);
	if (t < e) sor_row(ptr, col, val, diag, f, u, rows[t], omega);
}

__device__ __forceinline__ double resid_row(const int *__restrict__ ptr, const int *__restrict__ col,
                                            const double *__restrict__ val, const double *__restrict__ f,
                                            const double *__restrict__ u, int i)
{
	double p = 0.0;
	for (int k = ptr[i]; k < ptr[i + 1]; k++) p += val[k] * u[col[k]];
	return f[i] - p;
}

// f2[k] = (r[a] + r[b]) + (r[c] + r[d]) with absent members dropped, r = f - A u
// on level l; u2[k] = 0.
__global__ void k_restrict2(const int *__restrict__ ptr, const int *__restrict__ col,
                            const double *__restrict__ val, const double *__restrict__ f,
                            const double *__restrict__ u, const int4 *__restrict__ quad, int nc2,
                            double *__restrict__ f2, double *__restrict__ u2, const int *active)
{
	if (skip(active)) return;
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nc2) return;
	int4 q = quad[k];
	double s1 = resid_row(ptr, col, val, f, u, q.x);
	if (q.y >= 0) s1 = s1 + resid_row(ptr, col, val, f, u, q.y);
	if (q.z >= 0) {
		double s2 = resid_row(ptr, col, val, f, u, q.z);
		if (q.w >= 0) s2 = s2 + resid_row(ptr, col, val, f, u, q.w);
		s1 = s1 + s2;
	}
	f2[k] = s1;
	u2[k] = 0.0;
}

// u[i] += u2[agg2[i]]
__global__ void k_prolong2(const int *__restrict__ agg2, const double *__restrict__ u2, double *__restrict__ u,
                           int n, const int *active)
{
	if (skip(active)) return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) u[i] += u2[agg2[i]];
}

__global__ void k_copy_or_zero(const double *__restrict__ src, double *__restrict__ dst, int n, const int *active)
{
	if (skip(active)) return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) dst[i] = src ? src[i] : 0.0;
}

inline unsigned blocks(int n) { return (unsigned)((n + kThreads - 1) / kThreads); }

int sor(const femgpu_amg *g, const fg_amg_level *L, const double *f, double *u, int reverse, int sweeps,
        const int *active)
{
	const int *rows = reverse ? L->bw_rows : L->fw_rows;
	const int *lev = reverse ? L->bw_lev : L->fw_lev;
	const int *hlev = reverse ? L->h_bw_lev : L->h_fw_lev;
	const fg_amg_seg *seg = reverse ? L->bw_seg : L->fw_seg;
	int nseg = reverse ? L->bw_nseg : L->fw_nseg;
	if (nseg == 1 && !seg[0].wide) {
		k_sor_narrow<<<1, kNarrowThreads, 0, g->stream>>>(L->ptr, L->col, L->val, L->diag, f, u, rows, lev,
		                                                   seg[0].l0, seg[0].l1, sweeps, g->omega, active);
		return (int)cudaGetLastError();
	}
	for (int s = 0; s < sweeps; s++)
		for (int q = 0; q < nseg; q++) {
			if (seg[q].wide) {
				int b = hlev[seg[q].l0], e = hlev[seg[q].l0 + 1];
				k_sor_level<<<blocks(e - b), kThreads, 0, g->stream>>>(L->ptr, L->col, L->val, L->diag, f, u,
				                                                        rows, b, e, g->omega, active);
			} else {
				k_sor_narrow<<<1, kNarrowThreads, 0, g->stream>>>(L->ptr, L->col, L->val, L->diag, f, u, rows,
				                                                   lev, seg[q].l0, seg[q].l1, 1, g->omega, active);
			}
		}
	return (int)cudaGetLastError();
}

}  // namespace

extern "C" int fg_amg_vcycle(femgpu_amg *g, const double *q, double *z, const int *active)
{
	int top = g->nlevels - 1, l, rc;
	fg_amg_level *lv = g->lv;
	int n0 = lv[0].n;
	if (q == z) {
		k_copy_or_zero<<<blocks(n0), kThreads, 0, g->stream>>>(q, g->qcopy, n0, active);
		q = g->qcopy;
	}
	lv[0].f = (double *)q;           // level 0 works on the caller's vectors
	lv[0].u = z;
	k_copy_or_zero<<<blocks(n0), kThreads, 0, g->stream>>>(nullptr, z, n0, active);
	for (l = 0; l < top; l += 2) {
		fg_amg_level *L = &lv[l], *C = &lv[l + 2];
		if ((rc = sor(g, L, L->f, L->u, 0, g->nr, active))) return rc;
		k_restrict2<<<blocks(L->nc2), kThreads, 0, g->stream>>>(L->ptr, L->col, L->val, L->f, L->u, L->quad,
		                                                          L->nc2, C->f, C->u, active);
	}
	if ((rc = sor(g, &lv[top], lv[top].f, lv[top].u, 0, g->nr, active))) return rc;
	if ((rc = sor(g, &lv[top], lv[top].f, lv[top].u, 1, g->nr, active))) return rc;
	for (l = top; l > 0; l -= 2) {
		fg_amg_level *F = &lv[l - 2];
		k_prolong2<<<blocks(F->n), kThreads, 0, g->stream>>>(F->agg2, lv[l].u, F->u, F->n, active);
		if ((rc = sor(g, F, F->f, F->u, 1, g->nr, active))) return rc;
	}
	lv[0].f = nullptr;
	lv[0].u = nullptr;
	return (int)cudaGetLastError();
}
