// Storage patterns built on the device: element incidence lists, the CSR
// pattern of csr_Initialization.c:18-123 (rows of equations, ascending unique
// columns, CSR_by_Element slot map) and the edge structure of
// ede_Initialization.c:16-170.  Every list is sorted per row after an
// atomics-based fill, so the result never depends on scheduling order and is
// bit-identical to the reference's linked-list construction.
#include "fg_common.cuh"
#include <stdlib.h>

#define FG_MAXROW 64      // max distinct columns of one row (P1 triangles: ~7)

// ---------------------------------------------------------------- scan ----
__global__ void k_scan_block(const int *in, int *out, int n1, int *bsum)
{
	__shared__ int ws[32];
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int v = (i < n1 - 1) ? in[i] : 0;          // element n (the total slot) is 0
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	int x = v;
	#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		int y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= o) x += y;
	}
	if (lane == 31) ws[wid] = x;
	__syncthreads();
	if (wid == 0) {
		int nw = blockDim.x >> 5;
		int s = (lane < nw) ? ws[lane] : 0;
		#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			int y = __shfl_up_sync(0xffffffffu, s, o);
			if (lane >= o) s += y;
		}
		ws[lane] = s;
	}
	__syncthreads();
	int excl = x - v + (wid > 0 ? ws[wid - 1] : 0);
	if (i < n1) out[i] = excl;
	if (threadIdx.x == blockDim.x - 1) bsum[blockIdx.x] = excl + v;
}

__global__ void k_scan_add(int *out, int n1, const int *boff)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n1) out[i] += boff[blockIdx.x];
}

int fg_scan(const int *in, int *out, int n, cudaStream_t s)
{
	const int B = 1024;
	int n1 = n + 1, nb = (n1 + B - 1) / B;
	int *bsum = nullptr;
	FG_TRY(cudaMalloc(&bsum, sizeof(int) * (nb + 1)));
	k_scan_block<<<nb, B, 0, s>>>(in, out, n1, bsum);
	if (nb > 1) {
		int rc = fg_scan(bsum, bsum, nb, s);
		if (rc) { cudaFree(bsum); return rc; }
		k_scan_add<<<nb, B, 0, s>>>(out, n1, bsum);
	}
	cudaError_t e = cudaGetLastError();
	cudaStreamSynchronize(s);
	cudaFree(bsum);
	return (int)e;
}

// ------------------------------------------------------- inverted maps ----
__global__ void k_inv_count(const int *target, int stride, int m, int T, int *cnt)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
		int t = target[(long long)i * stride];
		if (t >= 0 && t < T) atomicAdd(&cnt[t], 1);
	}
}

__global__ void k_inv_fill(const int *target, int stride, int m, int T, const int *ptr,
                           int *cur, int *list)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
		int t = target[(long long)i * stride];
		if (t >= 0 && t < T) list[ptr[t] + atomicAdd(&cur[t], 1)] = i;
	}
}

__global__ void k_sort_lists(const int *ptr, int *list, int T)
{
	for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
		int b = ptr[t], e = ptr[t + 1];
		for (int i = b + 1; i < e; i++) {
			int v = list[i], j = i - 1;
			while (j >= b && list[j] > v) { list[j + 1] = list[j]; j--; }
			list[j + 1] = v;
		}
	}
}

int fg_invert_map(const int *target, int stride, int m, int T, int **ptr, int **list,
                  cudaStream_t s)
{
	int *cnt = nullptr, total = 0;
	FG_TRY(cudaMalloc(&cnt, sizeof(int) * (T + 1)));
	FG_TRY(cudaMalloc(ptr, sizeof(int) * (T + 1)));
	FG_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (T + 1), s));
	k_inv_count<<<fg_grid(m), FG_TPB, 0, s>>>(target, stride, m, T, cnt);
	int rc = fg_scan(cnt, *ptr, T, s);
	if (rc) return rc;
	FG_TRY(cudaMemcpy(&total, *ptr + T, sizeof(int), cudaMemcpyDeviceToHost));
	FG_TRY(cudaMalloc(list, sizeof(int) * (total > 0 ? total : 1)));
	FG_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (T + 1), s));
	k_inv_fill<<<fg_grid(m), FG_TPB, 0, s>>>(target, stride, m, T, *ptr, cnt, *list);
	k_sort_lists<<<fg_grid(T), FG_TPB, 0, s>>>(*ptr, *list, T);
	FG_TRY(cudaGetLastError());
	FG_TRY(cudaStreamSynchronize(s));
	cudaFree(cnt);
	return 0;
}

// ------------------------------------------------------- numbering ------
// Fill_LM.c:7-19: the equation of each element vertex, neq for prescribed.
__global__ void k_lm(const int *vert, const int *node_type, const int *node_id, int nel3,
                     int neq, int *lm)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nel3; i += gridDim.x * blockDim.x) {
		int v = vert[i];
		lm[i] = (node_type[v] >= 1) ? node_id[v] : neq;
	}
}

extern "C" int fg_compute_lm(femgpu_transport *t)
{
	k_lm<<<fg_grid(3LL * t->nel), FG_TPB, 0, t->stream>>>(t->vert, t->node_type, t->node_id,
	                                                      3 * t->nel, t->neq, t->lm);
	return (int)cudaGetLastError();
}

extern "C" int fg_build_incidence(femgpu_transport *t)
{
	if (t->ri_ptr) { cudaFree(t->ri_ptr); t->ri_ptr = nullptr; }
	if (t->ri) { cudaFree(t->ri); t->ri = nullptr; }
	return fg_invert_map(t->lm, 1, 3 * t->nel, t->neq, &t->ri_ptr, &t->ri, t->stream);
}

// Insert v into the sorted unique array a[0..*m); returns 0 on overflow.
__device__ __forceinline__ int ins_sorted(int *a, int *m, int v)
{
	int j = *m;
	for (int q = 0; q < *m; q++) if (a[q] == v) return 1;
	if (*m >= FG_MAXROW) return 0;
	while (j > 0 && a[j - 1] > v) { a[j] = a[j - 1]; j--; }
	a[j] = v;
	(*m)++;
	return 1;
}

// ------------------------------------------------------------- CSR -------
// Row I: every unknown equation sharing an element with I (csr_Initialization
// .c:24-53), ascending (csr_List_insertA keeps its lists sorted).
__global__ void k_csr_rows(const int *ri_ptr, const int *ri, const int *lm, int neq,
                           int *rowlen, const int *IA, int *JA, int *diag, int *err)
{
	int row[FG_MAXROW];
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x) {
		int m = 0, ok = 1;
		for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
			int e = ri[q] / 3;
			for (int b = 0; b < 3; b++) {
				int J = lm[3 * e + b];
				if (J != neq) ok &= ins_sorted(row, &m, J);
			}
		}
		if (!ok) fg_set_err(err, FEMGPU_E_MESH);
		if (rowlen) rowlen[I] = m;
		if (JA) {
			int base = IA[I];
			for (int q = 0; q < m; q++) {
				JA[base + q] = row[q];
				if (row[q] == I) diag[I] = base + q;
			}
		}
	}
}

__device__ __forceinline__ int bsearch_row(const int *JA, int lo, int hi, int col)
{
	while (lo < hi) {
		int mid = (lo + hi) >> 1;
		if (__ldg(&JA[mid]) < col) lo = mid + 1; else hi = mid;
	}
	return lo;
}

// CSR_by_Element (csr_Initialization.c:71-123): slot 3a+b of element e holds
// the position of (lm[a], lm[b]), or nnz when either is prescribed.
__global__ void k_csr_sbe(const int *lm, const int *IA, const int *JA, int nel, int neq, int nnz,
                          int *sbe)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		int l[3] = { lm[3 * e], lm[3 * e + 1], lm[3 * e + 2] };
		for (int a = 0; a < 3; a++)
			for (int b = 0; b < 3; b++) {
				int I = l[a], J = l[b];
				sbe[9 * e + 3 * a + b] = (I == neq || J == neq) ? nnz
					: bsearch_row(JA, IA[I], IA[I + 1], J);
			}
	}
}

extern "C" int fg_build_csr(femgpu_transport *t)
{
	cudaStream_t s = t->stream;
	int neq = t->neq, *rowlen = nullptr, *err = &t->st->err, herr = 0;
	if (t->IA) cudaFree(t->IA);
	if (t->JA) cudaFree(t->JA);
	if (t->sbe) cudaFree(t->sbe);
	if (t->diag) cudaFree(t->diag);
	t->IA = t->JA = t->sbe = t->diag = nullptr;
	FG_TRY(cudaMalloc(&rowlen, sizeof(int) * (neq + 1)));
	FG_TRY(cudaMalloc(&t->IA, sizeof(int) * (neq + 1)));
	FG_TRY(cudaMalloc(&t->diag, sizeof(int) * (neq + 1)));
	k_csr_rows<<<fg_grid(neq, 128), 128, 0, s>>>(t->ri_ptr, t->ri, t->lm, neq, rowlen, nullptr,
	                                             nullptr, nullptr, err);
	int rc = fg_scan(rowlen, t->IA, neq, s);
	if (rc) return rc;
	FG_TRY(cudaMemcpy(&t->nnz, t->IA + neq, sizeof(int), cudaMemcpyDeviceToHost));
	FG_TRY(cudaMalloc(&t->JA, sizeof(int) * (t->nnz + 1)));
	FG_TRY(cudaMalloc(&t->sbe, sizeof(int) * 9LL * t->nel));
	k_csr_rows<<<fg_grid(neq, 128), 128, 0, s>>>(t->ri_ptr, t->ri, t->lm, neq, nullptr, t->IA,
	                                             t->JA, t->diag, err);
	k_csr_sbe<<<fg_grid(t->nel), FG_TPB, 0, s>>>(t->lm, t->IA, t->JA, t->nel, neq, t->nnz, t->sbe);
	FG_TRY(cudaGetLastError());
	FG_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
	FG_TRY(cudaStreamSynchronize(s));
	cudaFree(rowlen);
	return herr ? herr : 0;
}

// ------------------------------------------------------- block CSR -----
// The same CSR set-up for M equations per element (the Navier-Stokes
// csr_Initialization.c:18-85: rows of lm[e][0..M), the diagonal included,
// sorted unique; CSR_by_Element slot M*a+b of element e, or nnz when either
// equation is prescribed).  Incidence codes e*M + a.
template <int M>
__global__ void k_csr_rows_m(const int *ri_ptr, const int *ri, const int *lm, int neq, int *rowlen, const int *IA,
                             int *JA, int *err)
{
	int row[FG_MAXROW];
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x) {
		int m = 0, ok = 1;
		for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
			int e = ri[q] / M;
			for (int b = 0; b < M; b++) {
				int J = lm[M * e + b];
				if (J != neq) ok &= ins_sorted(row, &m, J);
			}
		}
		if (!ok) fg_set_err(err, FEMGPU_E_MESH);
		if (rowlen) rowlen[I] = m;
		if (JA) {
			int base = IA[I];
			for (int q = 0; q < m; q++) JA[base + q] = row[q];
		}
	}
}

template <int M>
__global__ void k_csr_sbe_m(const int *lm, const int *IA, const int *JA, int nel, int neq, int nnz, int *sbe)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x)
		for (int a = 0; a < M; a++)
			for (int b = 0; b < M; b++) {
				int I = lm[M * e + a], J = lm[M * e + b];
				sbe[(long long)M * M * e + M * a + b] = (I == neq || J == neq) ? nnz
					: bsearch_row(JA, IA[I], IA[I + 1], J);
			}
}

// csr_assembly.c:3-19 per row: each slot sums its elements' entries in
// ascending element order (the reference's += over elements), AA[nnz] = 0.
template <int M>
__global__ void k_assemble_csr_m(int neq, int nnz, const int *IA, const int *sbe, const int *ri_ptr, const int *ri,
                                 const double *Ae, double *AA)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x) {
		for (int k = IA[I]; k < IA[I + 1]; k++) AA[k] = 0.0;
		for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
			int code = __ldg(&ri[q]), e = code / M, a = code - e * M;
			const int *sl = sbe + (long long)M * M * e + M * a;
			const double *row = Ae + (long long)M * M * e + M * a;
			for (int b = 0; b < M; b++) {
				int pos = __ldg(&sl[b]);
				if (pos < nnz) AA[pos] = AA[pos] + __ldg(&row[b]);
			}
		}
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) AA[nnz] = 0.0;
}

// M = 9 (Navier-Stokes, 3 dofs per node) or 12 (Euler, 4 dofs per node;
// 03_Euler_Equations/2D/01_CommonFiles/csr_Initialization.c is the same
// algorithm over 12 equations per element).
template <int M>
static int build_csr_m(int nel, int neq, const int *ri_ptr, const int *ri, const int *lm, cudaStream_t s, int *err,
                       int **IA, int **JA, int **sbe, int *nnz, int *rowlen)
{
	k_csr_rows_m<M><<<fg_grid(neq, 128), 128, 0, s>>>(ri_ptr, ri, lm, neq, rowlen, nullptr, nullptr, err);
	int rc = fg_scan(rowlen, *IA, neq, s);
	if (rc) return rc;
	FG_TRY(cudaMemcpy(nnz, *IA + neq, sizeof(int), cudaMemcpyDeviceToHost));
	FG_TRY(cudaMalloc(JA, sizeof(int) * ((size_t)*nnz + 1)));
	FG_TRY(cudaMalloc(sbe, sizeof(int) * M * M * (size_t)nel));
	k_csr_rows_m<M><<<fg_grid(neq, 128), 128, 0, s>>>(ri_ptr, ri, lm, neq, nullptr, *IA, *JA, err);
	k_csr_sbe_m<M><<<fg_grid(nel), FG_TPB, 0, s>>>(lm, *IA, *JA, nel, neq, *nnz, *sbe);
	return 0;
}

extern "C" int fg_build_csr_m(int M, int nel, int neq, const int *ri_ptr, const int *ri, const int *lm,
                              cudaStream_t s, int *err, int **IA, int **JA, int **sbe, int *nnz)
{
	int *rowlen = nullptr, herr = 0, rc;
	if (M != 9 && M != 12) return FEMGPU_E_ARG;
	FG_TRY(cudaMalloc(&rowlen, sizeof(int) * (neq + 1)));
	FG_TRY(cudaMalloc(IA, sizeof(int) * (neq + 1)));
	rc = M == 9 ? build_csr_m<9>(nel, neq, ri_ptr, ri, lm, s, err, IA, JA, sbe, nnz, rowlen)
	            : build_csr_m<12>(nel, neq, ri_ptr, ri, lm, s, err, IA, JA, sbe, nnz, rowlen);
	if (rc) { cudaFree(rowlen); return rc; }
	FG_TRY(cudaGetLastError());
	FG_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
	FG_TRY(cudaStreamSynchronize(s));
	cudaFree(rowlen);
	return herr ? herr : 0;
}

extern "C" int fg_assemble_csr_m(int M, int neq, int nnz, const int *IA, const int *sbe, const int *ri_ptr,
                                 const int *ri, const double *Ae, double *AA, cudaStream_t s)
{
	if (M == 9) k_assemble_csr_m<9><<<fg_grid(neq, 128, 32), 128, 0, s>>>(neq, nnz, IA, sbe, ri_ptr, ri, Ae, AA);
	else if (M == 12) k_assemble_csr_m<12><<<fg_grid(neq, 128, 32), 128, 0, s>>>(neq, nnz, IA, sbe, ri_ptr, ri, Ae, AA);
	else return FEMGPU_E_ARG;
	return (int)cudaGetLastError();
}

// ------------------------------------------------------------- EDE -------
// Sorted vertex triple of ede_Initialization.c:24-78 (its tie rule kept).
__device__ __forceinline__ void ede_sort3(const int *l, int *I, int *o)
{
	if (l[0] < l[1] && l[0] < l[2]) {
		if (l[1] < l[2]) { o[0] = 0; o[1] = 1; o[2] = 2; } else { o[0] = 0; o[1] = 2; o[2] = 1; }
	} else if (l[1] < l[2]) {
		if (l[0] < l[2]) { o[0] = 1; o[1] = 0; o[2] = 2; } else { o[0] = 1; o[1] = 2; o[2] = 0; }
	} else {
		if (l[0] < l[1]) { o[0] = 2; o[1] = 0; o[2] = 1; } else { o[0] = 2; o[1] = 1; o[2] = 0; }
	}
	I[0] = l[o[0]]; I[1] = l[o[1]]; I[2] = l[o[2]];
}

// Row I < neq of the edge list: every J > I that shares an element with I,
// where J may be the dump equation neq (edges (I1,I2), (I1,I3), (I2,I3) of
// each sorted triple).
__global__ void k_ede_rows(const int *ri_ptr, const int *ri, const int *lm, int neq,
                           int *rowlen, const int *ind, int *lm2, int *err)
{
	int row[FG_MAXROW];
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x) {
		int m = 0, ok = 1;
		for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
			int e = ri[q] / 3;
			for (int b = 0; b < 3; b++) {
				int J = lm[3 * e + b];
				if (J > I) ok &= ins_sorted(row, &m, J);
			}
		}
		if (!ok) fg_set_err(err, FEMGPU_E_MESH);
		if (rowlen) rowlen[I] = m;
		if (lm2) {
			int base = ind[I];
			for (int q = 0; q < m; q++) { lm2[2 * (base + q)] = I; lm2[2 * (base + q) + 1] = row[q]; }
		}
	}
}

__global__ void k_ede_dump(const int *lm, int nel, int neq, int *has)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		int c = (lm[3 * e] == neq) + (lm[3 * e + 1] == neq) + (lm[3 * e + 2] == neq);
		if (c >= 2) *has = 1;
	}
}

__device__ __forceinline__ int ede_pos(const int *ind, const int *lm2, int neq, int nedge, int I, int J)
{
	if (I == neq) return nedge;
	int lo = ind[I], hi = ind[I + 1];
	while (lo < hi) {
		int mid = (lo + hi) >> 1;
		if (lm2[2 * mid + 1] < J) lo = mid + 1; else hi = mid;
	}
	return lo;
}

// EDGE_by_Element and order (ede_Initialization.c:104-133).
__global__ void k_ede_sbe(const int *lm, const int *ind, const int *lm2, int nel, int neq, int nedge,
                          int *sbe, int *order)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		int l[3] = { lm[3 * e], lm[3 * e + 1], lm[3 * e + 2] }, I[3], o[3];
		ede_sort3(l, I, o);
		sbe[3 * e + 0] = ede_pos(ind, lm2, neq, nedge, I[0], I[1]);
		sbe[3 * e + 1] = ede_pos(ind, lm2, neq, nedge, I[0], I[2]);
		sbe[3 * e + 2] = ede_pos(ind, lm2, neq, nedge, I[1], I[2]);
		order[3 * e] = o[0]; order[3 * e + 1] = o[1]; order[3 * e + 2] = o[2];
	}
}

extern "C" int fg_build_ede(femgpu_transport *t)
{
	cudaStream_t s = t->stream;
	int neq = t->neq, *rowlen = nullptr, *ind = nullptr, *has = nullptr, hhas = 0, herr = 0;
	FG_TRY(cudaMalloc(&rowlen, sizeof(int) * (neq + 1)));
	FG_TRY(cudaMalloc(&ind, sizeof(int) * (neq + 2)));
	FG_TRY(cudaMalloc(&has, sizeof(int)));
	FG_TRY(cudaMemsetAsync(has, 0, sizeof(int), s));
	k_ede_rows<<<fg_grid(neq, 128), 128, 0, s>>>(t->ri_ptr, t->ri, t->lm, neq, rowlen, nullptr,
	                                             nullptr, &t->st->err);
	k_ede_dump<<<fg_grid(t->nel), FG_TPB, 0, s>>>(t->lm, t->nel, neq, has);
	int rc = fg_scan(rowlen, ind, neq, s);
	if (rc) return rc;
	FG_TRY(cudaMemcpy(&t->nedge, ind + neq, sizeof(int), cudaMemcpyDeviceToHost));
	FG_TRY(cudaMemcpy(&hhas, has, sizeof(int), cudaMemcpyDeviceToHost));
	// The reference keeps one (neq, neq) dump edge at index nedge and would
	// overflow its edge arrays without it (ede_Initialization.c:103-151).
	if (!hhas) { cudaFree(rowlen); cudaFree(ind); cudaFree(has); return FEMGPU_E_MESH; }
	FG_TRY(cudaMalloc(&t->lm2, sizeof(int) * 2LL * (t->nedge + 1)));
	FG_TRY(cudaMalloc(&t->sbe, sizeof(int) * 3LL * t->nel));
	FG_TRY(cudaMalloc(&t->order, sizeof(int) * 3LL * t->nel));
	k_ede_rows<<<fg_grid(neq, 128), 128, 0, s>>>(t->ri_ptr, t->ri, t->lm, neq, nullptr, ind, t->lm2,
	                                             &t->st->err);
	k_ede_sbe<<<fg_grid(t->nel), FG_TPB, 0, s>>>(t->lm, ind, t->lm2, t->nel, neq, t->nedge, t->sbe,
	                                             t->order);
	FG_TRY(cudaGetLastError());
	FG_TRY(cudaMemcpyAsync(&herr, &t->st->err, sizeof(int), cudaMemcpyDeviceToHost, s));
	FG_TRY(cudaStreamSynchronize(s));
	cudaFree(rowlen); cudaFree(has);
	t->IA = ind;                    // first-endpoint edge ranges per row
	if (herr) return herr;
	// Contributors of each edge (element slots, ascending element) for the
	// deterministic assembly gather, and for each row the edges where it is
	// the second endpoint (ascending edge index) for the matvec gather.
	rc = fg_invert_map(t->sbe, 1, 3 * t->nel, t->nedge, &t->ec_ptr, &t->ec, s);
	if (rc) return rc;
	return fg_invert_map(t->lm2 + 1, 2, t->nedge, neq, &t->e2_ptr, &t->e2, s);
}
