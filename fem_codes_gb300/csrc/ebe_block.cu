// Multi-dof element-by-element operators of the Euler (4 dof per node, 12x12
// element blocks) and Navier-Stokes (3 dof per node, 9x9) drivers:
//   ebemvNDOF4.c / ebemvNDOF3.c   Q = A P, element by element
//   ebe2mvNDOF4.c                 off-diagonal node blocks, then the nodal
//                                 blocks (BlockDiag2_precond.c / NOBlockDiag2_precond.c)
//   BlockDiag_precond_EBE_setup.c / BlockDiagDOF3_precond_EBE_setup.c and
//   BlockDiag_precond.c / BlockDiagDOF3_precond.c   nodal block-diagonal preconditioner
// Every product is a per-row (or per-node) gather over the incident elements
// in ascending element order, so the additions happen in the reference's
// order; this file is compiled without FMA contraction, so results are
// bit-identical to the reference.  The FP32 variants at the end serve the
// mixed-precision flexible solves only (explicit fused multiply-adds).
#include "fg_common.cuh"
#include "fg_ebe.h"

__global__ void k_lm_blk(int ndof, int nel, const int *vert, const int *node_id, int neq, int *lm)
{
	int m = 3 * ndof;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)nel * m;
	     i += (long long)gridDim.x * blockDim.x) {
		int e = (int)(i / m), l = (int)(i - (long long)e * m), a = l / ndof, k = l - a * ndof;
		int id = node_id[ndof * vert[3 * e + a] + k];
		lm[i] = (id == -1) ? neq : id;
	}
}

// Q[I] = sum over (e, a) incident to row I of sum_b A[e][a][b] P[lm[e][b]]
// (the element's row evaluated left to right, then added to Q[I]).
// OFFDIAG: the b of the row's own node block are skipped (ebe2mvNDOF4).
template <int NDOF, bool OFFDIAG>
__global__ void k_ebemv_blk(int neq, const int *__restrict__ ri_ptr, const int *__restrict__ ri,
                            const int *__restrict__ lm, const double *__restrict__ A,
                            const double *__restrict__ P, double *__restrict__ Q)
{
	constexpr int M = 3 * NDOF;
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double q = 0.0;
		if (I < neq) {
			for (int t = ri_ptr[I]; t < ri_ptr[I + 1]; t++) {
				int code = __ldg(&ri[t]), e = code / M, a = code - e * M;
				const int *l = lm + (long long)e * M;
				const double *row = A + (long long)e * M * M + a * M;
				double s = 0.0;
				bool first = true;
				#pragma unroll
				for (int b = 0; b < M; b++) {
					if (OFFDIAG && b / NDOF == a / NDOF) continue;
					int j = __ldg(&l[b]);
					double p = (j == neq) ? 0.0 : __ldg(&P[j]);
					double prod = __ldg(&row[b]) * p;
					s = first ? prod : s + prod;
					first = false;
				}
				q = q + s;
			}
		}
		Q[I] = q;
	}
}

// Mixed precision (not a reference operation): FP32 element matrices and
// vector, each element row accumulated by FP32 fused multiply-adds, the row's
// incident element rows summed in FP64.
template <int NDOF>
__global__ void k_ebemv_blk32(int neq, const int *__restrict__ ri_ptr, const int *__restrict__ ri,
                              const int *__restrict__ lm, const float *__restrict__ A,
                              const float *__restrict__ P, double *__restrict__ Q)
{
	constexpr int M = 3 * NDOF;
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double q = 0.0;
		if (I < neq) {
			for (int t = ri_ptr[I]; t < ri_ptr[I + 1]; t++) {
				int code = __ldg(&ri[t]), e = code / M, a = code - e * M;
				int l[M];
				float r[M];
				if constexpr (M % 4 == 0) {
					// rows of M floats and lm blocks of M ints start on 16-byte
					// boundaries: M/4 16-byte loads each
					#pragma unroll
					for (int v = 0; v < M / 4; v++) {
						int4 li = __ldg(reinterpret_cast<const int4 *>(lm + (long long)e * M) + v);
						float4 rv = __ldg(reinterpret_cast<const float4 *>(A + (long long)e * M * M + a * M) + v);
						l[4 * v] = li.x; l[4 * v + 1] = li.y; l[4 * v + 2] = li.z; l[4 * v + 3] = li.w;
						r[4 * v] = rv.x; r[4 * v + 1] = rv.y; r[4 * v + 2] = rv.z; r[4 * v + 3] = rv.w;
					}
				} else {
					#pragma unroll
					for (int b = 0; b < M; b++) {
						l[b] = __ldg(&lm[(long long)e * M + b]);
						r[b] = __ldg(&A[(long long)e * M * M + a * M + b]);
					}
				}
				float s = 0.0f;
				#pragma unroll
				for (int b = 0; b < M; b++) {
					float p = (l[b] == neq) ? 0.0f : __ldg(&P[l[b]]);
					s = fmaf(r[b], p, s);
				}
				q += (double)s;
			}
		}
		Q[I] = q;
	}
}

__device__ __forceinline__ int blk_id(const int *node_id, int ndof, int neq, int node, int k)
{
	int id = node_id[ndof * node + k];
	return id < 0 ? neq : id;
}

// Nodal diagonal blocks summed over the incident elements in element order.
template <int NDOF>
__global__ void k_blockdiag_assemble(int nnodes, const int *ni_ptr, const int *ni, const double *A, double *BD)
{
	constexpr int M = 3 * NDOF, D2 = NDOF * NDOF;
	for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnodes; n += gridDim.x * blockDim.x) {
		double b[D2];
		#pragma unroll
		for (int k = 0; k < D2; k++) b[k] = 0.0;
		for (int t = ni_ptr[n]; t < ni_ptr[n + 1]; t++) {
			int code = ni[t], e = code / 3, a = code - 3 * e;
			const double *Ae = A + (long long)e * M * M;
			#pragma unroll
			for (int I = 0; I < NDOF; I++)
				#pragma unroll
				for (int J = 0; J < NDOF; J++) b[NDOF * I + J] += Ae[(NDOF * a + I) * M + NDOF * a + J];
		}
		#pragma unroll
		for (int k = 0; k < D2; k++) BD[(long long)n * D2 + k] = b[k];
	}
}

// Adjugate over determinant, expanded as BlockDiag_precond_EBE_setup.c:88-145
// (4x4) and BlockDiagDOF3_precond_EBE_setup.c:90-120 (3x3) do.
__device__ __forceinline__ void inverse4(const double *B, double *V)
{
	double a = B[0], b = B[1], c = B[2], d = B[3], e = B[4], f = B[5], g = B[6], h = B[7];
	double i = B[8], j = B[9], k = B[10], l = B[11], m = B[12], n = B[13], o = B[14], p = B[15];
	double det = (a*f*k*p - a*f*l*o - a*g*j*p + a*g*l*n + a*h*j*o - a*h*k*n
		-b*e*k*p  + b*e*l*o + b*g*i*p - b*g*l*m - b*h*i*o + b*h*k*m +
		c*(e*j*p - e*l*n - f*i*p + f*l*m + h*i*n - h*j*m) +
		d*(-e*j*o + e*k*n + f*i*o - f*k*m - g*i*n + g*j*m));
	double q = 1.0/det;
	V[0] = q*(-h*k*n + g*l*n + h*j*o - f*l*o - g*j*p + f*k*p);
	V[1] = q*(d*k*n - c*l*n - d*j*o + b*l*o + c*j*p - b*k*p);
	V[2] = q*(-d*g*n + c*h*n + d*f*o - b*h*o - c*f*p + b*g*p);
	V[3] = q*(d*g*j - c*h*j - d*f*k + b*h*k + c*f*l - b*g*l);
	V[4] = q*(h*k*m - g*l*m - h*i*o + e*l*o + g*i*p - e*k*p);
	V[5] = q*(-d*k*m + c*l*m + d*i*o - a*l*o - c*i*p + a*k*p);
	V[6] = q*(d*g*m - c*h*m - d*e*o + a*h*o + c*e*p - a*g*p);
	V[7] = q*(-d*g*i + c*h*i + d*e*k - a*h*k - c*e*l + a*g*l);
	V[8] = q*(-h*j*m + f*l*m + h*i*n - e*l*n - f*i*p + e*j*p);
	V[9] = q*(d*j*m - b*l*m - d*i*n + a*l*n + b*i*p - a*j*p);
	V[10] = q*(-d*f*m + b*h*m + d*e*n - a*h*n - b*e*p + a*f*p);
	V[11] = q*(d*f*i - b*h*i - d*e*j + a*h*j + b*e*l - a*f*l);
	V[12] = q*(g*j*m - f*k*m - g*i*n + e*k*n + f*i*o - e*j*o);
	V[13] = q*(-c*j*m + b*k*m + c*i*n - a*k*n - b*i*o + a*j*o);
	V[14] = q*(c*j*m - b*g*m - c*e*n + a*g*n + b*e*o - a*f*o);
	V[15] = q*(-c*f*i + b*g*i + c*e*j - a*g*j - b*e*k + a*f*k);
}

__device__ __forceinline__ void inverse3(const double *B, double *V)
{
	double a = B[0], b = B[1], c = B[2], d = B[3], e = B[4], f = B[5], g = B[6], h = B[7], i = B[8];
	double det = a*e*i - a*f*h - b*d*i + b*f*g + c*d*h - c*e*g;
	double q = 1.0/det;
	V[0] = q*(e*i-f*h); V[1] = q*(c*h-b*i); V[2] = q*(b*f-c*e);
	V[3] = q*(f*g-d*i); V[4] = q*(a*i-c*g); V[5] = q*(c*d-a*f);
	V[6] = q*(d*h-e*g); V[7] = q*(b*g-a*h); V[8] = q*(a*e-b*d);
}

template <int NDOF>
__global__ void k_blockdiag_invert(int nnodes, const double *BD, double *invBD)
{
	constexpr int D2 = NDOF * NDOF;
	for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnodes; n += gridDim.x * blockDim.x) {
		double b[D2], v[D2];
		#pragma unroll
		for (int k = 0; k < D2; k++) b[k] = BD[(long long)n * D2 + k];
		if (NDOF == 4) inverse4(b, v); else inverse3(b, v);
		#pragma unroll
		for (int k = 0; k < D2; k++) invBD[(long long)n * D2 + k] = v[k];
	}
}

// MODE 0: z = D^-1 p (BlockDiag_precond), 1: z = p + D^-1 z (BlockDiag2_precond,
// z holds the off-diagonal product), 2: z += D p (NOBlockDiag2_precond).  Per
// node; the dump equation neq is never written (zeroed separately).
template <int NDOF, int MODE>
__global__ void k_blockdiag_apply(int nnodes, int neq, const int *node_id, const double *B,
                                  const double *p, double *z)
{
	constexpr int D2 = NDOF * NDOF;
	for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnodes; n += gridDim.x * blockDim.x) {
		int id[NDOF];
		double v[NDOF];
		#pragma unroll
		for (int c = 0; c < NDOF; c++) {
			id[c] = blk_id(node_id, NDOF, neq, n, c);
			// ebe2mvNDOF4.c:21 zeroes P[neq] and Q[neq] before modes 1 and 2 read them
			v[c] = (MODE == 1) ? (id[c] == neq ? 0.0 : z[id[c]])
			     : (MODE == 2 && id[c] == neq) ? 0.0 : p[id[c]];
		}
		const double *Bn = B + (long long)n * D2;
		#pragma unroll
		for (int r = 0; r < NDOF; r++) {
			double s;
			if (MODE == 1) {
				s = p[id[r]];
				#pragma unroll
				for (int c = 0; c < NDOF; c++) s = s + Bn[NDOF * r + c] * v[c];
			} else {
				s = Bn[NDOF * r] * v[0];
				#pragma unroll
				for (int c = 1; c < NDOF; c++) s = s + Bn[NDOF * r + c] * v[c];
				if (MODE == 2) s = (id[r] == neq ? 0.0 : z[id[r]]) + s;
			}
			if (id[r] != neq) z[id[r]] = s;
		}
	}
}

__global__ void k_zero_one(double *z, int i) { z[i] = 0.0; }
__global__ void k_zero_one32(float *z, int i) { z[i] = 0.0f; }

// z = D^-1 p per node (BlockDiag_precond's arithmetic), stored in FP32.
template <int NDOF>
__global__ void k_blockdiag_apply32(int nnodes, int neq, const int *node_id, const double *B, const double *p,
                                    float *z)
{
	constexpr int D2 = NDOF * NDOF;
	for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnodes; n += gridDim.x * blockDim.x) {
		int id[NDOF];
		double v[NDOF];
		#pragma unroll
		for (int c = 0; c < NDOF; c++) { id[c] = blk_id(node_id, NDOF, neq, n, c); v[c] = p[id[c]]; }
		const double *Bn = B + (long long)n * D2;
		#pragma unroll
		for (int r = 0; r < NDOF; r++) {
			double s = Bn[NDOF * r] * v[0];
			#pragma unroll
			for (int c = 1; c < NDOF; c++) s = s + Bn[NDOF * r + c] * v[c];
			if (id[r] != neq) z[id[r]] = (float)s;
		}
	}
}

__global__ void k_to_f32_blk(const double *__restrict__ a, float *__restrict__ b, long long n)
{
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		b[i] = (float)a[i];
}

// ------------------------------------------------------------- launchers
extern "C" int fg_ebe_lm(femgpu_ebe *c)
{
	k_lm_blk<<<fg_grid((long long)c->nel * c->m), FG_TPB, 0, c->stream>>>(c->ndof, c->nel, c->vert, c->node_id,
	                                                                      c->neq, c->lm);
	FG_TRY(cudaGetLastError());
	int rc = fg_invert_map(c->lm, 1, c->nel * c->m, c->neq, &c->ri_ptr, &c->ri, c->stream);
	if (rc) return rc;
	return fg_invert_map(c->vert, 1, 3 * c->nel, c->nnodes, &c->ni_ptr, &c->ni, c->stream);
}

extern "C" int fg_ebe_matvec(femgpu_ebe *c, const double *P, double *Q, int offdiag)
{
	int g = fg_grid(c->neq + 1LL, 128, 32);
	if (c->ndof == 4) {
		if (offdiag) k_ebemv_blk<4, true><<<g, 128, 0, c->stream>>>(c->neq, c->ri_ptr, c->ri, c->lm, c->A, P, Q);
		else k_ebemv_blk<4, false><<<g, 128, 0, c->stream>>>(c->neq, c->ri_ptr, c->ri, c->lm, c->A, P, Q);
	} else {
		k_ebemv_blk<3, false><<<g, 128, 0, c->stream>>>(c->neq, c->ri_ptr, c->ri, c->lm, c->A, P, Q);
	}
	return (int)cudaGetLastError();
}

// Block_scaling.c:7-110 for the 4-dof element matrices, one thread per
// element: every prescribed dof's row and column of Ae (12x12, row-major)
// become zero with a one on the diagonal (matrix_Bondary_Conditions), then
// each vertex's row block is replaced by invBD(vertex) times the adjusted
// row block, each entry summed over j in order from zero (matrix_Scaling).
__global__ void k_block_scale4(int nel, const int *__restrict__ vert, const int *__restrict__ node_id,
                               const double *__restrict__ invBD, double *A)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		double *a = A + 144LL * e;
		int v[3];
		for (int b = 0; b < 3; b++) v[b] = vert[3 * e + b];
		for (int b = 0; b < 3; b++)
			for (int d = 0; d < 4; d++) {
				if (node_id[4 * v[b] + d] >= 0) continue;
				const int r = 4 * b + d;
				for (int k = 0; k < 12; k++) { a[12 * r + k] = 0.0; a[12 * k + r] = 0.0; }
				a[12 * r + r] = 1.0;
			}
		for (int b = 0; b < 3; b++) {
			double m[4][12];
			const double *D = invBD + 16LL * v[b];
			for (int j = 0; j < 4; j++)
				for (int k = 0; k < 12; k++) m[j][k] = a[12 * (4 * b + j) + k];
			for (int i = 0; i < 4; i++)
				for (int k = 0; k < 12; k++) {
					double s = 0.0;
					for (int j = 0; j < 4; j++) s += D[4 * i + j] * m[j][k];
					a[12 * (4 * b + i) + k] = s;
				}
		}
	}
}

extern "C" int fg_ebe_block_scale(femgpu_ebe *c)
{
	if (c->ndof != 4) return FEMGPU_E_ARG;
	k_block_scale4<<<fg_grid(c->nel), FG_TPB, 0, c->stream>>>(c->nel, c->vert, c->node_id, c->invBD, c->A);
	return (int)cudaGetLastError();
}

extern "C" int fg_ebe_blockdiag_setup(femgpu_ebe *c)
{
	int g = fg_grid(c->nnodes);
	if (c->ndof == 4) {
		k_blockdiag_assemble<4><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->ni_ptr, c->ni, c->A, c->BD);
		k_blockdiag_invert<4><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->BD, c->invBD);
	} else {
		k_blockdiag_assemble<3><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->ni_ptr, c->ni, c->A, c->BD);
		k_blockdiag_invert<3><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->BD, c->invBD);
	}
	return (int)cudaGetLastError();
}

extern "C" int fg_ebe_blockdiag_apply(femgpu_ebe *c, const double *p, double *z, int mode)
{
	int g = fg_grid(c->nnodes);
	const double *B = (mode == 2) ? c->BD : c->invBD;
	if (c->ndof == 4) {
		if (mode == 0) k_blockdiag_apply<4, 0><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->neq, c->node_id, B, p, z);
		else if (mode == 1) k_blockdiag_apply<4, 1><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->neq, c->node_id, B, p, z);
		else k_blockdiag_apply<4, 2><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->neq, c->node_id, B, p, z);
	} else {
		k_blockdiag_apply<3, 0><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->neq, c->node_id, B, p, z);
	}
	k_zero_one<<<1, 1, 0, c->stream>>>(z, c->neq);
	return (int)cudaGetLastError();
}

extern "C" int fg_ebe_to_f32(femgpu_ebe *c)
{
	long long n = (long long)c->nel * c->m * c->m;
	if (!c->A32) FG_TRY(cudaMalloc((void **)&c->A32, sizeof(float) * (size_t)n));
	k_to_f32_blk<<<fg_grid(n), FG_TPB, 0, c->stream>>>(c->A, c->A32, n);
	return (int)cudaGetLastError();
}

extern "C" int fg_ebe_matvec32(femgpu_ebe *c, const float *P, double *Q)
{
	int g = fg_grid(c->neq + 1LL, 128, 32);
	if (!c->A32) return FEMGPU_E_NOT_BUILT;
	if (c->ndof == 4) k_ebemv_blk32<4><<<g, 128, 0, c->stream>>>(c->neq, c->ri_ptr, c->ri, c->lm, c->A32, P, Q);
	else k_ebemv_blk32<3><<<g, 128, 0, c->stream>>>(c->neq, c->ri_ptr, c->ri, c->lm, c->A32, P, Q);
	return (int)cudaGetLastError();
}

extern "C" int fg_ebe_blockdiag_apply32(femgpu_ebe *c, const double *p, float *z)
{
	int g = fg_grid(c->nnodes);
	if (c->ndof == 4) k_blockdiag_apply32<4><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->neq, c->node_id, c->invBD, p, z);
	else k_blockdiag_apply32<3><<<g, FG_TPB, 0, c->stream>>>(c->nnodes, c->neq, c->node_id, c->invBD, p, z);
	k_zero_one32<<<1, 1, 0, c->stream>>>(z, c->neq);
	return (int)cudaGetLastError();
}
