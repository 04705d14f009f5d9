// 2D Euler SUPG element build with CAU or YZBeta shock capturing
// (03_Euler_Equations/2D/01_CommonFiles: Build_M_K_F_SUPG.c:6-1072,
// Delta_CAU.c:4-84, Delta_YZBeta.c:6-108, Ax_Ay_calculations.c:3-98,
// eval_U_dU.c:3-94) and the predictor-multicorrector vector updates
// (00_CommonFiles/Time_Integration/Predictor_Old.c:57-62,115-116 and the
// BDF / TR-BDF2 combinations of Predictor_Old_BDF.c, Predictor_Old_TRBDF2.c).
//
// One thread per element computes the 12x12 matrix Ae = Me + alpha dt Ke and
// the 12 residual entries Re = -(Me dUe + Ke Ue) and writes Ae straight into
// the block-EBE storage (row-major, as ebe_assembly.c:3-16 stores it).  The
// residual is then assembled per equation over the incident elements in
// ascending element order, i.e. in the order of the reference's scatter loop
// (:1059-1060), so R is bit-identical.  This translation unit is compiled
// without FMA contraction; every expression keeps the reference's evaluation
// order.  The work is FP64-throughput bound (about 2.5k FP64 operations per
// element against 1.25 kB written).
#include "fg_common.cuh"
#include "fg_euler.h"
#include "euler_elem.cuh"

// Structure of the flux Jacobians: 0 structural zero, 1 unit entry, 2 general
// (row 0 of Ax is e_1 and of Ay e_2; Ax[2][3] = Ay[1][3] = 0).  The
// reference's hand-expanded products (Build_M_K_F_SUPG.c:163-237),
// Delta_CAU.c:18-26 and the C matrices (:277-332) leave out exactly the terms
// with a structural-zero factor and write a unit factor's partner alone.
__host__ __device__ constexpr int kax(int i, int j) { return i == 0 ? (j == 1 ? 1 : 0) : (i == 2 && j == 3) ? 0 : 2; }
__host__ __device__ constexpr int kay(int i, int j) { return i == 0 ? (j == 2 ? 1 : 0) : (i == 1 && j == 3) ? 0 : 2; }

// (X Y)[i][j] over the terms that are not structurally zero, ascending k.
template <bool XA, bool YA>
__device__ __forceinline__ double jprod(const double (&X)[4][4], const double (&Y)[4][4], int i, int j)
{
	double s = 0.0;
	bool first = true;
	#pragma unroll
	for (int k = 0; k < 4; k++) {
		int kx = XA ? kax(i, k) : kay(i, k), ky = YA ? kax(k, j) : kay(k, j);
		if (kx == 0 || ky == 0) continue;
		double t = kx == 1 ? Y[k][j] : (ky == 1 ? X[i][k] : X[i][k] * Y[k][j]);
		s = first ? t : s + t;
		first = false;
	}
	return s;
}

template <bool XA>
__device__ __forceinline__ double jvec(const double (&X)[4][4], const double *g, int i)
{
	double s = 0.0;
	bool first = true;
	#pragma unroll
	for (int k = 0; k < 4; k++) {
		int kx = XA ? kax(i, k) : kay(i, k);
		if (kx == 0) continue;
		double t = kx == 1 ? g[k] : X[i][k] * g[k];
		s = first ? t : s + t;
		first = false;
	}
	return s;
}

// Quadratic form v^T A0 v as Delta_CAU.c:36-43 writes it.
__device__ __forceinline__ double a0norm2(const double (&A0)[4][4], const double *v)
{
	return v[0] * (A0[0][0] * v[0] + 2.0 * A0[0][1] * v[1] + 2.0 * A0[0][2] * v[2] + 2.0 * A0[0][3] * v[3]) +
	       v[1] * (A0[1][1] * v[1] + 2.0 * A0[1][2] * v[2] + 2.0 * A0[1][3] * v[3]) +
	       v[2] * (A0[2][2] * v[2] + 2.0 * A0[2][3] * v[3]) +
	       v[3] * A0[3][3] * v[3];
}

struct EulerCoef {
	double gamma, mach, alpha, dt, stab_tol;
	int dimensionless, neq;
	int yzbeta;                 // shock capturing: 0 Delta_CAU, 1 Delta_YZBeta
	double invY[4];             // YZBeta: the deck's Y^-1
};

__global__ void __launch_bounds__(128) k_euler_element(int nel, const int *__restrict__ vert,
		const int *__restrict__ node_id, const double *__restrict__ xn, const double *__restrict__ yn,
		const double *__restrict__ upresc, const double *__restrict__ u, const double *__restrict__ du,
		EulerCoef cf, double *__restrict__ A, double *__restrict__ Re, double *__restrict__ dold)
{
	const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
	const double gamma = cf.gamma;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		double X[3], Y[3], yb[3], xb[3], Ue[12], dUe[12];
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			int J = __ldg(&vert[3 * e + a]);
			X[a] = __ldg(&xn[J]);
			Y[a] = __ldg(&yn[J]);
			#pragma unroll
			for (int k = 0; k < 4; k++) {                          // eval_U_dU.c:22-91
				int id = __ldg(&node_id[4 * J + k]);
				Ue[4 * a + k] = id >= 0 ? __ldg(&u[id]) : __ldg(&upresc[4 * J + k]);
				dUe[4 * a + k] = id >= 0 ? __ldg(&du[id]) : 0.0;
			}
		}
		yb[0] = Y[1] - Y[2]; yb[1] = Y[2] - Y[0]; yb[2] = Y[0] - Y[1];     // y23 y31 y12
		xb[0] = X[2] - X[1]; xb[1] = X[0] - X[2]; xb[2] = X[1] - X[0];     // x32 x13 x21
		double twoArea = fabs(xb[2] * yb[1] - xb[1] * yb[2]);
		double Area = 0.5 * twoArea;

		double Ub[4], dUb[4], gx[4], gy[4];
		#pragma unroll
		for (int i = 0; i < 4; i++) {
			Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
			dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
		}
		#pragma unroll
		for (int i = 0; i < 4; i++) {
			gx[i] = (Ue[i] * yb[0] + Ue[i + 4] * yb[1] + Ue[i + 8] * yb[2]) / twoArea;
			gy[i] = (Ue[i] * xb[0] + Ue[i + 4] * xb[1] + Ue[i + 8] * xb[2]) / twoArea;
		}
		double v1 = Ub[1] / Ub[0], v2 = Ub[2] / Ub[0], E = Ub[3] / Ub[0];

		// Flux Jacobians (Ax_Ay_calculations.c) and A0^-1 in entropy
		// variables (:131-159).
		double Ax[4][4], Ay[4][4], A0[4][4];
		euler_jacobians(Ub, gamma, cf.mach, cf.dimensionless, Ax, Ay);
		euler_a0(Ub, gamma, A0);

		// Shock-capturing delta: Delta_YZBeta.c:6-108 (stateful: blended with
		// the element's previous delta, which it replaces) or Delta_CAU.c:17-82.
		double delta;
		if (cf.yzbeta) {
			double Z[4];
			euler_residual4(Ax, Ay, gx, gy, dUb, Z);
			delta = euler_delta_yzbeta(Z, gx, gy, Ub, cf.invY, yb, xb, twoArea, &dold[e]);
		} else {
			double kx[4], ky[4], L[4];
			#pragma unroll
			for (int i = 0; i < 4; i++) {
				kx[i] = (yb[0] * gx[i] + xb[0] * gy[i]) / twoArea;
				ky[i] = (yb[1] * gx[i] + xb[1] * gy[i]) / twoArea;
			}
			double nk = sqrt(a0norm2(A0, kx) + a0norm2(A0, ky));
			#pragma unroll
			for (int i = 0; i < 4; i++) L[i] = dUb[i] + jvec<true>(Ax, gx, i) + jvec<false>(Ay, gy, i);
			double nL = sqrt(a0norm2(A0, L));
			double ng = sqrt(a0norm2(A0, gx) + a0norm2(A0, gy));
			delta = ng >= cf.stab_tol ? nL / nk : 0.0;
		}

		// SUPG tau (:244-269).
		double tau;
		{
			double bx = 2.0 * (gx[0] * Ub[0] + gx[1] * Ub[1] + gx[2] * Ub[2] + gx[3] * Ub[3]);
			double by = 2.0 * (gy[0] * Ub[0] + gy[1] * Ub[1] + gy[2] * Ub[2] + gy[3] * Ub[3]);
			double bxy = sqrt(bx * bx + by * by);
			if (bxy != 0.0) { bx = bx / bxy; by = by / bxy; }
			double h = sqrt(twoArea);
			double avb = fabs(v1 * bx + v2 * by);
			double cs = sqrt(gamma * (gamma - 1.0) * (E - 0.5 * ((v1 * v1) + (v2 * v2))));
			double CFL = ((cs + avb) * cf.dt) / h;
			double psi = (2.0 * cf.alpha * CFL) * (1.0 / (1.0 + 2.0 * cf.alpha * CFL));
			double tau_d = delta / ((cs + avb) * (cs + avb));
			double tau_a = h / (2.0 * (cs + avb));
			double tau_t = (2.0 / (3.0 * (1.0 + 2.0 * cf.alpha * CFL))) * tau_a;
			tau = tau_t + psi * (tau_a - tau_d);
			if (tau < 0.0) tau = 0.0;
		}

		// AxAx, AxAy, AyAx, AyAy (:163-237).
		double Pxx[4][4], Pxy[4][4], Pyx[4][4], Pyy[4][4];
		#pragma unroll
		for (int i = 0; i < 4; i++)
			#pragma unroll
			for (int j = 0; j < 4; j++) {
				Pxx[i][j] = jprod<true, true>(Ax, Ax, i, j);
				Pxy[i][j] = jprod<true, false>(Ax, Ay, i, j);
				Pyx[i][j] = jprod<false, true>(Ay, Ax, i, j);
				Pyy[i][j] = jprod<false, false>(Ay, Ay, i, j);
			}
		// C_a = (y_a Ax + x_a Ay)/6 (:277-332).
		double C[3][4][4];
		#pragma unroll
		for (int a = 0; a < 3; a++)
			#pragma unroll
			for (int i = 0; i < 4; i++)
				#pragma unroll
				for (int j = 0; j < 4; j++) {
					int kx_ = kax(i, j), ky_ = kay(i, j);
					double cv;
					if (!kx_ && !ky_) cv = 0.0;
					else if (kx_ == 1) cv = yb[a] * sixth;
					else if (ky_ == 1) cv = xb[a] * sixth;
					else if (!ky_) cv = yb[a] * Ax[i][j] * sixth;
					else if (!kx_) cv = xb[a] * Ay[i][j] * sixth;
					else cv = (yb[a] * Ax[i][j] + xb[a] * Ay[i][j]) * sixth;
					C[a][i][j] = cv;
				}
		const double Mg1 = Area * sixth, Mg2 = Area / 12.0;
		const double tau4area = tau / (4 * Area), delta4area = delta / (4.0 * Area);
		const double adt = cf.alpha * cf.dt;
		double Kc01 = delta4area * (yb[0] * yb[1] + xb[0] * xb[1]);
		double Kc02 = delta4area * (yb[0] * yb[2] + xb[0] * xb[2]);
		double Kc12 = delta4area * (yb[1] * yb[2] + xb[1] * xb[2]);
		double *Ae = A + (long long)e * 144;

		// Block rows a: Me (:401-561), Ke (:563-1026), Ae and Re (:1033-1042).
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			const int b1 = a == 0 ? 1 : 0, b2 = a == 2 ? 1 : 2;
			double axa[4][4], aya[4][4];   // y_a AxAx + x_a AyAx, y_a AxAy + x_a AyAy (:629-735)
			#pragma unroll
			for (int i = 0; i < 4; i++)
				#pragma unroll
				for (int j = 0; j < 4; j++) {
					axa[i][j] = yb[a] * Pxx[i][j] + xb[a] * Pyx[i][j];
					aya[i][j] = yb[a] * Pxy[i][j] + xb[a] * Pyy[i][j];
				}
			double m[4] = {0.0, 0.0, 0.0, 0.0}, q[4] = {0.0, 0.0, 0.0, 0.0};
			#pragma unroll
			for (int b = 0; b < 3; b++) {
				const double kc = (a + b == 1) ? Kc01 : (a + b == 2) ? Kc02 : Kc12;   // a != b
				const double kcd = a == 0 ? Kc01 + Kc02 : a == 1 ? Kc01 + Kc12 : Kc02 + Kc12;
				#pragma unroll
				for (int r = 0; r < 4; r++)
					#pragma unroll
					for (int c = 0; c < 4; c++) {
						double mpg = C[a][r][c] * tau;
						double me = (r == c) ? (a == b ? Mg1 : Mg2) + mpg : mpg;
						double ke;
						if (a != b) {
							double kpg = tau4area * (yb[b] * axa[r][c] + xb[b] * aya[r][c]);
							ke = C[b][r][c] + kpg;
							if (r == c) ke = ke + kc;
						} else {
							double k1 = tau4area * (yb[b1] * axa[r][c] + xb[b1] * aya[r][c]);
							double k2 = tau4area * (yb[b2] * axa[r][c] + xb[b2] * aya[r][c]);
							ke = C[a][r][c] - (k1 + k2);
							if (r == c) ke = ke - kcd;
						}
						m[r] += me * dUe[4 * b + c];
						q[r] += ke * Ue[4 * b + c];
						Ae[(4 * a + r) * 12 + 4 * b + c] = me + adt * ke;
					}
			}
			#pragma unroll
			for (int r = 0; r < 4; r++) Re[(long long)e * 12 + 4 * a + r] = -m[r] - q[r];
		}
	}
}

// R[I] = sum of the incident elements' Re entries in ascending element order
// (dzero + the scatter of :1059-1060); R[neq] = 0.
__global__ void k_euler_gather(int neq, const int *__restrict__ ri_ptr, const int *__restrict__ ri,
                               const double *__restrict__ Re, double *__restrict__ R)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double s = 0.0;
		if (I < neq)
			for (int t = ri_ptr[I]; t < ri_ptr[I + 1]; t++) s += __ldg(&Re[__ldg(&ri[t])]);
		R[I] = s;
	}
}

__global__ void k_euler_predict(int n, double *u, double *a, double c_pred)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		u[I] += c_pred * a[I];
		a[I] = 0.0;
	}
}

__global__ void k_euler_correct(int n, double *u, double *a, const double *Da, double c_corr)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		double d = Da[I];
		a[I] += 1.0 * d;
		u[I] += c_corr * d;
	}
}

// rotation.c:3-43 at Build_M_K_F_SUPG.c:1044-1056: for each vertex (in
// vertex order) on a slip wall, the element matrix's 4x4 blocks in that
// vertex's block row are transformed with the vertex's angle -- the velocity
// rows rotated by P^T and the velocity columns by P, the reference's own
// entry-by-entry formulas -- and the vertex's velocity entries of Re rotated.
__global__ void k_euler_rotate(int nslip, const int *__restrict__ slip_el, const int *__restrict__ vert,
                               const int *__restrict__ flag, const double *__restrict__ cs_n,
                               const double *__restrict__ sn_n, double *A, double *Re)
{
	for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nslip; t += gridDim.x * blockDim.x) {
		const int e = slip_el[t];
		double *M = A + 144LL * e, *F = Re + 12LL * e;
		for (int tag = 0; tag < 3; tag++) {
			const int v = vert[3 * e + tag];
			if (!flag[v]) continue;
			const double cs = cs_n[v], sn = sn_n[v];
			const int I = 4 * tag;
			for (int K = 0; K < 3; K++) {
				const int J = 4 * K;
				double *r0 = M + 12 * I, *r1 = M + 12 * (I + 1), *r2 = M + 12 * (I + 2), *r3 = M + 12 * (I + 3);
				const double b = r0[J + 1], c = r0[J + 2], ee = r1[J], f = r1[J + 1], g = r1[J + 2], h = r1[J + 3];
				const double i = r2[J], j = r2[J + 1], k = r2[J + 2], l = r2[J + 3], n = r3[J + 1], o = r3[J + 2];
				r0[J + 1] = b*cs - c*sn;
				r0[J + 2] = b*sn + c*cs;
				r1[J] = ee*cs - i*sn;
				r1[J + 1] = cs*(f*cs - j*sn) - sn*(g*cs - k*sn);
				r1[J + 2] = cs*(g*cs - k*sn) + sn*(f*cs - j*sn);
				r1[J + 3] = h*cs - l*sn;
				r2[J] = ee*sn + i*cs;
				r2[J + 1] = cs*(f*sn + j*cs) - sn*(g*sn + k*cs);
				r2[J + 2] = cs*(g*sn + k*cs) + sn*(f*sn + j*cs);
				r2[J + 3] = h*sn + l*cs;
				r3[J + 1] = n*cs - o*sn;
				r3[J + 2] = n*sn + o*cs;
			}
			const double b = F[I + 1], c = F[I + 2];
			F[I + 1] = b*cs - c*sn;
			F[I + 2] = b*sn + c*cs;
		}
	}
}

// Build_M_K_F_DD_Transiente.c:37-911 (StabilizationForm "DD"): one thread
// per element through euler_dd_element; the element's bubble uB [4] and
// delta_old advance in place.
__global__ void __launch_bounds__(128) k_euler_element_dd(int nel, const int *__restrict__ vert,
		const int *__restrict__ node_id, const double *__restrict__ xn, const double *__restrict__ yn,
		const double *__restrict__ upresc, const double *__restrict__ u, const double *__restrict__ du,
		EulerCoef cf, double *__restrict__ A, double *__restrict__ Re, double *__restrict__ dold,
		double *__restrict__ uB)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		double X[3], Y[3], Ue[12], dUe[12];
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			int J = __ldg(&vert[3 * e + a]);
			X[a] = __ldg(&xn[J]);
			Y[a] = __ldg(&yn[J]);
			#pragma unroll
			for (int k = 0; k < 4; k++) {                          // eval_U_dU.c:22-91
				int id = __ldg(&node_id[4 * J + k]);
				Ue[4 * a + k] = id >= 0 ? __ldg(&u[id]) : __ldg(&upresc[4 * J + k]);
				dUe[4 * a + k] = id >= 0 ? __ldg(&du[id]) : 0.0;
			}
		}
		euler_dd_element(X, Y, Ue, dUe, cf.gamma, cf.mach, cf.dimensionless, cf.alpha, cf.dt, cf.stab_tol,
		                 cf.yzbeta, cf.invY, &dold[e], uB + 4LL * e, A + 144LL * e, Re + 12LL * e);
	}
}

extern "C" int fg_euler_build(femgpu_euler *c, const double *u, const double *du)
{
	EulerCoef cf;
	cf.gamma = c->o.gamma; cf.mach = c->o.mach; cf.alpha = c->alpha_build; cf.dt = c->dt_build;
	cf.stab_tol = c->o.stab_tol; cf.dimensionless = c->o.dimensionless; cf.neq = c->neq;
	cf.yzbeta = c->o.shock == FEMGPU_SHOCK_YZBETA;
	for (int k = 0; k < 4; k++) cf.invY[k] = c->o.invY[k];
	femgpu_ebe *b = c->ebe;
	int g = (int)((c->nel + 127LL) / 128);
	if (c->o.stab == FEMGPU_STAB_DD)
		k_euler_element_dd<<<g, 128, 0, c->stream>>>(c->nel, b->vert, b->node_id, c->x, c->y, c->upresc, u, du,
		                                             cf, b->A, c->Re, c->dold, c->uB);
	else
		k_euler_element<<<g, 128, 0, c->stream>>>(c->nel, b->vert, b->node_id, c->x, c->y, c->upresc, u, du,
		                                          cf, b->A, c->Re, c->dold);
	FG_TRY(cudaGetLastError());
	if (c->nslip_el > 0 && c->o.stab != FEMGPU_STAB_DD) {
		k_euler_rotate<<<fg_grid(c->nslip_el), FG_TPB, 0, c->stream>>>(c->nslip_el, c->slip_el, b->vert,
		                                                              c->slip_flag, c->slip_cs, c->slip_sn,
		                                                              b->A, c->Re);
		FG_TRY(cudaGetLastError());
	}
	k_euler_gather<<<fg_grid(c->neq + 1LL), FG_TPB, 0, c->stream>>>(c->neq, b->ri_ptr, b->ri, c->Re, c->R);
	return (int)cudaGetLastError();
}

extern "C" int fg_euler_predict(femgpu_euler *c, double c_pred)
{
	k_euler_predict<<<fg_grid(c->neq), FG_TPB, 0, c->stream>>>(c->neq, c->u, c->a, c_pred);
	return (int)cudaGetLastError();
}

__global__ void k_euler_lin(int n, double *u, const double *p, const double *q, double *a, double cp, double cq)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		u[I] = cp*p[I] - cq*q[I];
		a[I] = 0.0;
	}
}

extern "C" int fg_euler_lin(femgpu_euler *c, const double *p, const double *q, double cp, double cq)
{
	k_euler_lin<<<fg_grid(c->neq), FG_TPB, 0, c->stream>>>(c->neq, c->u, p, q, c->a, cp, cq);
	return (int)cudaGetLastError();
}

extern "C" int fg_euler_correct(femgpu_euler *c, double c_corr)
{
	k_euler_correct<<<fg_grid(c->neq), FG_TPB, 0, c->stream>>>(c->neq, c->u, c->a, c->Da, c_corr);
	return (int)cudaGetLastError();
}
