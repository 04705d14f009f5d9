// Steady incompressible Navier-Stokes VMS/NSGS element build with bubble
// condensation (04_SS_NavierStokes_Equations/2D/01_CommonFiles/
// Build_K_F_MS.c:8-1190, the branch it executes; eval_U.c:3-36) and the
// vector updates of the damped Newton loop (Process.c:97-166).
//
// One thread per element computes the 9x9 tangent Ke (dof order u1 v1 p1 u2
// v2 p2 u3 v3 p3), the 9 residual entries and updates the element's
// stabilisation state (delta_old, normres_old); Ke goes straight into the
// 3-dof block-EBE storage.  The residual is assembled per equation over the
// incident elements in ascending element order (the order of the reference's
// scatter, :1083-1086), so F is bit-identical.  Compiled without FMA
// contraction; FP64-issue bound on GB300.
#include "fg_common.cuh"
#include "fg_ns.h"

struct NSCoef {
	double re;
	int first, neq;
};

__device__ __forceinline__ double ns_delta_aux(double normgradU, double hRGN, double normres, double cont)
{
	const double coe01 = 1.0, coe02 = 1.0;
	if (normgradU > 1e-5) return (coe01 * hRGN * normres / normgradU + coe02 * hRGN * hRGN * sqrt(cont * cont)) / 2.0;
	return 0.0;
}

__device__ __forceinline__ double ns_hrgn(double ux, double uy, const double *yb, const double *xb, double Area,
                                          double unorm)
{
	double auxh = fabs(ux * yb[0] + uy * xb[0]) + fabs(ux * yb[1] + uy * xb[1]) + fabs(ux * yb[2] + uy * xb[2]);
	return fabs(auxh) >= 1e-6 ? 4 * Area * unorm / auxh : 0.0;
}

__global__ void __launch_bounds__(128) k_ns_element(int nel, const int *__restrict__ vert,
		const int *__restrict__ node_id, const double *__restrict__ xn, const double *__restrict__ yn,
		const double *__restrict__ upresc, const double *__restrict__ fnod, const double *__restrict__ u,
		NSCoef cf, double *dold_a, double *nold_a, double *__restrict__ A, double *__restrict__ Re)
{
	const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, ninefortieth = 9.0 / 40.0, ninetwentieth = 9.0 / 20.0,
	             twelfth = 1.0 / 12.0, epsilon = 1e-7, coefnorm = 0.8, w = 0.5, rho = 1.;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		double X[3], Y[3], yb[3], xb[3], uxn[3], uyn[3], pn[3], fx[3], fy[3];
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			int J = __ldg(&vert[3 * e + a]);
			X[a] = __ldg(&xn[J]);
			Y[a] = __ldg(&yn[J]);
			double U3[3];
			#pragma unroll
			for (int k = 0; k < 3; k++) {                        // eval_U.c:13-35
				int id = __ldg(&node_id[3 * J + k]);
				U3[k] = id >= 0 ? __ldg(&u[id]) : __ldg(&upresc[3 * J + k]);
			}
			uxn[a] = U3[0]; uyn[a] = U3[1]; pn[a] = U3[2];
			fx[a] = __ldg(&fnod[2 * J]);
			fy[a] = __ldg(&fnod[2 * J + 1]);
		}
		yb[0] = Y[1] - Y[2]; yb[1] = Y[2] - Y[0]; yb[2] = Y[0] - Y[1];
		xb[0] = X[2] - X[1]; xb[1] = X[0] - X[2]; xb[2] = X[1] - X[0];
		double twoArea = fabs(xb[2] * yb[1] - xb[1] * yb[2]), Area = 0.5 * twoArea, invArea = 1.0 / Area;
		double ux = third * (uxn[0] + uxn[1] + uxn[2]), uy = third * (uyn[0] + uyn[1] + uyn[2]);
		double duxdx = 0.5 * invArea * (uxn[0] * yb[0] + uxn[1] * yb[1] + uxn[2] * yb[2]);
		double duxdy = 0.5 * invArea * (uxn[0] * xb[0] + uxn[1] * xb[1] + uxn[2] * xb[2]);
		double duydx = 0.5 * invArea * (uyn[0] * yb[0] + uyn[1] * yb[1] + uyn[2] * yb[2]);
		double duydy = 0.5 * invArea * (uyn[0] * xb[0] + uyn[1] * xb[1] + uyn[2] * xb[2]);
		double duxduy = uxn[0] * yb[0] + uyn[0] * xb[0] + uxn[1] * yb[1] + uyn[1] * xb[1] + uxn[2] * yb[2] +
		                uyn[2] * xb[2];
		double p = third * (pn[0] + pn[1] + pn[2]);
		double dpdx = 0.5 * invArea * (pn[0] * yb[0] + pn[1] * yb[1] + pn[2] * yb[2]);
		double dpdy = 0.5 * invArea * (pn[0] * xb[0] + pn[1] * xb[1] + pn[2] * xb[2]);
		double h = sqrt(twoArea), visc = 1. / cf.re;
		double unorm = sqrt(ux * ux + uy * uy);
		double tau_l = 0.333 * h * unorm;
		double fxB = third * (fx[0] + fx[1] + fx[2]), fyB = third * (fy[0] + fy[1] + fy[2]);
		double f1 = rho * third * Area * fxB, f2 = rho * third * Area * fyB;
		double f1B = rho * ninetwentieth * Area * fxB, f2B = rho * ninetwentieth * Area * fyB;
		double dold = dold_a[e], nold = nold_a[e];

		// first pass: the bubble velocity from the macro field
		double ne1 = ux * duxdx + uy * duydx + dpdx - f1, ne2 = ux * duxdy + uy * duydy + dpdy - f2;
		double cont = duxdx + duydy;
		double normres = sqrt(ne1 * ne1 + ne2 * ne2);
		double normgradU = sqrt(duxdx * duxdx + duxdy * duxdy + duydx * duydx + duydy * duydy);
		double hR = ns_hrgn(ux, uy, yb, xb, Area, unorm);
		double da = ns_delta_aux(normgradU, hR, normres, cont);
		double deltam = (cf.first || normres < coefnorm * nold) ? w * da + (1 - w) * dold : dold;
		double A_ = yb[0] * yb[0] + yb[1] * yb[1] + yb[2] * yb[2] + yb[0] * yb[1] + yb[0] * yb[2] + yb[1] * yb[2];
		double B_ = xb[0] * xb[0] + xb[1] * xb[1] + xb[2] * xb[2] + xb[0] * xb[1] + xb[0] * xb[2] + xb[1] * xb[2];
		double C_ = yb[0] * xb[0] + yb[1] * xb[1] + yb[2] * xb[2];
		const double NBB = 0.0;
		double KBB11 = 81.0 * ((2 * visc + deltam) * A_ + (visc + deltam) * B_) / (40.0 * Area) + NBB;
		double KBB12 = 81.0 * visc * C_ / (80.0 * Area);
		double KBB22 = 81.0 * ((2 * visc + deltam) * B_ + (visc + deltam) * A_) / (40.0 * Area) + NBB;
		double D = KBB11 * KBB22 - KBB12 * KBB12;
		double I11 = KBB22 / D, I12 = -KBB12 / D, I22 = KBB11 / D;
		double NBh[3], G0[3], G1[3];
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			NBh[a] = rho * ninefortieth * (ux * yb[a] + uy * xb[a]);
			G0[a] = -ninefortieth * yb[a];
			G1[a] = -ninefortieth * xb[a];
		}
		{
			double r1 = f1B - (NBh[0] * uxn[0] + NBh[1] * uxn[1] + NBh[2] * uxn[2]) +
			            (G0[0] * pn[0] + G0[1] * pn[1] + G0[2] * pn[2]);
			double r2 = f2B - (NBh[0] * uyn[0] + NBh[1] * uyn[1] + NBh[2] * uyn[2]) +
			            (G1[0] * pn[0] + G1[1] * pn[1] + G1[2] * pn[2]);
			double uxB = I11 * r1 + I12 * r2, uyB = I12 * r1 + I22 * r2;
			ux = ux + uxB;
			uy = uy + uyB;
		}
		double N1[3];
		#pragma unroll
		for (int a = 0; a < 3; a++) N1[a] = rho * third * Area * (0.5 * invArea * (ux * yb[a] + uy * xb[a]));
		const double kv = visc * 0.25 * invArea, ks = tau_l * rho * 0.25 * invArea;
		const double C11 = epsilon * Area * sixth, C12 = epsilon * Area * twelfth;
		double Nv0 = rho * third * Area * (duxdx * ux + duxdy * uy), Nv1 = rho * third * Area * (duydx * ux + duydy * uy);
		double GTv = third * Area * (duxdx + duydy);

		// second pass: stabilisation state with the total velocity
		ne1 = ux * duxdx + uy * duydx + dpdx - f1;
		ne2 = ux * duxdy + uy * duydy + dpdy - f2;
		normres = sqrt(ne1 * ne1 + ne2 * ne2);
		normgradU = sqrt(duxdx * duxdx + duydy * duydy + duxdy * duxdy + duydx * duydx);
		unorm = sqrt(ux * ux + uy * uy);
		hR = ns_hrgn(ux, uy, yb, xb, Area, unorm);
		da = ns_delta_aux(normgradU, hR, normres, cont);
		double delta;
		if (cf.first || normres < coefnorm * nold) {
			delta = w * da + (1 - w) * dold;
			dold_a[e] = delta;
		} else {
			delta = dold;
		}
		nold_a[e] = normres;
		deltam = delta;
		delta = 0.0;
		KBB11 = 81.0 * ((2 * visc + deltam) * A_ + (visc + deltam) * B_) / (40.0 * Area) + NBB;
		KBB12 = 81.0 * visc * C_ / (80.0 * Area);
		KBB22 = 81.0 * ((2 * visc + deltam) * B_ + (visc + deltam) * A_) / (40.0 * Area) + NBB;
		D = KBB11 * KBB22 - KBB12 * KBB12;
		I11 = KBB22 / D; I12 = -KBB12 / D; I22 = KBB11 / D;
		const double Inv[2][2] = {{I11, I12}, {I12, I22}};
		double delta4area = delta / (4.0 * Area), NhB[3];
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			NBh[a] = rho * ninefortieth * (ux * yb[a] + uy * xb[a]);
			NhB[a] = -NBh[a];
		}
		double Nd[6][6], Gd[6][3], Gphi[3][3];
		#pragma unroll
		for (int a = 0; a < 3; a++)
			#pragma unroll
			for (int i = 0; i < 2; i++)
				#pragma unroll
				for (int b = 0; b < 3; b++) {
					#pragma unroll
					for (int j = 0; j < 2; j++) Nd[2 * a + i][2 * b + j] = NhB[a] * Inv[i][j] * NBh[b];
					Gd[2 * a + i][b] = NhB[a] * Inv[i][0] * G0[b] + NhB[a] * Inv[i][1] * G1[b];
				}
		#pragma unroll
		for (int a = 0; a < 3; a++)
			#pragma unroll
			for (int b = 0; b < 3; b++)
				Gphi[a][b] = G0[b] * (G0[a] * I11 + G1[a] * I12) + G1[b] * (G0[a] * I12 + G1[a] * I22);

		const double uv[6] = {uxn[0], uyn[0], uxn[1], uyn[1], uxn[2], uyn[2]};
		const double shear = duxdy + duydx;
		double *re = Re + (long long)e * 9;
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			double fe0 = f1 + (-(NhB[a] * I11 * f1B + NhB[a] * I12 * f2B));
			double fe1 = f2 + (-(NhB[a] * I12 * f1B + NhB[a] * I22 * f2B));
			double fe2 = -((G0[a] * I11 + G1[a] * I12) * f1B + (G0[a] * I12 + G1[a] * I22) * f2B);
			double Kv[2] = {0.5 * visc * (2 * yb[a] * duxdx + xb[a] * shear), 0.5 * visc * (2 * xb[a] * duydy + yb[a] * shear)};
			double Kdd[2] = {0.5 * delta * (yb[a] * duxdx + xb[a] * duxdy), 0.5 * delta * (yb[a] * duydx + xb[a] * duydy)};
			double ga[2] = {yb[a], xb[a]};
			#pragma unroll
			for (int i = 0; i < 2; i++) {
				int r = 2 * a + i;
				double ndv = Nd[r][0] * uv[0] + Nd[r][1] * uv[1] + Nd[r][2] * uv[2] + Nd[r][3] * uv[3] + Nd[r][4] * uv[4] +
				             Nd[r][5] * uv[5];
				double gdv = Gd[r][0] * pn[0] + Gd[r][1] * pn[1] + Gd[r][2] * pn[2];
				double Ksv = ks * ga[i] * duxduy, Gv = 0.5 * p * ga[i];
				re[3 * a + i] = (i == 0 ? fe0 : fe1) - ((i == 0 ? Nv0 : Nv1) - ndv + Kv[i] + Ksv + Kdd[i] - (Gv - gdv));
			}
			const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
			double Cv = C11 * pn[a] + C12 * (pn[o1] + pn[o2]);
			double Nphiv = -Gd[0][a] * uv[0];
			#pragma unroll
			for (int q = 1; q < 6; q++) Nphiv = Nphiv + (-Gd[q][a] * uv[q]);
			double Gphiv = Gphi[a][0] * pn[0] + Gphi[a][1] * pn[1] + Gphi[a][2] * pn[2];
			re[3 * a + 2] = fe2 - (GTv + Cv - Nphiv + Gphiv);
		}

		double *Ke = A + (long long)e * 81;
		#pragma unroll
		for (int a = 0; a < 3; a++)
			#pragma unroll
			for (int b = 0; b < 3; b++) {
				const int lo = a < b ? a : b, hi = a < b ? b : a;
				double kdd = delta4area * (yb[lo] * yb[hi] + xb[lo] * xb[hi]);
				const double ga[2] = {yb[a], xb[a]}, gb[2] = {yb[b], xb[b]};
				#pragma unroll
				for (int i = 0; i < 2; i++) {
					#pragma unroll
					for (int j = 0; j < 2; j++) {
						double K = (i == 0 && j == 0) ? kv * (2 * yb[a] * yb[b] + xb[a] * xb[b])
						         : (i == 1 && j == 1) ? kv * (yb[a] * yb[b] + 2 * xb[a] * xb[b])
						         : (i == 0) ? kv * (xb[a] * yb[b]) : kv * (yb[a] * xb[b]);
						double Ks = ks * gb[j] * ga[i];
						double val;
						if (i == j) {
							// coupling read from the (lower node, higher node) entry; added for
							// the (3, 2) pair's x component (Build_K_F_MS.c:939)
							double nd = Nd[2 * lo + i][2 * hi + i];
							double t = (a == 2 && b == 1 && i == 0) ? N1[b] + nd : N1[b] - nd;
							val = t + K + Ks + kdd;
						} else {
							val = K + Ks;
						}
						Ke[9 * (3 * a + i) + 3 * b + j] = val;
					}
					Ke[9 * (3 * a + i) + 3 * b + 2] = -((i == 0 ? sixth * yb[a] : sixth * xb[a]) - Gd[2 * a + i][b]);
				}
				#pragma unroll
				for (int j = 0; j < 2; j++)
					Ke[9 * (3 * a + 2) + 3 * b + j] = (j == 0 ? sixth * yb[b] : sixth * xb[b]) - (-Gd[2 * b + j][a]);
				Ke[9 * (3 * a + 2) + 3 * b + 2] = Gphi[lo][hi] + (a == b ? C11 : C12);
			}
	}
}

// F[I] = sum of the incident elements' residual entries in element order.
__global__ void k_ns_gather(int neq, const int *__restrict__ ri_ptr, const int *__restrict__ ri,
                            const double *__restrict__ Re, double *__restrict__ F)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double s = 0.0;
		if (I < neq)
			for (int t = ri_ptr[I]; t < ri_ptr[I + 1]; t++) s += __ldg(&Re[__ldg(&ri[t])]);
		F[I] = s;
	}
}

// y += a x on n entries (daxpy, BLAS_Operations/daxpy.c).
__global__ void k_ns_axpy(int n, double a, const double *x, double *y)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += a * x[i];
}

extern "C" int fg_ns_build(femgpu_ns *c, int first)
{
	NSCoef cf;
	cf.re = c->o.re;
	cf.first = first;
	cf.neq = c->neq;
	femgpu_ebe *b = c->ebe;
	int g = (int)((c->nel + 127LL) / 128);
	k_ns_element<<<g, 128, 0, c->stream>>>(c->nel, b->vert, b->node_id, c->x, c->y, c->upresc, c->f, c->u, cf,
	                                       c->dold, c->nold, b->A, c->Re);
	FG_TRY(cudaGetLastError());
	k_ns_gather<<<fg_grid(c->neq + 1LL), FG_TPB, 0, c->stream>>>(c->neq, b->ri_ptr, b->ri, c->Re, c->F);
	return (int)cudaGetLastError();
}

extern "C" int fg_ns_axpy(femgpu_ns *c, double a, const double *x, double *y)
{
	k_ns_axpy<<<fg_grid(c->neq), FG_TPB, 0, c->stream>>>(c->neq, a, x, y);
	return (int)cudaGetLastError();
}
