// Pieces of the 2D Euler element builds shared by the SUPG and the DD build
// (03_Euler_Equations/2D/01_CommonFiles), written once for the device and,
// compiled as plain C++, for host checks: the flux Jacobians
// (Ax_Ay_calculations.c), A0^-1 in entropy variables (Build_M_K_F_SUPG.c:
// 131-159, the same lines in Build_M_K_F_DD_Transiente.c:131-162), the
// YZBeta and DD shock-capturing parameters (Delta_YZBeta.c:6-108,
// Delta_DD.c:4-89) and the DD element (Build_M_K_F_DD_Transiente.c:37-911).
// Every expression keeps the reference's evaluation order; the translation
// units that include this file are compiled without FMA contraction.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define FG_HD __host__ __device__ __forceinline__
#else
#define FG_HD inline
#endif

// Ax_Ay_calculations.c: dimensional (:3-51) or dimensionless (:54-98) form.
FG_HD void euler_jacobians(const double *Ub, double gamma, double mach, int dimensionless, double (&Ax)[4][4],
                           double (&Ay)[4][4])
{
	double v1 = Ub[1] / Ub[0], v2 = Ub[2] / Ub[0], E = Ub[3] / Ub[0];
	double nU23 = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++) { Ax[i][j] = 0.0; Ay[i][j] = 0.0; }
	Ax[0][1] = 1.0;
	Ay[0][2] = 1.0;
	if (!dimensionless) {
		double rho = Ub[0], r2 = rho * rho;
		Ax[1][0] = -(v1 * v1) + (((gamma - 1) * nU23 * 0.5) / r2);
		Ax[1][1] = (3.0 - gamma) * v1;
		Ax[1][2] = -(gamma - 1.0) * v2;
		Ax[1][3] = gamma - 1.0;
		Ax[2][0] = -v1 * v2;
		Ax[2][1] = v2;
		Ax[2][2] = v1;
		Ax[3][0] = (-gamma * v1 * E) + ((gamma - 1.0) * v1 * (nU23 / r2));
		Ax[3][1] = (gamma * E) - ((gamma - 1.0) * 0.5 * ((nU23 / r2) + (2.0 * v1 * v1)));
		Ax[3][2] = -((gamma - 1.0) * v1 * v2);
		Ax[3][3] = gamma * v1;
		Ay[2][0] = -(v2 * v2) + (((gamma - 1.0) * nU23 * 0.5) / r2);
		Ay[3][0] = (-gamma * v2 * E) + (((gamma - 1.0) * v2 * nU23) / r2);
		Ay[3][2] = (gamma * E) - ((gamma - 1.0) * 0.5 * ((nU23 / r2) + (2.0 * v2 * v2)));
	} else {
		double nv = v1 * v1 + v2 * v2, eps2 = mach * mach;
		Ax[1][0] = -(v1 * v1) + ((gamma - 1) * nv * 0.5);
		Ax[1][1] = (3.0 - gamma) * v1;
		Ax[1][2] = -(gamma - 1.0) * v2;
		Ax[1][3] = (gamma - 1.0) / eps2;
		Ax[2][0] = -v1 * v2;
		Ax[2][1] = v2;
		Ax[2][2] = v1;
		Ax[3][0] = -v1 * (gamma * E - ((gamma - 1.0) * eps2 * nv));
		Ax[3][1] = gamma * E - (gamma - 1.0) * eps2 * (0.5 * nv + v1 * v1);
		Ax[3][2] = -(gamma - 1.0) * eps2 * v1 * v2;
		Ax[3][3] = gamma * v1;
		Ay[2][0] = -(v2 * v2) + (((gamma - 1.0) * nv * 0.5));
		Ay[3][0] = -v2 * (gamma * E - (gamma - 1.0) * eps2 * nv);
		Ay[3][2] = gamma * E - (gamma - 1.0) * eps2 * (0.5 * nv + v2 * v2);
	}
	Ay[1][0] = Ax[2][0];
	Ay[1][1] = v2;
	Ay[1][2] = v1;
	Ay[2][1] = -(gamma - 1.0) * v1;
	Ay[2][2] = (3.0 - gamma) * v2;
	Ay[2][3] = Ax[1][3];
	Ay[3][1] = Ax[3][2];
	Ay[3][3] = gamma * v2;
}

// A0^-1 in entropy variables at the centroid state.
FG_HD void euler_a0(const double *Ub, double gamma, double (&A0)[4][4])
{
	double nU23 = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
	double rho_i = Ub[3] - ((nU23 * 0.5) / Ub[0]);
	double V2 = Ub[1] / rho_i, V3 = Ub[2] / rho_i, V4 = (-Ub[0]) / rho_i;
	double re = -1.0 / (rho_i * V4), k1 = (V2 * V2 + V3 * V3) * 0.5 / V4;
	A0[0][0] = re * (k1 * k1 + gamma);
	A0[0][1] = re * (k1 * V2);
	A0[0][2] = re * (k1 * V3);
	A0[0][3] = re * ((k1 + 1.0) * V4);
	A0[1][1] = re * (V2 * V2 - V4);
	A0[1][2] = re * (V2 * V3);
	A0[1][3] = re * (V2 * V4);
	A0[2][2] = re * (V3 * V3 - V4);
	A0[2][3] = re * (V3 * V4);
	A0[3][3] = re * V4 * V4;
	A0[1][0] = A0[0][1]; A0[2][0] = A0[0][2]; A0[3][0] = A0[0][3];
	A0[2][1] = A0[1][2]; A0[3][1] = A0[1][3]; A0[3][2] = A0[2][3];
}

// Ax gradUx + Ay gradUy with the terms the reference writes (Delta_CAU.c:
// 18-26, Delta_DD.c:17-25, Delta_YZBeta.c:16-24: Ax[2][3] and Ay[1][3] are
// structural zeros left out, row 0 the unit entry alone), plus dUb.
FG_HD void euler_residual4(const double (&Ax)[4][4], const double (&Ay)[4][4], const double *gx, const double *gy,
                           const double *dUb, double *L)
{
	const double ax0 = gx[1];
	const double ax1 = Ax[1][0] * gx[0] + Ax[1][1] * gx[1] + Ax[1][2] * gx[2] + Ax[1][3] * gx[3];
	const double ax2 = Ax[2][0] * gx[0] + Ax[2][1] * gx[1] + Ax[2][2] * gx[2];
	const double ax3 = Ax[3][0] * gx[0] + Ax[3][1] * gx[1] + Ax[3][2] * gx[2] + Ax[3][3] * gx[3];
	const double ay0 = gy[2];
	const double ay1 = Ay[1][0] * gy[0] + Ay[1][1] * gy[1] + Ay[1][2] * gy[2];
	const double ay2 = Ay[2][0] * gy[0] + Ay[2][1] * gy[1] + Ay[2][2] * gy[2] + Ay[2][3] * gy[3];
	const double ay3 = Ay[3][0] * gy[0] + Ay[3][1] * gy[1] + Ay[3][2] * gy[2] + Ay[3][3] * gy[3];
	L[0] = dUb[0] + ax0 + ay0;
	L[1] = dUb[1] + ax1 + ay1;
	L[2] = dUb[2] + ax2 + ay2;
	L[3] = dUb[3] + ax3 + ay3;
}

// v^T A0 v as Delta_CAU.c / Delta_DD.c write the quadratic form.
FG_HD double euler_a0norm2(const double (&A0)[4][4], const double *v)
{
	return v[0] * (A0[0][0] * v[0] + 2.0 * A0[0][1] * v[1] + 2.0 * A0[0][2] * v[2] + 2.0 * A0[0][3] * v[3]) +
	       v[1] * (A0[1][1] * v[1] + 2.0 * A0[1][2] * v[2] + 2.0 * A0[1][3] * v[3]) +
	       v[2] * (A0[2][2] * v[2] + 2.0 * A0[2][3] * v[3]) +
	       v[3] * A0[3][3] * v[3];
}

// Delta_YZBeta.c:6-108: *dold (the element's previous delta) is blended in
// and replaced.  yb = (y23, y31, y12), xb = (x32, x13, x21).
FG_HD double euler_delta_yzbeta(const double *Z, const double *gx, const double *gy, const double *Ub,
                                const double *iY, const double *yb, const double *xb, double twoArea, double *dold)
{
	double nYZ = sqrt(iY[0] * Z[0] * iY[0] * Z[0] + iY[1] * Z[1] * iY[1] * Z[1] +
	                  iY[2] * Z[2] * iY[2] * Z[2] + iY[3] * Z[3] * iY[3] * Z[3]);
	double nYx = iY[0] * gx[0] * iY[0] * gx[0] + iY[1] * gx[1] * iY[1] * gx[1] +
	             iY[2] * gx[2] * iY[2] * gx[2] + iY[3] * gx[3] * iY[3] * gx[3];
	double nYy = iY[0] * gy[0] * iY[0] * gy[0] + iY[1] * gy[1] * iY[1] * gy[1] +
	             iY[2] * gy[2] * iY[2] * gy[2] + iY[3] * gy[3] * iY[3] * gy[3];
	double sYdU = nYx + nYy;
	double nYU = sqrt(iY[0] * Ub[0] * iY[0] * Ub[0] + iY[1] * Ub[1] * iY[1] * Ub[1] +
	                  iY[2] * Ub[2] * iY[2] * Ub[2] + iY[3] * Ub[3] * iY[3] * Ub[3]);
	double nrho = sqrt(gx[0] * gx[0] + gy[0] * gy[0]), J1 = 0.0, J2 = 0.0;
	if (fabs(nrho) >= 1e-12) { J1 = gx[0] / nrho; J2 = gy[0] / nrho; }
	double H = (fabs(J1 * yb[0] + J2 * xb[0]) + fabs(J1 * yb[1] + J2 * xb[1]) +
	            fabs(J1 * yb[2] + J2 * xb[2])) / twoArea;
	H = fabs(H) >= 1e-12 ? 2.0 * (1.0 / H) : 0.0;
	const bool sok = fabs(sYdU) >= 1e-12, uok = fabs(nYU) >= 1e-12;
	double d1 = nYZ * (sok ? 1.0 / sqrt(sYdU) : 0.0) * (uok ? 1.0 : 0.0) * (H * 0.5);
	double d2 = nYZ * (sok ? 1.0 : 0.0) * (uok ? 1.0 / nYU : 0.0) * (H * 0.5 * H * 0.5);
	const double w = 0.5;
	double ad = w * (d1 + d2);
	double delta = w * (ad) + (1 - w) * (*dold);
	*dold = delta;
	return delta;
}

// Delta_DD.c:4-89 (ShockCapture "CAUDD" of the DD build): the CAU ratio
// under the tolerance switch, blended with the element's previous value
// (which it replaces), then scaled by sqrt(2 Area).
FG_HD double euler_delta_dd(const double *L, const double *gx, const double *gy, const double (&A0)[4][4],
                            const double *yb, const double *xb, double twoArea, double tol, double *dold)
{
	double kx[4], ky[4];
	for (int i = 0; i < 4; i++) {
		kx[i] = (yb[0] * gx[i] + xb[0] * gy[i]) / twoArea;
		ky[i] = (yb[1] * gx[i] + xb[1] * gy[i]) / twoArea;
	}
	double nk = sqrt(euler_a0norm2(A0, kx) + euler_a0norm2(A0, ky));
	double nL = sqrt(euler_a0norm2(A0, L));
	double ng = sqrt(euler_a0norm2(A0, gx) + euler_a0norm2(A0, gy));
	double aux = ng >= tol ? 0.5 * nL / nk : 0.0;
	const double w = 0.5;
	double delta = w * (aux) + (1 - w) * (*dold);
	*dold = delta;
	return delta * sqrt(twoArea);
}

// Build_M_K_F_DD_Transiente.c:37-911 for one element: the bubble condensed
// out of the 12x12 matrices, Ae = Me + alpha dt Ke into Ae [144] (row-major),
// the element residual entries N + Re into Re [12], the element's bubble uB
// [4] advanced, delta from euler_delta_dd or euler_delta_yzbeta (yz != 0).
FG_HD void euler_dd_element(const double *X, const double *Y, const double *Ue, const double *dUe, double gamma,
                            double mach, int dimensionless, double alpha, double delta_t, double tol, int yz,
                            const double *invY, double *dold, double *uB, double *Ae, double *Re)
{
	const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, ninefortieth = 9.0 / 40.0;
	double yb[3], xb[3];
	yb[0] = Y[1] - Y[2]; yb[1] = Y[2] - Y[0]; yb[2] = Y[0] - Y[1];             // y23 y31 y12
	xb[0] = X[2] - X[1]; xb[1] = X[0] - X[2]; xb[2] = X[1] - X[0];             // x32 x13 x21
	const double twoArea = fabs(xb[2] * yb[1] - xb[1] * yb[2]);
	const double Area = 0.5 * twoArea;
	double Ub[4], dUb[4], gx[4], gy[4], uBaux[4];
	for (int i = 0; i < 4; i++) {
		Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
		dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
		uBaux[i] = uB[i];
	}
	for (int i = 0; i < 4; i++) {
		gx[i] = (Ue[i] * yb[0] + Ue[i + 4] * yb[1] + Ue[i + 8] * yb[2]) / twoArea;
		gy[i] = (Ue[i] * xb[0] + Ue[i + 4] * xb[1] + Ue[i + 8] * xb[2]) / twoArea;
	}
	double Ax[4][4], Ay[4][4], A0[4][4], L[4];
	euler_jacobians(Ub, gamma, mach, dimensionless, Ax, Ay);
	euler_a0(Ub, gamma, A0);
	euler_residual4(Ax, Ay, gx, gy, dUb, L);
	const double delta = yz ? euler_delta_yzbeta(L, gx, gy, Ub, invY, yb, xb, twoArea, dold)
	                        : euler_delta_dd(L, gx, gy, A0, yb, xb, twoArea, tol, dold);

	// K_b = yb[b] Ax + xb[b] Ay (Ka, Kb, Kc of :172-225); Khhg = K_b / 6 in
	// every row block, KBh = 9/40 K_b, KhB of node a = (c_a1 Ax + c_a2 Ay)
	double K[3][4][4];
	for (int b = 0; b < 3; b++)
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++) K[b][i][j] = yb[b] * Ax[i][j] + xb[b] * Ay[i][j];
	const double Mhh1 = Area * sixth, Mhh2 = Area / 12.0;
	const double MhB = (3.0 * Area) / 20.0, MBB = (81.0 * Area) / 280.0;
	const double delta4area = delta / (4.0 * Area);
	double Kdd[3][3];
	for (int a = 0; a < 3; a++)
		for (int b = a; b < 3; b++) Kdd[a][b] = Kdd[b][a] = delta4area * (yb[a] * yb[b] + xb[a] * xb[b]);
	// (a1, a2), (b1, b2), (c1, c2) of :306-311
	double cy[3], cx[3];
	cy[0] = ninefortieth * (yb[0] + 2.0 * yb[1] + 2.0 * yb[2]);
	cx[0] = ninefortieth * (xb[0] + 2.0 * xb[1] + 2.0 * xb[2]);
	cy[1] = ninefortieth * (2.0 * yb[0] + yb[1] + 2.0 * yb[2]);
	cx[1] = ninefortieth * (2.0 * xb[0] + xb[1] + 2.0 * xb[2]);
	cy[2] = ninefortieth * (2.0 * yb[0] + 2.0 * yb[1] + yb[2]);
	cx[2] = ninefortieth * (2.0 * xb[0] + 2.0 * xb[1] + xb[2]);
	const double KBB = (81.0 * delta * (yb[0] * yb[0] + yb[1] * yb[1] + yb[2] * yb[2] + yb[0] * yb[1] + yb[0] * yb[2] +
	                                    yb[1] * yb[2] + xb[0] * xb[0] + xb[1] * xb[1] + xb[2] * xb[2] + xb[0] * xb[1] +
	                                    xb[0] * xb[2] + xb[1] * xb[2])) / (40.0 * Area);
	const double invBB = 1.0 / (MBB + delta_t * KBB);
	const double invdelta_t = 1.0 / delta_t;
	const double adt = alpha * delta_t;
	// P = (MBB + dt KBB)^-1 (MhB + dt KhB), row 4a + i (:437-486)
	double P[12][4];
	for (int a = 0; a < 3; a++)
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++) {
				const double khb = cy[a] * Ax[i][j] + cx[a] * Ay[i][j];
				P[4 * a + i][j] = i == j ? invBB * (MhB + delta_t * khb) : invBB * delta_t * khb;
			}
	double KBh[3][4][4];
	for (int b = 0; b < 3; b++)
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++) KBh[b][i][j] = ninefortieth * K[b][i][j];
	for (int a = 0; a < 3; a++)
		for (int i = 0; i < 4; i++) {
			const int r = 4 * a + i;
			double MedUe = 0.0, KeUe = 0.0;
			for (int b = 0; b < 3; b++)
				for (int j = 0; j < 4; j++) {
					const int c = 4 * b + j;
					// Me (:488-649): Mhh - P MhB on the component diagonal
					const double me = i == j ? (a == b ? Mhh1 : Mhh2) - P[r][j] * MhB : -P[r][j] * MhB;
					// Ke (:651-814): Khhg (+ Khhdd) - P KBh
					double ke = K[b][i][j] * sixth;
					if (i == j) ke = ke + Kdd[a][b];
					ke = ke - P[r][0] * KBh[b][0][j];
					ke = ke - P[r][1] * KBh[b][1][j];
					ke = ke - P[r][2] * KBh[b][2][j];
					ke = ke - P[r][3] * KBh[b][3][j];
					MedUe += me * dUe[c];
					KeUe += ke * Ue[c];
					Ae[12 * r + c] = me + adt * ke;
				}
			// Ne (:816-870) times uBaux
			double N = 0.0;
			for (int k = 0; k < 4; k++) {
				const double ne = (i == k ? MhB - P[r][k] * MBB : -P[r][k] * MBB) * invdelta_t;
				N = k == 0 ? ne * uBaux[0] : N + ne * uBaux[k];
			}
			const double re = -MedUe - KeUe;
			Re[r] = N + re;
		}
	// the bubble's new value (:888-895)
	for (int k = 0; k < 4; k++) {
		double s = KBh[0][k][0] * Ue[0];
		for (int b = 0; b < 3; b++)
			for (int j = 0; j < 4; j++)
				if (b || j) s = s + KBh[b][k][j] * Ue[4 * b + j];
		uB[k] = invBB * (MBB * uBaux[k] - delta_t * MhB * (dUe[k] + dUe[k + 4] + dUe[k + 8]) - delta_t * s);
	}
}
