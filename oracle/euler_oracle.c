/*
 * Test infrastructure only -- CPU oracle for the 2D Euler SUPG+CAU element
 * build and predictor-multicorrector (mod-comp-ufes/FEM_CODES,
 * 03_Euler_Equations/2D/01_CommonFiles and 00_CommonFiles/Time_Integration).
 * A restatement in this project's own code; every floating-point expression
 * keeps the reference's operation order so that, compiled without contraction
 * or reassociation, element matrices and residuals are bit-identical to the
 * reference's own sources (pinned by tests/golden/euler_*.npz).  Never linked
 * into the product.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Structure of the flux Jacobians (Ax_Ay_calculations.c:3-98): 0 structural
 * zero, 1 unit entry, 2 general.  The reference's hand-expanded products
 * (Build_M_K_F_SUPG.c:163-237), Delta_CAU.c:18-26 and the C matrices
 * (:277-332) leave out exactly the terms with a structural zero factor and
 * write a unit factor's partner alone; summing the remaining terms in
 * ascending inner index reproduces them. */
static const unsigned char KAX[4][4] = {{0, 1, 0, 0}, {2, 2, 2, 2}, {2, 2, 2, 0}, {2, 2, 2, 2}};
static const unsigned char KAY[4][4] = {{0, 0, 1, 0}, {2, 2, 2, 0}, {2, 2, 2, 2}, {2, 2, 2, 2}};

static double jprod(const double X[4][4], const unsigned char KX[4][4], const double Y[4][4],
                    const unsigned char KY[4][4], int i, int j)
{
	double s = 0.0, t;
	int k, first = 1;
	for (k = 0; k < 4; k++) {
		if (!KX[i][k] || !KY[k][j]) continue;
		t = KX[i][k] == 1 ? Y[k][j] : (KY[k][j] == 1 ? X[i][k] : X[i][k]*Y[k][j]);
		s = first ? t : s + t;
		first = 0;
	}
	return s;
}

static double jvec(const double X[4][4], const unsigned char KX[4][4], const double *g, int i)
{
	double s = 0.0, t;
	int k, first = 1;
	for (k = 0; k < 4; k++) {
		if (!KX[i][k]) continue;
		t = KX[i][k] == 1 ? g[k] : X[i][k]*g[k];
		s = first ? t : s + t;
		first = 0;
	}
	return s;
}

/* dimensional_Ax_Ay_calculations (Ax_Ay_calculations.c:54-98) and the
 * dimensionless variant (:3-52); Ay[0][3] is never written there and acts as 0. */
static void jacobians(int dimensionless, double gamma, double mach, const double *Ub, double Ax[4][4],
                      double Ay[4][4])
{
	double rho = Ub[0], v1 = Ub[1]/Ub[0], v2 = Ub[2]/Ub[0], E = Ub[3]/Ub[0];
	memset(Ax, 0, 16 * sizeof(double));
	memset(Ay, 0, 16 * sizeof(double));
	Ax[0][1] = 1.0;
	Ay[0][2] = 1.0;
	if (!dimensionless) {
		double nU = (Ub[1]*Ub[1]) + (Ub[2]*Ub[2]);
		Ax[1][0] = -(v1*v1) + (((gamma - 1)*nU*0.5)/(rho*rho));
		Ax[1][1] = (3.0 - gamma)*v1;
		Ax[1][2] = -(gamma - 1.0)*v2;
		Ax[1][3] = gamma - 1.0;
		Ax[2][0] = -v1*v2;
		Ax[2][1] = v2;
		Ax[2][2] = v1;
		Ax[3][0] = (-gamma*v1*E) + ((gamma - 1.0)*v1*(nU/(rho*rho)));
		Ax[3][1] = (gamma*E) - ((gamma - 1.0)*0.5*((nU/(rho*rho)) + (2.0*v1*v1)));
		Ax[3][2] = -((gamma - 1.0)*v1*v2);
		Ax[3][3] = gamma*v1;
		Ay[1][0] = Ax[2][0];
		Ay[1][1] = v2;
		Ay[1][2] = v1;
		Ay[2][0] = -(v2*v2) + (((gamma - 1.0)*nU*0.5)/(rho*rho));
		Ay[2][1] = -(gamma - 1.0)*v1;
		Ay[2][2] = (3.0 - gamma)*v2;
		Ay[2][3] = Ax[1][3];
		Ay[3][0] = (-gamma*v2*E) + (((gamma - 1.0)*v2*nU)/(rho*rho));
		Ay[3][1] = Ax[3][2];
		Ay[3][2] = (gamma*E) - ((gamma - 1.0)*0.5*((nU/(rho*rho)) + (2.0*v2*v2)));
		Ay[3][3] = gamma*v2;
	} else {
		double nv = v1*v1 + v2*v2, eps2 = mach*mach;
		Ax[1][0] = -(v1*v1) + ((gamma - 1)*nv*0.5);
		Ax[1][1] = (3.0 - gamma)*v1;
		Ax[1][2] = -(gamma - 1.0)*v2;
		Ax[1][3] = (gamma - 1.0)/eps2;
		Ax[2][0] = -v1*v2;
		Ax[2][1] = v2;
		Ax[2][2] = v1;
		Ax[3][0] = -v1*(gamma*E - ((gamma - 1.0)*eps2*nv));
		Ax[3][1] = gamma*E - (gamma - 1.0)*eps2*(0.5*nv + v1*v1);
		Ax[3][2] = -(gamma - 1.0)*eps2*v1*v2;
		Ax[3][3] = gamma*v1;
		Ay[1][0] = Ax[2][0];
		Ay[1][1] = v2;
		Ay[1][2] = v1;
		Ay[2][0] = -(v2*v2) + (((gamma - 1.0)*nv*0.5));
		Ay[2][1] = -(gamma - 1.0)*v1;
		Ay[2][2] = (3.0 - gamma)*v2;
		Ay[2][3] = Ax[1][3];
		Ay[3][0] = -v2*(gamma*E - (gamma - 1.0)*eps2*nv);
		Ay[3][1] = Ax[3][2];
		Ay[3][2] = gamma*E - (gamma - 1.0)*eps2*(0.5*nv + v2*v2);
		Ay[3][3] = gamma*v2;
	}
}

/* Quadratic form v^T A0 v as Delta_CAU.c:36-43 writes it (upper triangle,
 * off-diagonal terms doubled). */
static double a0norm2(const double A0[4][4], const double *v)
{
	return v[0]*(A0[0][0]*v[0] + 2.0*A0[0][1]*v[1] + 2.0*A0[0][2]*v[2] + 2.0*A0[0][3]*v[3]) +
	       v[1]*(A0[1][1]*v[1] + 2.0*A0[1][2]*v[2] + 2.0*A0[1][3]*v[3]) +
	       v[2]*(A0[2][2]*v[2] + 2.0*A0[2][3]*v[3]) +
	       v[3]*A0[3][3]*v[3];
}

/* Delta_CAU.c:4-84. */
static double delta_cau(double tol, const double *gx, const double *gy, const double Ax[4][4],
                        const double Ay[4][4], const double A0[4][4], const double *dUb, double y23,
                        double y31, double x32, double x13, double twoArea)
{
	double Axg[4], Ayg[4], kx[4], ky[4], L[4], nk, nL, ng;
	int i;
	for (i = 0; i < 4; i++) {
		Axg[i] = jvec(Ax, KAX, gx, i);
		Ayg[i] = jvec(Ay, KAY, gy, i);
	}
	for (i = 0; i < 4; i++) {
		kx[i] = (y23*gx[i] + x32*gy[i])/twoArea;
		ky[i] = (y31*gx[i] + x13*gy[i])/twoArea;
	}
	nk = sqrt(a0norm2(A0, kx) + a0norm2(A0, ky));
	for (i = 0; i < 4; i++) L[i] = dUb[i] + Axg[i] + Ayg[i];
	nL = sqrt(a0norm2(A0, L));
	ng = sqrt(a0norm2(A0, gx) + a0norm2(A0, gy));
	return ng >= tol ? nL/nk : 0.0;
}

/* One element of Build_M_K_F_SUPG.c:39-1042: Ae (12x12) and Re. */
static void euler_element(const orc_euler *p, int e, const double *U, const double *dU, double *Ae,
                          double *Re)
{
	const double third = 1.0/3.0, sixth = 1.0/6.0;
	const int *v = p->vert + 3*e;
	double X[3], Y[3], yb[3], xb[3], Ue[12], dUe[12], Ub[4], dUb[4], gx[4], gy[4];
	double Ax[4][4], Ay[4][4], A0[4][4], P[4][4][4], C[3][4][4], ax[3][4][4], ay[3][4][4];
	double twoArea, Area, gamma = p->gamma, alpha = p->alpha, dt = p->dt;
	int a, b, i, j, r, c, k;

	for (a = 0; a < 3; a++) { X[a] = p->x[v[a]]; Y[a] = p->y[v[a]]; }
	yb[0] = Y[1] - Y[2]; yb[1] = Y[2] - Y[0]; yb[2] = Y[0] - Y[1];     /* y23 y31 y12 */
	xb[0] = X[2] - X[1]; xb[1] = X[0] - X[2]; xb[2] = X[1] - X[0];     /* x32 x13 x21 */
	twoArea = fabs(xb[2]*yb[1] - xb[1]*yb[2]);
	Area = 0.5*twoArea;
	for (a = 0; a < 3; a++)
		for (k = 0; k < 4; k++) { Ue[4*a + k] = U[4*v[a] + k]; dUe[4*a + k] = dU[4*v[a] + k]; }
	for (i = 0; i < 4; i++) {
		Ub[i] = (Ue[i] + Ue[i+4] + Ue[i+8])*third;
		dUb[i] = (dUe[i] + dUe[i+4] + dUe[i+8])*third;
	}
	for (i = 0; i < 4; i++) {
		gx[i] = (Ue[i]*yb[0] + Ue[i+4]*yb[1] + Ue[i+8]*yb[2])/twoArea;
		gy[i] = (Ue[i]*xb[0] + Ue[i+4]*xb[1] + Ue[i+8]*xb[2])/twoArea;
	}
	double v1 = Ub[1]/Ub[0], v2 = Ub[2]/Ub[0], E = Ub[3]/Ub[0];
	double nU23 = (Ub[1]*Ub[1]) + (Ub[2]*Ub[2]);
	jacobians(p->dimensionless, gamma, p->mach, Ub, Ax, Ay);

	/* A0^-1 in entropy variables (:131-159). */
	{
		double rho_i = Ub[3] - ((nU23*0.5)/Ub[0]);
		double V2 = Ub[1]/rho_i, V3 = Ub[2]/rho_i, V4 = (-Ub[0])/rho_i;
		double re = -1.0/(rho_i*V4), k1 = (V2*V2 + V3*V3)*0.5/V4;
		A0[0][0] = re*(k1*k1 + gamma);
		A0[0][1] = re*(k1*V2);
		A0[0][2] = re*(k1*V3);
		A0[0][3] = re*((k1 + 1.0)*V4);
		A0[1][1] = re*(V2*V2 - V4);
		A0[1][2] = re*(V2*V3);
		A0[1][3] = re*(V2*V4);
		A0[2][2] = re*(V3*V3 - V4);
		A0[2][3] = re*(V3*V4);
		A0[3][3] = re*V4*V4;
		A0[1][0] = A0[0][1]; A0[2][0] = A0[0][2]; A0[3][0] = A0[0][3];
		A0[2][1] = A0[1][2]; A0[3][1] = A0[1][3]; A0[3][2] = A0[2][3];
	}
	/* AxAx, AxAy, AyAx, AyAy (:163-237). */
	for (i = 0; i < 4; i++)
		for (j = 0; j < 4; j++) {
			P[0][i][j] = jprod(Ax, KAX, Ax, KAX, i, j);
			P[1][i][j] = jprod(Ax, KAX, Ay, KAY, i, j);
			P[2][i][j] = jprod(Ay, KAY, Ax, KAX, i, j);
			P[3][i][j] = jprod(Ay, KAY, Ay, KAY, i, j);
		}
	double delta = delta_cau(p->stab_tol, gx, gy, Ax, Ay, A0, dUb, yb[0], yb[1], xb[0], xb[1], twoArea);

	/* SUPG tau (:244-269). */
	double tau;
	{
		double bx = 2.0*(gx[0]*Ub[0] + gx[1]*Ub[1] + gx[2]*Ub[2] + gx[3]*Ub[3]);
		double by = 2.0*(gy[0]*Ub[0] + gy[1]*Ub[1] + gy[2]*Ub[2] + gy[3]*Ub[3]);
		double bxy = sqrt(bx*bx + by*by);
		if (bxy != 0.0) { bx = bx/bxy; by = by/bxy; }
		double h = sqrt(twoArea);
		double avb = fabs(v1*bx + v2*by);
		double cs = sqrt(gamma*(gamma - 1.0)*(E - 0.5*((v1*v1) + (v2*v2))));
		double CFL = ((cs + avb)*dt)/h;
		double psi = (2.0*alpha*CFL)*(1.0/(1.0 + 2.0*alpha*CFL));
		double tau_d = delta/((cs + avb)*(cs + avb));
		double tau_a = h/(2.0*(cs + avb));
		double tau_t = (2.0/(3.0*(1.0 + 2.0*alpha*CFL)))*tau_a;
		tau = tau_t + psi*(tau_a - tau_d);
		if (tau < 0.0) tau = 0.0;
	}
	/* C_a = (y_a Ax + x_a Ay)/6 (:277-332) and the SUPG convection factors
	 * y_a AxAx + x_a AyAx, y_a AxAy + x_a AyAy (:629-735). */
	for (a = 0; a < 3; a++)
		for (i = 0; i < 4; i++)
			for (j = 0; j < 4; j++) {
				int kx = KAX[i][j], ky = KAY[i][j];
				double cv;
				if (!kx && !ky) cv = 0.0;
				else if (kx == 1) cv = yb[a]*sixth;
				else if (ky == 1) cv = xb[a]*sixth;
				else if (!ky) cv = yb[a]*Ax[i][j]*sixth;
				else if (!kx) cv = xb[a]*Ay[i][j]*sixth;
				else cv = (yb[a]*Ax[i][j] + xb[a]*Ay[i][j])*sixth;
				C[a][i][j] = cv;
				ax[a][i][j] = yb[a]*P[0][i][j] + xb[a]*P[2][i][j];
				ay[a][i][j] = yb[a]*P[1][i][j] + xb[a]*P[3][i][j];
			}
	double Mg1 = Area*sixth, Mg2 = Area/12.0;
	double tau4area = tau/(4*Area), delta4area = delta/(4.0*Area);
	double Kcau[3][3];
	for (a = 0; a < 3; a++)
		for (b = a + 1; b < 3; b++)
			Kcau[a][b] = Kcau[b][a] = delta4area*(yb[a]*yb[b] + xb[a]*xb[b]);

	/* Blocks (a, b) of Me (:401-561), Ke (:563-1026), Ae, Re (:1033-1042). */
	double Me[12][12], Ke[12][12];
	for (a = 0; a < 3; a++) {
		int b1 = a == 0 ? 1 : 0, b2 = a == 2 ? 1 : 2;
		for (b = 0; b < 3; b++)
			for (r = 0; r < 4; r++)
				for (c = 0; c < 4; c++) {
					double mpg = C[a][r][c]*tau, me, ke;
					me = (r == c) ? (a == b ? Mg1 : Mg2) + mpg : mpg;
					if (a != b) {
						double kpg = tau4area*(yb[b]*ax[a][r][c] + xb[b]*ay[a][r][c]);
						ke = C[b][r][c] + kpg;
						if (r == c) ke = ke + Kcau[a][b];
					} else {
						double k1 = tau4area*(yb[b1]*ax[a][r][c] + xb[b1]*ay[a][r][c]);
						double k2 = tau4area*(yb[b2]*ax[a][r][c] + xb[b2]*ay[a][r][c]);
						ke = C[a][r][c] - (k1 + k2);
						if (r == c) ke = ke - (Kcau[a][b1] + Kcau[a][b2]);
					}
					Me[4*a + r][4*b + c] = me;
					Ke[4*a + r][4*b + c] = ke;
				}
	}
	for (i = 0; i < 12; i++) {
		double m = 0, q = 0;
		for (j = 0; j < 12; j++) {
			m += Me[i][j]*dUe[j];
			q += Ke[i][j]*Ue[j];
			Ae[12*i + j] = Me[i][j] + alpha*dt*Ke[i][j];
		}
		Re[i] = -m - q;
	}
}

/* eval_U_dU.c:3-94: nodal U, dU from u, du and the prescribed values. */
static void eval_u_du(const orc_euler *p, const double *u, const double *du, double *U, double *dU)
{
	int I, k;
	for (I = 0; I < p->nnodes; I++)
		for (k = 0; k < 4; k++) {
			int id = p->node_id[4*I + k];
			U[4*I + k] = id >= 0 ? u[id] : p->upresc[4*I + k];
			dU[4*I + k] = id >= 0 ? du[id] : 0.0;
		}
}

void orc_euler_build(const orc_euler *p, const double *u, const double *du, double *Ae, double *R)
{
	double *U = malloc(sizeof(double) * 4 * (size_t)p->nnodes);
	double *dU = malloc(sizeof(double) * 4 * (size_t)p->nnodes);
	double Re[12];
	int e, i, a, k;
	eval_u_du(p, u, du, U, dU);
	memset(R, 0, sizeof(double) * ((size_t)p->neq + 1));
	for (e = 0; e < p->nel; e++) {
		euler_element(p, e, U, dU, Ae + (size_t)144*e, Re);
		for (a = 0; a < 3; a++)
			for (k = 0; k < 4; k++) {
				int id = p->node_id[4*p->vert[3*e + a] + k];
				i = id >= 0 ? id : p->neq;
				R[i] += Re[4*a + k];
			}
		R[p->neq] = 0;
	}
	free(U);
	free(dU);
}

/* ---- predictor-multicorrector ------------------------------------------- */
typedef struct {
	const orc_euler *p;
	const int *lm;
	const double *Ae, *invBD;
} euler_ops;

static void euler_mv(const void *ctx, double *P, double *Q)
{
	const euler_ops *o = ctx;
	orc_ebemv_blk(4, o->p->neq, o->p->nel, o->lm, o->Ae, P, Q);
}

static void euler_prec(const void *ctx, double *p, double *z)
{
	const euler_ops *o = ctx;
	orc_blockdiag_apply(4, o->p->nnodes, o->p->neq, o->p->node_id, o->invBD, p, z);
}

int orc_euler_predictor(const orc_euler *p, int kmax, int lmax, double tol, int nsteps, int ncorr,
                        double *u, double *uhist, int *iters)
{
	size_t n1 = (size_t)p->neq + 1;
	double *a = calloc(n1, sizeof(double)), *R = calloc(n1, sizeof(double)), *Da = calloc(n1, sizeof(double));
	double *Ae = malloc(sizeof(double) * 144 * (size_t)p->nel);
	double *BD = malloc(sizeof(double) * 16 * (size_t)p->nnodes);
	double *invBD = malloc(sizeof(double) * 16 * (size_t)p->nnodes);
	int *lm = malloc(sizeof(int) * 12 * (size_t)p->nel);
	double c_pred = (1.0 - p->alpha)*p->dt, c_corr = p->alpha*p->dt;
	int step, i, I, total = 0;
	euler_ops o = { p, lm, Ae, invBD };
	orc_fill_lm_blk(4, p->nel, p->vert, p->node_id, p->neq, lm);
	for (step = 0; step < nsteps; step++) {
		for (I = 0; I < p->neq; I++) {                       /* Predictor_Old.c:57-62 */
			u[I] += c_pred*a[I];
			a[I] = 0.0;
		}
		for (i = 0; i < ncorr; i++) {                         /* :68-126 */
			int it;
			orc_euler_build(p, u, a, Ae, R);
			orc_blockdiag_setup(4, p->nnodes, p->nel, p->neq, p->vert, p->node_id, Ae, BD, invBD, R);
			it = orc_pgmres_cb(p->neq, euler_mv, euler_prec, &o, kmax, lmax, tol, R, Da);
			if (iters) iters[step*ncorr + i] = it;
			total += it;
			for (I = 0; I < p->neq; I++) a[I] += 1*Da[I];   /* daxpy(neq, 1, Da, a) */
			for (I = 0; I < p->neq; I++) u[I] += c_corr*Da[I];
		}
		if (uhist) memcpy(uhist + (size_t)step*n1, u, sizeof(double)*n1);
	}
	free(a); free(R); free(Da); free(Ae); free(BD); free(invBD); free(lm);
	return total;
}
