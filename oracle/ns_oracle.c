/*
 * Test infrastructure only -- CPU oracle for the steady incompressible
 * Navier-Stokes path (mod-comp-ufes/FEM_CODES, 04_SS_NavierStokes_Equations/
 * 2D/01_CommonFiles): the VMS/NSGS element build with bubble condensation
 * (Build_K_F_MS.c:8-1190, the branch it executes), the damped Newton loop
 * (Process.c:62-194) and its forcing terms (eta_newton.c:5-68).  A
 * restatement in this project's own code, organised by node pairs (a, b) and
 * velocity components (i, j); every floating-point expression keeps the
 * reference's operation order, so element matrices and residuals are
 * bit-identical (pinned by tests/golden/ns_*.npz).  Never linked into the
 * product.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* eval_U.c:3-36: nodal (u, v, p). */
static void ns_eval_u(const orc_ns *p, const double *u, double *U)
{
	int I, k;
	for (I = 0; I < p->nnodes; I++)
		for (k = 0; k < 3; k++) {
			int id = p->node_id[3*I + k];
			U[3*I + k] = id >= 0 ? u[id] : p->upresc[3*I + k];
		}
}

/* Stabilisation state update of Build_K_F_MS.c:212-265 / :505-575: the
 * artificial diffusion delta from the residual and gradient norms. */
static double delta_aux(double normgradU, double hRGN, double normres, double cont)
{
	const double coe01 = 1.0, coe02 = 1.0;
	if (normgradU > 1e-5)
		return (coe01*hRGN*normres/normgradU + coe02*hRGN*hRGN*sqrt(cont*cont))/2.0;
	return 0.0;
}

static double h_rgn(double ux, double uy, const double *yb, const double *xb, double Area, double unorm)
{
	double auxh = fabs(ux*yb[0] + uy*xb[0]) + fabs(ux*yb[1] + uy*xb[1]) + fabs(ux*yb[2] + uy*xb[2]);
	return fabs(auxh) >= 1e-6 ? 4*Area*unorm/auxh : 0.0;
}

/* One element: Ke (9x9 row-major, dof order u1 v1 p1 u2 v2 p2 u3 v3 p3) and
 * Res (9), with the element's stabilisation state updated. */
static void ns_element(const orc_ns *pr, int e, const double *U, int first, double *dold, double *nold,
                       double *Ke, double *Res)
{
	const double third = 1.0/3.0, sixth = 1.0/6.0, ninefortieth = 9.0/40.0, ninetwentieth = 9.0/20.0,
	             twelfth = 1.0/12.0, epsilon = 1e-7, coefnorm = 0.8, w = 0.5, rho = 1.;
	const int *v = pr->vert + 3*e;
	double X[3], Y[3], yb[3], xb[3], uxn[3], uyn[3], pn[3], fx[3], fy[3];
	int a, b, i, j;
	for (a = 0; a < 3; a++) {
		X[a] = pr->x[v[a]]; Y[a] = pr->y[v[a]];
		uxn[a] = U[3*v[a]]; uyn[a] = U[3*v[a] + 1]; pn[a] = U[3*v[a] + 2];
		fx[a] = pr->f[2*v[a]]; fy[a] = pr->f[2*v[a] + 1];
	}
	yb[0] = Y[1] - Y[2]; yb[1] = Y[2] - Y[0]; yb[2] = Y[0] - Y[1];     /* y23 y31 y12 */
	xb[0] = X[2] - X[1]; xb[1] = X[0] - X[2]; xb[2] = X[1] - X[0];     /* x32 x13 x21 */
	double twoArea = fabs(xb[2]*yb[1] - xb[1]*yb[2]), Area = 0.5*twoArea, invArea = 1.0/Area;
	double ux = third*(uxn[0] + uxn[1] + uxn[2]), uy = third*(uyn[0] + uyn[1] + uyn[2]);
	double duxdx = 0.5*invArea*(uxn[0]*yb[0] + uxn[1]*yb[1] + uxn[2]*yb[2]);
	double duxdy = 0.5*invArea*(uxn[0]*xb[0] + uxn[1]*xb[1] + uxn[2]*xb[2]);
	double duydx = 0.5*invArea*(uyn[0]*yb[0] + uyn[1]*yb[1] + uyn[2]*yb[2]);
	double duydy = 0.5*invArea*(uyn[0]*xb[0] + uyn[1]*xb[1] + uyn[2]*xb[2]);
	double duxduy = uxn[0]*yb[0] + uyn[0]*xb[0] + uxn[1]*yb[1] + uyn[1]*xb[1] + uxn[2]*yb[2] + uyn[2]*xb[2];
	double p = third*(pn[0] + pn[1] + pn[2]);
	double dpdx = 0.5*invArea*(pn[0]*yb[0] + pn[1]*yb[1] + pn[2]*yb[2]);
	double dpdy = 0.5*invArea*(pn[0]*xb[0] + pn[1]*xb[1] + pn[2]*xb[2]);
	double h = sqrt(twoArea), visc = 1./pr->re;
	double unorm = sqrt(ux*ux + uy*uy);
	double tau_l = 0.333*h*unorm;
	double fxB = third*(fx[0] + fx[1] + fx[2]), fyB = third*(fy[0] + fy[1] + fy[2]);
	double f1 = rho*third*Area*fxB, f2 = rho*third*Area*fyB;
	double f1B = rho*ninetwentieth*Area*fxB, f2B = rho*ninetwentieth*Area*fyB;

	/* micro-scale (bubble) velocity from the macro field (:212-315) */
	double ne1 = ux*duxdx + uy*duydx + dpdx - f1, ne2 = ux*duxdy + uy*duydy + dpdy - f2;
	double cont = duxdx + duydy;
	double normres = sqrt(ne1*ne1 + ne2*ne2);
	double normgradU = sqrt(duxdx*duxdx + duxdy*duxdy + duydx*duydx + duydy*duydy);
	double hR = h_rgn(ux, uy, yb, xb, Area, unorm);
	double da = delta_aux(normgradU, hR, normres, cont);
	double delta = (first || normres < coefnorm*(*nold)) ? w*da + (1-w)*(*dold) : *dold;
	double deltam = delta;
	double A = yb[0]*yb[0] + yb[1]*yb[1] + yb[2]*yb[2] + yb[0]*yb[1] + yb[0]*yb[2] + yb[1]*yb[2];
	double B = xb[0]*xb[0] + xb[1]*xb[1] + xb[2]*xb[2] + xb[0]*xb[1] + xb[0]*xb[2] + xb[1]*xb[2];
	double C = yb[0]*xb[0] + yb[1]*xb[1] + yb[2]*xb[2];
	double NBB = 0.0;
	double KBB11 = 81.0*((2*visc + deltam)*A + (visc + deltam)*B)/(40.0*Area) + NBB;
	double KBB12 = 81.0*visc*C/(80.0*Area);
	double KBB22 = 81.0*((2*visc + deltam)*B + (visc + deltam)*A)/(40.0*Area) + NBB;
	double D = KBB11*KBB22 - KBB12*KBB12;
	double I11 = KBB22/D, I12 = -KBB12/D, I22 = KBB11/D;
	double NBh[3], G0[3], G1[3];           /* NBh_a, GBh row 0 (y), GBh row 1 (x) */
	for (a = 0; a < 3; a++) {
		NBh[a] = rho*ninefortieth*(ux*yb[a] + uy*xb[a]);
		G0[a] = -ninefortieth*yb[a];
		G1[a] = -ninefortieth*xb[a];
	}
	{
		double r1 = f1B - (NBh[0]*uxn[0] + NBh[1]*uxn[1] + NBh[2]*uxn[2]) + (G0[0]*pn[0] + G0[1]*pn[1] + G0[2]*pn[2]);
		double r2 = f2B - (NBh[0]*uyn[0] + NBh[1]*uyn[1] + NBh[2]*uyn[2]) + (G1[0]*pn[0] + G1[1]*pn[1] + G1[2]*pn[2]);
		double uxB = I11*r1 + I12*r2, uyB = I12*r1 + I22*r2;
		ux = ux + uxB;
		uy = uy + uyB;
	}
	double Cc[3];
	for (a = 0; a < 3; a++) Cc[a] = 0.5*invArea*(ux*yb[a] + uy*xb[a]);

	/* Galerkin, LSIC and mean-zero pressure terms (:334-412) */
	double N1[3], GT[3][2], g[3][2];
	for (a = 0; a < 3; a++) {
		N1[a] = rho*third*Area*Cc[a];
		g[a][0] = yb[a]; g[a][1] = xb[a];
		GT[a][0] = sixth*yb[a]; GT[a][1] = sixth*xb[a];
	}
	const double kv = visc*0.25*invArea, ks = tau_l*rho*0.25*invArea;
	const double C11 = epsilon*Area*sixth, C12 = epsilon*Area*twelfth;

	/* residual pieces (:416-456), with the total velocity */
	double Nv0 = rho*third*Area*(duxdx*ux + duxdy*uy), Nv1 = rho*third*Area*(duydx*ux + duydy*uy);
	double GTv = third*Area*(duxdx + duydy);

	/* second pass of the stabilisation state (:458-575) */
	ne1 = ux*duxdx + uy*duydx + dpdx - f1;
	ne2 = ux*duxdy + uy*duydy + dpdy - f2;
	normres = sqrt(ne1*ne1 + ne2*ne2);
	normgradU = sqrt(duxdx*duxdx + duydy*duydy + duxdy*duxdy + duydx*duydx);
	unorm = sqrt(ux*ux + uy*uy);
	hR = h_rgn(ux, uy, yb, xb, Area, unorm);
	da = delta_aux(normgradU, hR, normres, cont);
	if (first || normres < coefnorm*(*nold)) {
		delta = w*da + (1-w)*(*dold);
		*dold = delta;
	} else {
		delta = *dold;
	}
	*nold = normres;
	deltam = delta;
	delta = 0.0;
	KBB11 = 81.0*((2*visc + deltam)*A + (visc + deltam)*B)/(40.0*Area) + NBB;
	KBB12 = 81.0*visc*C/(80.0*Area);
	KBB22 = 81.0*((2*visc + deltam)*B + (visc + deltam)*A)/(40.0*Area) + NBB;
	D = KBB11*KBB22 - KBB12*KBB12;
	I11 = KBB22/D; I12 = -KBB12/D; I22 = KBB11/D;
	const double Inv[2][2] = {{I11, I12}, {I12, I22}};
	double delta4area = delta/(4.0*Area), NhB[3];
	for (a = 0; a < 3; a++) {
		NBh[a] = rho*ninefortieth*(ux*yb[a] + uy*xb[a]);
		NhB[a] = -NBh[a];
	}

	/* micro-scale coupling matrices (:610-790):
	 *   Ndelta[(a,i)][(b,j)] = NhB_a Inv_ij NBh_b
	 *   Gdelta[(a,i)][b]     = NhB_a Inv_i0 G0_b + NhB_a Inv_i1 G1_b
	 *   Gphi[a][b]           = G0_b (G0_a I11 + G1_a I12) + G1_b (G0_a I12 + G1_a I22) */
	double Nd[6][6], Gd[6][3], Gphi[3][3];
	for (a = 0; a < 3; a++)
		for (i = 0; i < 2; i++) {
			for (b = 0; b < 3; b++) {
				for (j = 0; j < 2; j++) Nd[2*a + i][2*b + j] = NhB[a]*Inv[i][j]*NBh[b];
				Gd[2*a + i][b] = NhB[a]*Inv[i][0]*G0[b] + NhB[a]*Inv[i][1]*G1[b];
			}
		}
	for (a = 0; a < 3; a++)
		for (b = 0; b < 3; b++)
			Gphi[a][b] = G0[b]*(G0[a]*I11 + G1[a]*I12) + G1[b]*(G0[a]*I12 + G1[a]*I22);

	/* element RHS (:795-818) */
	double Fe[9];
	for (a = 0; a < 3; a++) {
		double fd0 = -(NhB[a]*I11*f1B + NhB[a]*I12*f2B), fd1 = -(NhB[a]*I12*f1B + NhB[a]*I22*f2B);
		Fe[3*a] = f1 + fd0;
		Fe[3*a + 1] = f2 + fd1;
		Fe[3*a + 2] = -((G0[a]*I11 + G1[a]*I12)*f1B + (G0[a]*I12 + G1[a]*I22)*f2B);
	}

	/* residual of the Newton step (:820-859) */
	double uv[6] = {uxn[0], uyn[0], uxn[1], uyn[1], uxn[2], uyn[2]};
	double shear = duxdy + duydx;
	for (a = 0; a < 3; a++) {
		double Kv[2], Kdd[2], Nd_v[2], Gd_v[2];
		Kv[0] = 0.5*visc*(2*yb[a]*duxdx + xb[a]*shear);
		Kv[1] = 0.5*visc*(2*xb[a]*duydy + yb[a]*shear);
		Kdd[0] = 0.5*delta*(yb[a]*duxdx + xb[a]*duxdy);
		Kdd[1] = 0.5*delta*(yb[a]*duydx + xb[a]*duydy);
		for (i = 0; i < 2; i++) {
			int r = 2*a + i;
			Nd_v[i] = Nd[r][0]*uv[0] + Nd[r][1]*uv[1] + Nd[r][2]*uv[2] + Nd[r][3]*uv[3] + Nd[r][4]*uv[4] +
			          Nd[r][5]*uv[5];
			Gd_v[i] = Gd[r][0]*pn[0] + Gd[r][1]*pn[1] + Gd[r][2]*pn[2];
			double Ksv = ks*g[a][i]*duxduy, Gv = 0.5*p*g[a][i];
			Res[3*a + i] = Fe[3*a + i] - ((i == 0 ? Nv0 : Nv1) - Nd_v[i] + Kv[i] + Ksv + Kdd[i] - (Gv - Gd_v[i]));
		}
		/* pressure row: Cv and the GhB coupling terms */
		int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
		double Cv = C11*pn[a] + C12*(pn[o1] + pn[o2]);
		double Nphiv = 0.0, Gphiv;
		for (b = 0; b < 3; b++)
			for (j = 0; j < 2; j++) {
				double t = -Gd[2*b + j][a]*uv[2*b + j];
				Nphiv = (b == 0 && j == 0) ? t : Nphiv + t;
			}
		Gphiv = Gphi[a][0]*pn[0] + Gphi[a][1]*pn[1] + Gphi[a][2]*pn[2];
		Res[3*a + 2] = Fe[3*a + 2] - (GTv + Cv - Nphiv + Gphiv);
	}

	/* tangent matrix (:865-960, the branch taken) */
	for (a = 0; a < 3; a++)
		for (b = 0; b < 3; b++) {
			int lo = a < b ? a : b, hi = a < b ? b : a;
			double kdd = delta4area*(yb[lo]*yb[hi] + xb[lo]*xb[hi]);
			for (i = 0; i < 2; i++) {
				double *row = Ke + 9*(3*a + i) + 3*b;
				for (j = 0; j < 2; j++) {
					double K = (i == 0 && j == 0) ? kv*(2*yb[a]*yb[b] + xb[a]*xb[b])
					         : (i == 1 && j == 1) ? kv*(yb[a]*yb[b] + 2*xb[a]*xb[b])
					         : (i == 0) ? kv*(xb[a]*yb[b]) : kv*(yb[a]*xb[b]);
					double Ks = ks*g[b][j]*g[a][i];
					if (i == j) {
						/* the node pair's coupling term is read from the (lower node,
						 * higher node) entry, and added for (a, b) = (3, 2), i = 0 */
						double nd = Nd[2*lo + i][2*hi + i];
						double t = (a == 2 && b == 1 && i == 0) ? N1[b] + nd : N1[b] - nd;
						row[j] = t + K + Ks + kdd;
					} else {
						row[j] = K + Ks;
					}
				}
				row[2] = -(GT[a][i] - Gd[2*a + i][b]);
			}
			double *prow = Ke + 9*(3*a + 2) + 3*b;
			for (j = 0; j < 2; j++) prow[j] = GT[b][j] - (-Gd[2*b + j][a]);
			prow[2] = Gphi[lo][hi] + (a == b ? C11 : C12);
		}
}

void orc_ns_build(const orc_ns *p, const double *u, int first, double *dold, double *nold, double *Ae, double *F)
{
	double *U = malloc(sizeof(double) * 3 * (size_t)p->nnodes);
	double Res[9];
	int e, a, k;
	ns_eval_u(p, u, U);
	memset(F, 0, sizeof(double) * ((size_t)p->neq + 1));
	for (e = 0; e < p->nel; e++) {
		ns_element(p, e, U, first, dold + e, nold + e, Ae + (size_t)81*e, Res);
		for (a = 0; a < 3; a++)
			for (k = 0; k < 3; k++) {
				int id = p->node_id[3*p->vert[3*e + a] + k];
				F[id >= 0 ? id : p->neq] += Res[3*a + k];
			}
		F[p->neq] = 0;
	}
	free(U);
}

/* eta_newton.c:5-68: forcing term of the inexact Newton step. */
double orc_eta_newton(int ecase, double nF, double nFold, double etaold, int pricek, int it, double talnl,
                      double eta0)
{
	double delta1 = nF, delta2 = nFold, delta = delta1/delta2, eta = 0, etaa, old, etaaux;
	if (ecase == 1) {
		eta = (eta0 < delta) ? eta0 : delta*delta;
	} else if (ecase == 2 || ecase == 3) {
		double alpha = ecase == 2 ? 2. : (1. + sqrt(5))*0.5, gamma = ecase == 2 ? 0.9 : 1.0;
		double beta = ecase == 2 ? 0.1 : 0.;
		etaa = gamma*pow(delta, alpha);
		old = gamma*pow(etaold, alpha);
		if (old < beta) {
			eta = (eta0 < etaa) ? eta0 : etaa;
		} else {
			etaaux = (etaa > old) ? etaa : old;
			eta = (eta0 < etaaux) ? eta0 : etaaux;
		}
	} else if (ecase == 4) {
		double ak = log10(delta1) - log10(delta2), bk = log10(pricek);
		double thetak = bk/sqrt(ak*ak + bk*bk);
		double gamma = pow(1./(it + 1), 1.1)*cos(thetak)*cos(thetak);
		etaa = gamma*delta;
		eta = (eta0 < etaa) ? eta0 : etaa;
	}
	old = 0.5*talnl/delta1;
	etaaux = (eta > old) ? eta : old;
	eta = (eta0 < etaaux) ? eta0 : etaaux;
	if (ecase == 0) eta = eta0;
	return eta;
}

/* ---- damped Newton (Process.c:62-194) ----------------------------------- */
typedef struct {
	const orc_ns *p;
	const int *lm;
	const double *Ae, *invBD;
} ns_ops;

static void ns_mv(const void *ctx, double *P, double *Q)
{
	const ns_ops *o = ctx;
	orc_ebemv_blk(3, o->p->neq, o->p->nel, o->lm, o->Ae, P, Q);
}

static void ns_prec(const void *ctx, double *pv, double *z)
{
	const ns_ops *o = ctx;
	orc_blockdiag_apply(3, o->p->nnodes, o->p->neq, o->p->node_id, o->invBD, pv, z);
}

int orc_ns_newton(const orc_ns *p, int kmax, int lmax, double eta0, int ecase, double tolnl, int maxit,
                  double *uhist, double *normF, double *wout, int *gmres)
{
	size_t n1 = (size_t)p->neq + 1;
	int neq = p->neq, it, iter = 0, iterold, pricek, fd, cont, nit = 0, I, first = 1;
	double *u = calloc(n1, sizeof(double)), *F = calloc(n1, sizeof(double)), *s = calloc(n1, sizeof(double));
	double *Fold = calloc(n1, sizeof(double)), *Ae = malloc(sizeof(double) * 81 * (size_t)p->nel);
	double *dold = calloc((size_t)p->nel, sizeof(double)), *nold = calloc((size_t)p->nel, sizeof(double));
	double *BD = malloc(sizeof(double) * 9 * (size_t)p->nnodes), *invBD = malloc(sizeof(double) * 9 * (size_t)p->nnodes);
	int *lm = malloc(sizeof(int) * 9 * (size_t)p->nel);
	double w_min = 0.05, w_max = 1.00, c1 = 1.001, c2 = 1.1, c3 = 1.001, c4 = 0.9, c5 = 0.5, w = w_max, w_old;
	double norm_F, norm_Fold, epsilon, tol = eta0;
	ns_ops o = { p, lm, Ae, invBD };
	orc_fill_lm_blk(3, p->nel, p->vert, p->node_id, neq, lm);
	orc_ns_build(p, u, first, dold, nold, Ae, F);
	first = 0;
	it = 1;
	orc_blockdiag_setup(3, p->nnodes, p->nel, neq, p->vert, p->node_id, Ae, BD, invBD, F);
	norm_F = sqrt(orc_ddot(neq, F, F));
	epsilon = tolnl*norm_F;
	pricek = 1;
	memcpy(Fold, F, sizeof(double)*(size_t)neq);
	while (norm_F > epsilon && it < 2000 && nit < maxit) {
		it++;
		iterold = iter;
		norm_Fold = sqrt(orc_ddot(neq, Fold, Fold));
		iter += orc_pgmres_cb(neq, ns_mv, ns_prec, &o, kmax, lmax, tol, F, s);
		pricek = iter - iterold + 1;
		fd = 1; cont = 1;
		do {
			w_old = w;
			for (I = 0; I < neq; I++) u[I] += w*s[I];                 /* daxpy(neq, w, s, u) */
			orc_ns_build(p, u, first, dold, nold, Ae, F);
			orc_blockdiag_setup(3, p->nnodes, p->nel, neq, p->vert, p->node_id, Ae, BD, invBD, F);
			{
				double etaold = tol;
				tol = orc_eta_newton(ecase, sqrt(orc_ddot(neq, F, F)), sqrt(orc_ddot(neq, Fold, Fold)), etaold,
				                     pricek, it, epsilon, eta0);
			}
			norm_F = sqrt(orc_ddot(neq, F, F));
			if (norm_F < norm_Fold || w < c1*w_min) {
				if (norm_F < norm_Fold && fd == 1) {
					w_max = (1.0 < c3*w_max) ? 1.0 : c3*w_max;
					w = (w_max < c2*w) ? w_max : c2*w;
				}
				cont = 0;
			} else {
				w = (w_min > c5*w) ? w_min : c5*w;
				if (fd == 1) {
					w_max = (w_min > c4*w_max) ? w_min : c4*w_max;
					fd = 0;
				}
				for (I = 0; I < neq; I++) u[I] += -1.*w_old*s[I];    /* daxpy(neq, -w_old, s, u) */
			}
		} while (cont == 1);
		memcpy(Fold, F, sizeof(double)*(size_t)neq);
		if (uhist) memcpy(uhist + (size_t)nit*n1, u, sizeof(double)*n1);
		if (normF) normF[nit] = norm_F;
		if (wout) wout[nit] = w_old;
		if (gmres) gmres[nit] = pricek - 1;
		nit++;
	}
	free(u); free(F); free(s); free(Fold); free(Ae); free(dold); free(nold); free(BD); free(invBD); free(lm);
	return nit;
}
