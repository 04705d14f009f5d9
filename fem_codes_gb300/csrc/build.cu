// Element build of the steady scalar transport equation -- SUPG with
// CAU/YZBeta shock capturing on linear triangles (Build_K_F_SUPG.c:35-157,
// CAU_ShockCapture.c, YZBeta_ShockCapture.c, h_shock_*.c) -- and the
// deterministic assembly of its element matrices into EDE/CSR storage and of
// the load vector (F_assembly.c, ede_assembly.c, csr_assembly.c).
//
// One thread per element computes ke (3x3) and Fe (3) in FP64 and stores them
// element-major.  Assembly then gathers, for every CSR row / edge, the
// contributions of its incident elements in ascending element order: the same
// sequence of additions the reference's serial element loop performs, so the
// assembled values and F are reproducible run to run (no atomics).
//
// This translation unit is compiled with --fmad=false: every product and sum
// is rounded separately, as in the reference compiled without contraction.
#include "fg_common.cuh"

struct BuildArgs {
	const double *x, *y, *u, *upresc, *beta, *fsrc;
	const int *vert, *node_id;
	double k, gamma, cbx, cby;
	int nel, shock, hshock, beta_const, fsrc_zero;
	double *ke, *fe;
	// transient builds only
	const double *du;             // the time derivative a (neq+1)
	double adt;                   // Alpha * DeltaT
	double *re;                   // per element and local row: load term, then three products
	double *dold;                 // DD: the previous build's shock parameter per element
	// Build_M_F_DD (Predictor_New): the bubble unknowns and the condensation
	const double *uB, *aB;        // per element
	double *bub;                  // per element: invN2, R2, M2[3] (calculate_DaB's inputs)
};

// Shock length scale: h_shock_2sqrtArea.c:3-8, h_shock_sqrtArea.c:3-61 (every
// branch yields 2*sqrt|A|), h_shock_Option1.c:3-19, h_shock_Option2.c:3-19.
__device__ __forceinline__ double h_shock(int opt, double bx, double by, double u1, double u2,
                                          double u3, double y23, double y31, double y12,
                                          double x32, double x13, double x21, double Area)
{
	if (opt == FEMGPU_H_SQRTAREA) return 2 * sqrt(fabs(Area));
	if (opt == FEMGPU_H_OPTION1) {
		double P1 = fabs(u1*y23*y23 + u2*y31*y23 + u3*y12*y23 + u1*x32*x32 + u2*x13*x32 + u3*x21*x32);
		double P2 = fabs(u1*y23*y31 + u2*y31*y31 + u3*y12*y31 + u1*x32*x13 + u2*x13*x13 + u3*x21*x13);
		double P3 = fabs(u1*y23*y12 + u2*y31*y12 + u3*y12*y12 + u1*x32*x21 + u2*x13*x21 + u3*x21*x21);
		double a1 = y23*u1 + y31*u2 + y12*u3, a2 = x32*u1 + x13*u2 + x21*u3;
		double ng = sqrt(a1*a1 + a2*a2);
		return (P1 + P2 + P3 >= 1e-12) ? 4*Area*ng/(P1 + P2 + P3) : 0.0;
	}
	if (opt == FEMGPU_H_OPTION2) {
		double P1 = fabs(bx*y23 + by*x32), P2 = fabs(bx*y31 + by*x13), P3 = fabs(bx*y12 + by*x21);
		double nb = sqrt(bx*bx + by*by);
		return (P1 + P2 + P3 >= 1e-12) ? 4*Area*nb/(P1 + P2 + P3) : 0.0;
	}
	return sqrt(fabs(2*Area));
}

// CAU_ShockCapture.c:3-30 (the division by |grad u|^2 is only evaluated when
// |grad u| > 0; the reference computes it first and discards a NaN) and
// YZBeta_ShockCapture.c:3-27.
__device__ __forceinline__ double shock_capture(int kind, double kx, double ky, double bx, double by,
                                                double g, double ue1, double ue2, double ue3,
                                                double ueb, double feb, double y23, double y31,
                                                double y12, double x32, double x13, double x21,
                                                double invArea, double h)
{
	double BetaGradu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
	double Ru = BetaGradu + g*ueb - feb;
	double G0 = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
	double G1 = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
	double nG = sqrt(G0*G0 + G1*G1);
	if (kind == FEMGPU_SHOCK_YZBETA) {
		double nRu = fabs(Ru), nu = fabs(ueb);
		return (nu >= 1e-12 && nG >= 1e-12) ? 0.25*h*nRu/nG + 0.125*h*h*nRu/nu : 0.0;
	}
	if (!(nG > 0)) return 0.0;
	const double third = 1./3.;
	double bxp = BetaGradu*G0/(nG*nG), byp = BetaGradu*G1/(nG*nG);
	double kp = bxp*bxp*kx + byp*byp*ky;
	double nbp = sqrt(bxp*bxp + byp*byp);
	double Pee = 0.5*h*nbp*nbp*nbp/kp;
	if (third*Pee < 0.7) return 0.5*h*third*Pee*fabs(Ru)/nG;
	return 0.5*h*0.7*fabs(Ru)/nG;
}

__global__ void __launch_bounds__(128) k_build_supg(BuildArgs a)
{
	const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
	const double kx = a.k, ky = a.k, gamma = a.gamma;
	for (int E = blockIdx.x * blockDim.x + threadIdx.x; E < a.nel; E += gridDim.x * blockDim.x) {
		int J1 = __ldg(&a.vert[3*E]), J2 = __ldg(&a.vert[3*E+1]), J3 = __ldg(&a.vert[3*E+2]);
		double X0 = __ldg(&a.x[J1]), X1 = __ldg(&a.x[J2]), X2 = __ldg(&a.x[J3]);
		double Y0 = __ldg(&a.y[J1]), Y1 = __ldg(&a.y[J2]), Y2 = __ldg(&a.y[J3]);
		double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
		double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
		double TwoA = x21*y31 - x13*y12, Area = 0.5*TwoA, invArea = 1.0/Area;
		double h = sqrt(fabs(TwoA));
		double bx, by;
		if (a.beta_const) { bx = a.cbx; by = a.cby; }
		else { bx = __ldg(&a.beta[2*E]); by = __ldg(&a.beta[2*E+1]); }
		double norm = sqrt(bx*bx + by*by), tau = (norm > 0) ? 0.5*h/norm : 0.0;
		double fe1 = 0.0, fe2 = 0.0, fe3 = 0.0;
		if (!a.fsrc_zero) { fe1 = __ldg(&a.fsrc[3*E]); fe2 = __ldg(&a.fsrc[3*E+1]); fe3 = __ldg(&a.fsrc[3*E+2]); }
		double feb = third*(fe1+fe2+fe3);
		// eval_U.c:12-22
		int i1 = __ldg(&a.node_id[J1]), i2 = __ldg(&a.node_id[J2]), i3 = __ldg(&a.node_id[J3]);
		double ue1 = (i1 >= 0) ? a.u[i1] : __ldg(&a.upresc[J1]);
		double ue2 = (i2 >= 0) ? a.u[i2] : __ldg(&a.upresc[J2]);
		double ue3 = (i3 >= 0) ? a.u[i3] : __ldg(&a.upresc[J3]);
		double ueb = third * (ue1 + ue2 + ue3);

		double D12 = 0.25*invArea*((kx * y23 * y31) + (ky * x32 * x13));
		double D13 = 0.25*invArea*((kx * y23 * y12) + (ky * x32 * x21));
		double D23 = 0.25*invArea*((kx * y31 * y12) + (ky * x13 * x21));
		double C11 = sixth*(bx*y23 + by*x32);
		double C12 = sixth*(bx*y31 + by*x13);
		double C13 = sixth*(bx*y12 + by*x21);
		double R11 = sixth*(gamma*Area);
		double R12 = twelfth*(gamma * Area);
		double Cpg12 = 0.25*invArea*tau * (y23*(bx*bx*y31 + bx*by*x13) + x32*(bx*by*y31 + by*by*x13));
		double Cpg13 = 0.25*invArea*tau * (y23*(bx*bx*y12 + bx*by*x21) + x32*(bx*by*y12 + by*by*x21));
		double Cpg23 = 0.25*invArea*tau * (y31*(bx*bx*y12 + bx*by*x21) + x13*(bx*by*y12 + by*by*x21));
		double Rpg11 = sixth*tau*gamma * (bx*y23 + by*x32);
		double Rpg21 = sixth*tau*gamma * (bx*y31 + by*x13);
		double Rpg31 = sixth*tau*gamma * (bx*y12 + by*x21);

		double hs = h_shock(a.hshock, bx, by, ue1, ue2, ue3, y23, y31, y12, x32, x13, x21, Area);
		double Eu = shock_capture(a.shock, kx, ky, bx, by, gamma, ue1, ue2, ue3, ueb, feb,
		                          y23, y31, y12, x32, x13, x21, invArea, hs);
		double Csc12 = Eu*0.25*invArea*(y23*y31 + x32*x13);
		double Csc13 = Eu*0.25*invArea*(y23*y12 + x32*x21);
		double Csc23 = Eu*0.25*invArea*(y31*y12 + x13*x21);

		double *ke = a.ke + 9LL*E;
		ke[0] = -(D12 + D13) + C11 - (Cpg12 + Cpg13) + R11 + Rpg11 - (Csc12 + Csc13);
		ke[1] = D12 + C12 + Cpg12 + R12 + Rpg11 + Csc12;
		ke[2] = D13 + C13 + Cpg13 + R12 + Rpg11 + Csc13;
		ke[3] = D12 + C11 + Cpg12 + R12 + Rpg21 + Csc12;
		ke[4] = -(D12 + D23) + C12 - (Cpg12 + Cpg23) + R11 + Rpg21 - (Csc12 + Csc23);
		ke[5] = D23 + C13 + Cpg23 + R12 + Rpg21 + Csc23;
		ke[6] = D13 + C11 + Cpg13 + R12 + Rpg31 + Csc13;
		ke[7] = D23 + C12 + Cpg23 + R12 + Rpg31 + Csc23;
		ke[8] = -(D13 + D23) + C13 - (Cpg13 + Cpg23) + R11 + Rpg31 - (Csc13 + Csc23);

		double *fe = a.fe + 3LL*E;
		fe[0] = Area*twelfth*(2*fe1 +  fe2  +  fe3 ) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32);
		fe[1] = Area*twelfth*(  fe1 + 2*fe2 +  fe3 ) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13);
		fe[2] = Area*twelfth*(  fe1 +  fe2  + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21);
	}
}

extern "C" int fg_build_elements(femgpu_transport *t)
{
	BuildArgs a;
	a.x = t->x; a.y = t->y; a.u = t->u; a.upresc = t->upresc; a.beta = t->beta; a.fsrc = t->fsrc;
	a.vert = t->vert; a.node_id = t->node_id;
	a.k = t->k; a.gamma = t->gamma; a.cbx = t->cbx; a.cby = t->cby;
	a.nel = t->nel; a.shock = t->o.shock; a.hshock = t->o.hshock;
	a.beta_const = t->beta_const; a.fsrc_zero = t->fsrc_zero;
	a.ke = (t->o.scheme == FEMGPU_EBE) ? t->A : t->ke;
	a.fe = t->fe;
	k_build_supg<<<fg_grid(t->nel, 128, 32), 128, 0, t->stream>>>(a);
	return (int)cudaGetLastError();
}

// ------------------------------------------------------ transient builds ---
// Shock capturing of the transient builds (02_Transport_Equation/2D/
// 01_CommonFiles/CAU_ShockCapture.c:3-30, YZBeta_ShockCapture.c:3-24,
// CAU_DD_ShockCapture.c:3-19): the residual carries the time derivative,
// Ru = dueb + beta.grad u + gamma ueb - feb.  As in the steady form, the CAU
// division by |grad u|^2 is only evaluated when |grad u| > 0 (the reference
// discards its NaN otherwise).
__device__ __forceinline__ double shock_capture_tr(int kind, double kx, double ky, double bx, double by,
                                                   double g, double ue1, double ue2, double ue3,
                                                   double ueb, double dueb, double feb, double y23, double y31,
                                                   double y12, double x32, double x13, double x21,
                                                   double invArea, double h)
{
	double BetaGradu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
	double Ru = dueb + BetaGradu + g*ueb - feb;
	double G0 = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
	double G1 = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
	double nG = sqrt(G0*G0 + G1*G1);
	if (kind == FEMGPU_SHOCK_YZBETA) {
		double nRu = fabs(Ru), nu = fabs(ueb);
		return (nu >= 1e-12 && nG >= 1e-12) ? 0.25*h*nRu/nG + 0.125*h*h*nRu/nu : 0.0;
	}
	if (kind == FEMGPU_SHOCK_CAUDD) return (nG > 1e-10) ? 0.5*h*fabs(Ru)/nG : 0.0;
	if (!(nG > 0)) return 0.0;
	const double third = 1./3.;
	double bxp = BetaGradu*G0/(nG*nG), byp = BetaGradu*G1/(nG*nG);
	double kp = bxp*bxp*kx + byp*byp*ky;
	double nbp = sqrt(bxp*bxp + byp*byp);
	double Pee = 0.5*h*nbp*nbp*nbp/kp;
	if (third*Pee < 0.7) return 0.5*h*third*Pee*fabs(Ru)/nG;
	return 0.5*h*0.7*fabs(Ru)/nG;
}

// Build_M_K_R_SUPG.c:36-180 (DD == false) and Build_M_K_R_DD.c:39-188
// (DD == true), one thread per element: Ae = Me + Alpha*DeltaT*Ke to the
// element buffer and, for the residual gather, per local row i the load term
// and the three products me[i][j]*due[j] + ke[i][j]*ue[j] the reference
// subtracts from R[lm[E][i]] in that order.  U and dU follow eval_U_dU.c
// (prescribed nodes: upresc and 0).  The DD form keeps the shock parameter
// of the previous build per element (cb = w cbtil + (1-w) cbtil_old, w = 1/2).
template <bool DD>
__global__ void __launch_bounds__(128) k_build_transient(BuildArgs a)
{
	const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
	const double seventh = 1.0/7.0, three_twentieth = 3./20.0, nine_twentieth = 9./20.0,
	             nine_forty_cents = 9./40.0, w = 0.5;
	const double kx = a.k, ky = a.k, gamma = a.gamma;
	for (int E = blockIdx.x * blockDim.x + threadIdx.x; E < a.nel; E += gridDim.x * blockDim.x) {
		int J1 = __ldg(&a.vert[3*E]), J2 = __ldg(&a.vert[3*E+1]), J3 = __ldg(&a.vert[3*E+2]);
		double X0 = __ldg(&a.x[J1]), X1 = __ldg(&a.x[J2]), X2 = __ldg(&a.x[J3]);
		double Y0 = __ldg(&a.y[J1]), Y1 = __ldg(&a.y[J2]), Y2 = __ldg(&a.y[J3]);
		double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
		double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
		double TwoA = x21*y31 - x13*y12, Area = 0.5*TwoA, invArea = 1.0/Area;
		double bx, by;
		if (a.beta_const) { bx = a.cbx; by = a.cby; }
		else { bx = __ldg(&a.beta[2*E]); by = __ldg(&a.beta[2*E+1]); }
		double fe1 = 0.0, fe2 = 0.0, fe3 = 0.0;
		if (!a.fsrc_zero) { fe1 = __ldg(&a.fsrc[3*E]); fe2 = __ldg(&a.fsrc[3*E+1]); fe3 = __ldg(&a.fsrc[3*E+2]); }
		double feb = third*(fe1+fe2+fe3);
		int i1 = __ldg(&a.node_id[J1]), i2 = __ldg(&a.node_id[J2]), i3 = __ldg(&a.node_id[J3]);
		double ue[3], due[3];
		ue[0] = (i1 >= 0) ? a.u[i1] : __ldg(&a.upresc[J1]);
		ue[1] = (i2 >= 0) ? a.u[i2] : __ldg(&a.upresc[J2]);
		ue[2] = (i3 >= 0) ? a.u[i3] : __ldg(&a.upresc[J3]);
		due[0] = (i1 >= 0) ? a.du[i1] : 0.0;
		due[1] = (i2 >= 0) ? a.du[i2] : 0.0;
		due[2] = (i3 >= 0) ? a.du[i3] : 0.0;
		double ueb = third * (ue[0] + ue[1] + ue[2]);
		double dueb = third * (due[0] + due[1] + due[2]);
		double D12 = 0.25*invArea*((kx * y23 * y31) + (ky * x32 * x13));
		double D13 = 0.25*invArea*((kx * y23 * y12) + (ky * x32 * x21));
		double D23 = 0.25*invArea*((kx * y31 * y12) + (ky * x13 * x21));
		double me[3][3], ke[3][3], f[3];
		if (!DD) {
			double h = sqrt(fabs(TwoA));
			double norm = sqrt(bx*bx + by*by), tau = (norm > 0) ? 0.5*h/norm : 0.0;
			double C11 = sixth*(bx*y23 + by*x32);
			double C12 = sixth*(bx*y31 + by*x13);
			double C13 = sixth*(bx*y12 + by*x21);
			double R11 = sixth*(gamma*Area);
			double R12 = twelfth*(gamma * Area);
			double Cpg12 = 0.25*invArea*tau * (y23*(bx*bx*y31 + bx*by*x13) + x32*(bx*by*y31 + by*by*x13));
			double Cpg13 = 0.25*invArea*tau * (y23*(bx*bx*y12 + bx*by*x21) + x32*(bx*by*y12 + by*by*x21));
			double Cpg23 = 0.25*invArea*tau * (y31*(bx*bx*y12 + bx*by*x21) + x13*(bx*by*y12 + by*by*x21));
			double Rpg11 = sixth*tau*gamma * (bx*y23 + by*x32);
			double Rpg21 = sixth*tau*gamma * (bx*y31 + by*x13);
			double Rpg31 = sixth*tau*gamma * (bx*y12 + by*x21);
			double hs = h_shock(a.hshock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
			double Eu = shock_capture_tr(a.shock, kx, ky, bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb,
			                             y23, y31, y12, x32, x13, x21, invArea, hs);
			double Csc12 = Eu*0.25*invArea*(y23*y31 + x32*x13);
			double Csc13 = Eu*0.25*invArea*(y23*y12 + x32*x21);
			double Csc23 = Eu*0.25*invArea*(y31*y12 + x13*x21);
			me[0][0] = sixth*Area  + tau*C11;
			me[0][1] = twelfth*Area + tau*C11;
			me[0][2] = twelfth*Area + tau*C11;
			me[1][0] = twelfth*Area + tau*C12;
			me[1][1] = sixth*Area  + tau*C12;
			me[1][2] = twelfth*Area + tau*C12;
			me[2][0] = twelfth*Area + tau*C13;
			me[2][1] = twelfth*Area + tau*C13;
			me[2][2] = sixth*Area  + tau*C13;
			ke[0][0] = -(D12 + D13) + C11 - (Cpg12 + Cpg13) + R11 + Rpg11 - (Csc12 + Csc13);
			ke[0][1] = D12 + C12 + Cpg12 + R12 + Rpg11 + Csc12;
			ke[0][2] = D13 + C13 + Cpg13 + R12 + Rpg11 + Csc13;
			ke[1][0] = D12 + C11 + Cpg12 + R12 + Rpg21 + Csc12;
			ke[1][1] = -(D12 + D23) + C12 - (Cpg12 + Cpg23) + R11 + Rpg21 - (Csc12 + Csc23);
			ke[1][2] = D23 + C13 + Cpg23 + R12 + Rpg21 + Csc23;
			ke[2][0] = D13 + C11 + Cpg13 + R12 + Rpg31 + Csc13;
			ke[2][1] = D23 + C12 + Cpg23 + R12 + Rpg31 + Csc23;
			ke[2][2] = -(D13 + D23) + C13 - (Cpg13 + Cpg23) + R11 + Rpg31 - (Csc13 + Csc23);
			f[0] = Area*twelfth*(2*fe1 +  fe2  +  fe3 ) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32);
			f[1] = Area*twelfth*(  fe1 + 2*fe2 +  fe3 ) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13);
			f[2] = Area*twelfth*(  fe1 +  fe2  + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21);
		} else {
			double Mhh_1_12 = twelfth*Area, MhB_3_20 = three_twentieth*Area, MBh_3_20 = MhB_3_20;
			double a1 = bx*y23 + by*x32, a2 = bx*y31 + by*x13, a3 = bx*y12 + by*x21;
			double C12 = y23*y31 + x32*x13, C13 = y23*y12 + x32*x21, C23 = y31*y12 + x13*x21;
			double R11 = sixth*gamma*Area, R12 = twelfth*gamma*Area;
			double hs = h_shock(a.hshock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
			double cbtil = shock_capture_tr(a.shock, kx, ky, bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb,
			                                y23, y31, y12, x32, x13, x21, invArea, hs);
			double Eu = w*cbtil + (1-w)*a.dold[E];
			a.dold[E] = cbtil;
			double KDD12 = 0.25*Eu*invArea*C12, KDD13 = 0.25*Eu*invArea*C13, KDD23 = 0.25*Eu*invArea*C23;
			double Khh[3][3], KhB[3], KBh[3];
			Khh[0][0] = -(D12 + D13) + sixth*a1 + R11 -(KDD12 + KDD13);
			Khh[0][1] = D12 + sixth*a2 + R12 + KDD12;
			Khh[0][2] = D13 + sixth*a3 + R12 + KDD13;
			Khh[1][0] = D12 + sixth*a1 + R12 + KDD12;
			Khh[1][1] = -(D12 + D23) + sixth*a2 + R11 -(KDD12 + KDD23);
			Khh[1][2] = D23 + sixth*a3 + R12 + KDD23;
			Khh[2][0] = D13 + sixth*a1 + R12 + KDD13;
			Khh[2][1] = D23 + sixth*a2 + R12 + KDD23;
			Khh[2][2] = -(D13 + D23) + sixth*a3 + R11 -(KDD13 + KDD23);
			KhB[0] = nine_twentieth*(0.5*a1 + a2 + a3) + three_twentieth*gamma*Area;
			KhB[1] = nine_twentieth*(a1 + 0.5*a2 + a3) + three_twentieth*gamma*Area;
			KhB[2] = nine_twentieth*(a1 + a2 + 0.5*a3) + three_twentieth*gamma*Area;
			KBh[0] = nine_forty_cents*a1 + three_twentieth*gamma*Area;
			KBh[1] = nine_forty_cents*a2 + three_twentieth*gamma*Area;
			KBh[2] = nine_forty_cents*a3 + three_twentieth*gamma*Area;
			double KBB = -9*nine_forty_cents*(D12+D13+D23) + seventh*three_twentieth*(a1+ a2+ a3)
			             + 9*seventh*nine_forty_cents*Area - Eu*invArea*(C12 + C13 + C23)/360.;
			double invKBB = 1.0/KBB;
			double Fh[3];
			Fh[0] = twelfth*Area*(2*fe1 + fe2 + fe3);
			Fh[1] = twelfth*Area*(fe1 + 2*fe2 + fe3);
			Fh[2] = twelfth*Area*(fe1 + fe2 + 2*fe3);
			double FB = three_twentieth*Area*(fe1 + fe2 + fe3);
			for (int i = 0; i < 3; i++) {
				double m = Mhh_1_12 - invKBB*KhB[i]*MBh_3_20;
				me[i][0] = m; me[i][1] = m; me[i][2] = m;
				me[i][i] += Mhh_1_12;
				f[i] = Fh[i] - invKBB*KhB[i]*FB;
				for (int j = 0; j < 3; j++) ke[i][j] = Khh[i][j] - invKBB*KhB[i]*KBh[j];
			}
		}
		double *Ae = a.ke + 9LL*E, *re = a.re + 12LL*E;
		for (int i = 0; i < 3; i++) {
			re[4*i] = f[i];
			for (int j = 0; j < 3; j++) {
				Ae[3*i + j] = me[i][j] + a.adt*ke[i][j];
				re[4*i + 1 + j] = me[i][j]*due[j] + ke[i][j]*ue[j];
			}
		}
	}
}

// Build_M_F_DD.c:58-215, one thread per element: the DD form with the
// bubble kept as an unknown of the time loop (Predictor_New).  The bubble
// row is condensed with N2 = MBB + alpha dt KBB: Me = M1 - invN2 N1 M2^T goes
// to the element buffer, the residual contribution R1[i] - invN2 N1[i] R2 to
// re[12E + 4i] (the three product slots zero, so the gather adds it alone),
// and invN2, R2, M2 to the bubble buffer for calculate_DaB.
__global__ void __launch_bounds__(128) k_build_mfdd(BuildArgs a)
{
	const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
	const double seventh = 1.0/7.0, three_twentieth = 3./20.0, nine_twentieth = 9./20.0,
	             nine_forty_cents = 9./40.0, w = 0.5;
	const double kx = a.k, ky = a.k, gamma = a.gamma;
	for (int E = blockIdx.x * blockDim.x + threadIdx.x; E < a.nel; E += gridDim.x * blockDim.x) {
		int J1 = __ldg(&a.vert[3*E]), J2 = __ldg(&a.vert[3*E+1]), J3 = __ldg(&a.vert[3*E+2]);
		double X0 = __ldg(&a.x[J1]), X1 = __ldg(&a.x[J2]), X2 = __ldg(&a.x[J3]);
		double Y0 = __ldg(&a.y[J1]), Y1 = __ldg(&a.y[J2]), Y2 = __ldg(&a.y[J3]);
		double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
		double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
		double TwoA = x21*y31 - x13*y12, Area = 0.5*TwoA, invArea = 1.0/Area;
		double bx, by;
		if (a.beta_const) { bx = a.cbx; by = a.cby; }
		else { bx = __ldg(&a.beta[2*E]); by = __ldg(&a.beta[2*E+1]); }
		double fe1 = 0.0, fe2 = 0.0, fe3 = 0.0;
		if (!a.fsrc_zero) { fe1 = __ldg(&a.fsrc[3*E]); fe2 = __ldg(&a.fsrc[3*E+1]); fe3 = __ldg(&a.fsrc[3*E+2]); }
		double feb = third*(fe1+fe2+fe3);
		int i1 = __ldg(&a.node_id[J1]), i2 = __ldg(&a.node_id[J2]), i3 = __ldg(&a.node_id[J3]);
		double ue[3], due[3];
		ue[0] = (i1 >= 0) ? a.u[i1] : __ldg(&a.upresc[J1]);
		ue[1] = (i2 >= 0) ? a.u[i2] : __ldg(&a.upresc[J2]);
		ue[2] = (i3 >= 0) ? a.u[i3] : __ldg(&a.upresc[J3]);
		due[0] = (i1 >= 0) ? a.du[i1] : 0.0;
		due[1] = (i2 >= 0) ? a.du[i2] : 0.0;
		due[2] = (i3 >= 0) ? a.du[i3] : 0.0;
		double ueb = third * (ue[0] + ue[1] + ue[2]);
		double dueb = third * (due[0] + due[1] + due[2]);
		double Mhh_1_12 = twelfth*Area, MhB_3_20 = three_twentieth*Area, MBh_3_20 = MhB_3_20;
		double MBB = (81.0/280.)*Area;
		double a1 = bx*y23 + by*x32, a2 = bx*y31 + by*x13, a3 = bx*y12 + by*x21;
		double C12 = y23*y31 + x32*x13, C13 = y23*y12 + x32*x21, C23 = y31*y12 + x13*x21;
		double D12 = 0.25*invArea*((kx * y23 * y31) + (ky * x32 * x13));
		double D13 = 0.25*invArea*((kx * y23 * y12) + (ky * x32 * x21));
		double D23 = 0.25*invArea*((kx * y31 * y12) + (ky * x13 * x21));
		double R11 = sixth*gamma*Area, R12 = twelfth*gamma*Area;
		double hs = h_shock(a.hshock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
		double cbtil = shock_capture_tr(a.shock, kx, ky, bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb,
		                                y23, y31, y12, x32, x13, x21, invArea, hs);
		double Eu = w*cbtil + (1-w)*a.dold[E];
		a.dold[E] = cbtil;
		double KDD12 = 0.25*Eu*invArea*C12, KDD13 = 0.25*Eu*invArea*C13, KDD23 = 0.25*Eu*invArea*C23;
		double Khh[3][3], KhB[3], KBh[3];
		Khh[0][0] = -(D12 + D13) + sixth*a1 + R11 -(KDD12 + KDD13);
		Khh[0][1] = D12 + sixth*a2 + R12 + KDD12;
		Khh[0][2] = D13 + sixth*a3 + R12 + KDD13;
		Khh[1][0] = D12 + sixth*a1 + R12 + KDD12;
		Khh[1][1] = -(D12 + D23) + sixth*a2 + R11 -(KDD12 + KDD23);
		Khh[1][2] = D23 + sixth*a3 + R12 + KDD23;
		Khh[2][0] = D13 + sixth*a1 + R12 + KDD13;
		Khh[2][1] = D23 + sixth*a2 + R12 + KDD23;
		Khh[2][2] = -(D13 + D23) + sixth*a3 + R11 -(KDD13 + KDD23);
		KhB[0] = nine_twentieth*(0.5*a1 + a2 + a3) + three_twentieth*gamma*Area;
		KhB[1] = nine_twentieth*(a1 + 0.5*a2 + a3) + three_twentieth*gamma*Area;
		KhB[2] = nine_twentieth*(a1 + a2 + 0.5*a3) + three_twentieth*gamma*Area;
		KBh[0] = nine_forty_cents*a1 + three_twentieth*gamma*Area;
		KBh[1] = nine_forty_cents*a2 + three_twentieth*gamma*Area;
		KBh[2] = nine_forty_cents*a3 + three_twentieth*gamma*Area;
		double KBB = -9*nine_forty_cents*(D12+D13+D23) + seventh*three_twentieth*(a1+ a2+ a3)
		             + 9*seventh*nine_forty_cents*Area - Eu*invArea*(C12 + C13 + C23)/360.;
		double Fh[3];
		Fh[0] = twelfth*Area*(2*fe1 + fe2 + fe3);
		Fh[1] = twelfth*Area*(fe1 + 2*fe2 + fe3);
		Fh[2] = twelfth*Area*(fe1 + fe2 + 2*fe3);
		double FB = three_twentieth*Area*(fe1 + fe2 + fe3);
		const double alpha_dt_N2 = a.adt;                  // Alpha_Build * DeltaT_Build
		double N2 = MBB + alpha_dt_N2*KBB;
		double invN2 = 1.0/N2;
		const double uBe = a.uB[E], duBe = a.aB[E];
		double R2 = FB - MBB*duBe - KBB*uBe;
		double M1[3][3], M2[3], N1[3], R1[3];
		for (int i = 0; i < 3; i++) {
			M1[i][0] = Mhh_1_12; M1[i][1] = Mhh_1_12; M1[i][2] = Mhh_1_12;
			M1[i][i] += Mhh_1_12;
			M2[i] = MBh_3_20 + alpha_dt_N2*KBh[i];
			N1[i] = MhB_3_20 + alpha_dt_N2*KhB[i];
			R1[i] = Fh[i] - MhB_3_20*duBe - KhB[i]*uBe;
			R1[i] -= Mhh_1_12*due[i];
			for (int j = 0; j < 3; j++) {
				M1[i][j] += alpha_dt_N2*Khh[i][j];
				R1[i] -= Mhh_1_12*due[j] + Khh[i][j]*ue[j];
			}
			R2 -= MBh_3_20*due[i] + KBh[i]*ue[i];
		}
		double *Me = a.ke + 9LL*E, *re = a.re + 12LL*E, *bb = a.bub + 5LL*E;
		for (int i = 0; i < 3; i++) {
			for (int j = 0; j < 3; j++) Me[3*i + j] = M1[i][j] - invN2*N1[i]*M2[j];
			re[4*i] = R1[i] - invN2*N1[i]*R2;
			re[4*i + 1] = 0.0; re[4*i + 2] = 0.0; re[4*i + 3] = 0.0;
		}
		bb[0] = invN2; bb[1] = R2; bb[2] = M2[0]; bb[3] = M2[1]; bb[4] = M2[2];
	}
}

// calculate_DaB.c:8-29 and the bubble updates of Predictor_New.c:112-116:
// DaB = invN2 (R2 - M2 . Da[lm]), aB += DaB, uB += (alpha dt) DaB.
__global__ void k_bubble_correct(int nel, const int *__restrict__ lm, const double *__restrict__ bub,
                                 const double *__restrict__ Da, int neq, double *aB, double *uB, double c)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		const double *b = bub + 5LL * e;
		const int q1 = lm[3 * e], q2 = lm[3 * e + 1], q3 = lm[3 * e + 2];
		const double d1 = q1 == neq ? 0.0 : Da[q1], d2 = q2 == neq ? 0.0 : Da[q2], d3 = q3 == neq ? 0.0 : Da[q3];
		const double M2Da = b[2]*d1 + b[3]*d2 + b[4]*d3;
		const double DaB = b[0]*(b[1] - M2Da);
		aB[e] = aB[e] + 1.0*DaB;
		uB[e] = uB[e] + c*DaB;
	}
}

// Predictor_New.c:72-76 for the bubbles: uB += ((1 - alpha) dt) aB, aB = 0.
__global__ void k_bubble_predict(int nel, double *aB, double *uB, double c)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		uB[e] = uB[e] + c*aB[e];
		aB[e] = 0.0;
	}
}

// uB_InitialSolution.c:4-41: the mean of the element's nodal values.
__global__ void k_bubble_init(int nel, const int *__restrict__ vert, const int *__restrict__ node_id,
                              const double *__restrict__ u, const double *__restrict__ upresc, double *uB,
                              double *aB)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int k = 0; k < 3; k++) {
			const int v = vert[3 * e + k], id = node_id[v];
			s += id >= 0 ? u[id] : upresc[v];
		}
		uB[e] = s / 3;
		aB[e] = 0.0;
	}
}

extern "C" int fg_build_mfdd(femgpu_transport *t, double adt)
{
	BuildArgs a;
	a.x = t->x; a.y = t->y; a.u = t->u; a.upresc = t->upresc; a.beta = t->beta; a.fsrc = t->fsrc;
	a.vert = t->vert; a.node_id = t->node_id;
	a.k = t->k; a.gamma = t->gamma; a.cbx = t->cbx; a.cby = t->cby;
	a.nel = t->nel; a.shock = t->o.shock; a.hshock = t->o.hshock;
	a.beta_const = t->beta_const; a.fsrc_zero = t->fsrc_zero;
	a.ke = (t->o.scheme == FEMGPU_EBE) ? t->A : t->ke;
	a.fe = NULL;
	a.du = t->du; a.adt = adt; a.re = t->re; a.dold = t->dold;
	a.uB = t->uB; a.aB = t->aB; a.bub = t->bub;
	k_build_mfdd<<<fg_grid(t->nel, 128, 32), 128, 0, t->stream>>>(a);
	return (int)cudaGetLastError();
}

extern "C" int fg_bubble_correct(femgpu_transport *t, double c)
{
	k_bubble_correct<<<fg_grid(t->nel), FG_TPB, 0, t->stream>>>(t->nel, t->lm, t->bub, t->Da, t->neq, t->aB, t->uB, c);
	return (int)cudaGetLastError();
}

extern "C" int fg_bubble_predict(femgpu_transport *t, double c)
{
	k_bubble_predict<<<fg_grid(t->nel), FG_TPB, 0, t->stream>>>(t->nel, t->aB, t->uB, c);
	return (int)cudaGetLastError();
}

extern "C" int fg_bubble_init(femgpu_transport *t)
{
	k_bubble_init<<<fg_grid(t->nel), FG_TPB, 0, t->stream>>>(t->nel, t->vert, t->node_id, t->u, t->upresc, t->uB,
	                                                         t->aB);
	return (int)cudaGetLastError();
}

extern "C" int fg_build_transient(femgpu_transport *t, int dd, double adt)
{
	BuildArgs a;
	a.x = t->x; a.y = t->y; a.u = t->u; a.upresc = t->upresc; a.beta = t->beta; a.fsrc = t->fsrc;
	a.vert = t->vert; a.node_id = t->node_id;
	a.k = t->k; a.gamma = t->gamma; a.cbx = t->cbx; a.cby = t->cby;
	a.nel = t->nel; a.shock = t->o.shock; a.hshock = t->o.hshock;
	a.beta_const = t->beta_const; a.fsrc_zero = t->fsrc_zero;
	a.ke = (t->o.scheme == FEMGPU_EBE) ? t->A : t->ke;
	a.fe = NULL;
	a.du = t->du; a.adt = adt; a.re = t->re; a.dold = t->dold;
	if (dd) k_build_transient<true><<<fg_grid(t->nel, 128, 32), 128, 0, t->stream>>>(a);
	else k_build_transient<false><<<fg_grid(t->nel, 128, 32), 128, 0, t->stream>>>(a);
	return (int)cudaGetLastError();
}

// The transient residual gathered per equation: for each incident element in
// ascending order, R += load term, then R -= each of the three products
// (the reference's scatter order); R[neq] = 0.
__global__ void k_gather_R(int neq, const int *__restrict__ ri_ptr, const int *__restrict__ ri,
                           const double *__restrict__ re, double *R)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= neq; I += gridDim.x * blockDim.x) {
		double r = 0.0;
		if (I < neq) {
			for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
				int code = __ldg(&ri[q]), e = code / 3, aa = code - 3 * e;
				const double *p = re + 12LL * e + 4 * aa;
				r += __ldg(&p[0]);
				r -= __ldg(&p[1]);
				r -= __ldg(&p[2]);
				r -= __ldg(&p[3]);
			}
		}
		R[I] = r;
	}
}

// Predictor_Old.c:75-80: u_old = u, u += ((1 - alpha) dt) a, a = 0 ...
__global__ void k_tr_predict(double *u, double *a, double *uold, int n, double c)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		double ui = u[I];
		uold[I] = ui;
		u[I] = ui + c*a[I];
		a[I] = 0.0;
	}
}

// ... and :124-125 (daxpy): a += 1*Da, u += (alpha dt) Da.
__global__ void k_tr_correct(double *u, double *a, const double *Da, int n, double c)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		double d = Da[I];
		a[I] = a[I] + 1.0*d;
		u[I] = u[I] + c*d;
	}
}

// Predictor_Old_TRBDF2.c:57-58 (daxpy): y += c x, then x = 0.
__global__ void k_tr_axpy_zero(double *y, double *x, int n, double c)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		y[I] = y[I] + c*x[I];
		x[I] = 0.0;
	}
}

// Predictor_Old_BDF.c:111-115 / Predictor_Old_TRBDF2.c:101-105:
// u = cp p - cq q, a = 0 (u may be p).
__global__ void k_tr_lin(double *u, const double *p, const double *q, double *a, int n, double cp, double cq)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
		u[I] = cp*p[I] - cq*q[I];
		a[I] = 0.0;
	}
}

extern "C" int fg_tr_axpy_zero(femgpu_transport *t, double c)
{
	k_tr_axpy_zero<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(t->u, t->du, t->neq, c);
	return (int)cudaGetLastError();
}

extern "C" int fg_tr_lin(femgpu_transport *t, const double *p, const double *q, double cp, double cq)
{
	k_tr_lin<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(t->u, p, q, t->du, t->neq, cp, cq);
	return (int)cudaGetLastError();
}

// Predictor_New_BDF.c:144-147 / Predictor_New_TRBDF2.c:155-158 for the
// bubbles: uB = cp p - cq q, aB = 0 (uB may be p).
extern "C" int fg_bubble_lin(femgpu_transport *t, const double *p, const double *q, double cp, double cq)
{
	k_tr_lin<<<fg_grid(t->nel), FG_TPB, 0, t->stream>>>(t->uB, p, q, t->aB, t->nel, cp, cq);
	return (int)cudaGetLastError();
}

// Criteria.c:52-53: diff = u - u_old (into Da, free between steps).
__global__ void k_tr_diff(const double *u, const double *uold, double *d, int n)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) d[I] = u[I] - uold[I];
}

extern "C" int fg_tr_diff(femgpu_transport *t)
{
	k_tr_diff<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(t->u, t->uold, t->Da, t->neq);
	return (int)cudaGetLastError();
}

extern "C" int fg_tr_predict(femgpu_transport *t, double c)
{
	k_tr_predict<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(t->u, t->du, t->uold, t->neq, c);
	return (int)cudaGetLastError();
}

extern "C" int fg_tr_correct(femgpu_transport *t, double c)
{
	k_tr_correct<<<fg_grid(t->neq), FG_TPB, 0, t->stream>>>(t->u, t->du, t->Da, t->neq, c);
	return (int)cudaGetLastError();
}

// ------------------------------------------------------------ assembly ---
#define FG_ROWCAP 32

// F_assembly.c:5-27 for row I: for each incident element (ascending), add Fe
// then subtract the Dirichlet lift of every other vertex with Type == 0.
__device__ __forceinline__ double gather_F(int I, const int *ri_ptr, const int *ri, const double *ke,
                                           const double *fe, const int *vert, const int *node_type,
                                           const double *upresc)
{
	double F = 0.0;
	for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
		int code = __ldg(&ri[q]), e = code / 3, aa = code - 3 * e;
		F += __ldg(&fe[3LL * e + aa]);
		for (int b = 0; b < 3; b++) {
			if (b == aa) continue;
			int v = __ldg(&vert[3 * e + b]);
			if (__ldg(&node_type[v]) == 0) F -= __ldg(&ke[9LL * e + 3 * aa + b]) * __ldg(&upresc[v]);
		}
	}
	return F;
}

// CSR rows: csr_assembly.c:9-22 gathered per row, plus F.
__global__ void k_assemble_csr(int neq, int nnz, const int *IA, const int *sbe, const int *ri_ptr,
                               const int *ri, const double *ke, const double *fe, const int *vert,
                               const int *node_type, const double *upresc, double *AA, double *F,
                               int *err)
{
	double acc[FG_ROWCAP];
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x) {
		int base = IA[I], len = IA[I + 1] - base;
		if (len > FG_ROWCAP) { fg_set_err(err, FEMGPU_E_MESH); continue; }
		for (int q = 0; q < len; q++) acc[q] = 0.0;
		for (int q = ri_ptr[I]; q < ri_ptr[I + 1]; q++) {
			int code = __ldg(&ri[q]), e = code / 3, aa = code - 3 * e;
			for (int b = 0; b < 3; b++) {
				int pos = __ldg(&sbe[9 * e + 3 * aa + b]);
				if (pos < nnz) acc[pos - base] += __ldg(&ke[9LL * e + 3 * aa + b]);
			}
		}
		for (int q = 0; q < len; q++) AA[base + q] = acc[q];
		if (F) F[I] = gather_F(I, ri_ptr, ri, ke, fe, vert, node_type, upresc);
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) AA[nnz] = 0.0;
}

// EDE edges: ede_assembly.c:21-36 gathered per edge.
__global__ void k_assemble_ede(int nedge, const int *ec_ptr, const int *ec, const int *order,
                               const double *ke, double *A)
{
	for (int E = blockIdx.x * blockDim.x + threadIdx.x; E <= nedge; E += gridDim.x * blockDim.x) {
		double K0 = 0.0, K1 = 0.0, K2 = 0.0, K3 = 0.0;
		if (E < nedge) {
			for (int q = ec_ptr[E]; q < ec_ptr[E + 1]; q++) {
				int code = __ldg(&ec[q]), e = code / 3, s = code - 3 * e;
				int o0 = __ldg(&order[3 * e]), o1 = __ldg(&order[3 * e + 1]), o2 = __ldg(&order[3 * e + 2]);
				int Ia = (s == 2) ? o1 : o0, Ib = (s == 0) ? o1 : o2;
				const double *k = ke + 9LL * e;
				K0 += 0.5*__ldg(&k[3 * Ia + Ia]);
				K1 += __ldg(&k[3 * Ia + Ib]);
				K2 += __ldg(&k[3 * Ib + Ia]);
				K3 += 0.5*__ldg(&k[3 * Ib + Ib]);
			}
		}
		A[4LL * E] = K0; A[4LL * E + 1] = K1; A[4LL * E + 2] = K2; A[4LL * E + 3] = K3;
	}
}

__global__ void k_assemble_F(int neq, const int *ri_ptr, const int *ri, const double *ke,
                             const double *fe, const int *vert, const int *node_type,
                             const double *upresc, double *F)
{
	for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < neq; I += gridDim.x * blockDim.x)
		F[I] = gather_F(I, ri_ptr, ri, ke, fe, vert, node_type, upresc);
}

// Storage assembly of the transient element matrices (the same gathers as
// the steady build) and the residual gather into F.
extern "C" int fg_assemble_transient(femgpu_transport *t)
{
	cudaStream_t s = t->stream;
	int neq = t->neq;
	if (t->o.scheme == FEMGPU_CSR)
		k_assemble_csr<<<fg_grid(neq, 128, 32), 128, 0, s>>>(neq, t->nnz, t->IA, t->sbe, t->ri_ptr,
			t->ri, t->ke, NULL, t->vert, t->node_type, t->upresc, t->A, NULL, &t->st->err);
	else if (t->o.scheme == FEMGPU_EDE)
		k_assemble_ede<<<fg_grid(t->nedge + 1LL), FG_TPB, 0, s>>>(t->nedge, t->ec_ptr, t->ec, t->order,
			t->ke, t->A);
	k_gather_R<<<fg_grid(neq + 1LL), FG_TPB, 0, s>>>(neq, t->ri_ptr, t->ri, t->re, t->F);
	FG_TRY(cudaGetLastError());
	return t->o.scheme == FEMGPU_CSR ? fg_sell_refresh(t) : 0;
}

extern "C" int fg_assemble(femgpu_transport *t)
{
	cudaStream_t s = t->stream;
	int neq = t->neq;
	if (t->o.scheme == FEMGPU_CSR) {
		k_assemble_csr<<<fg_grid(neq, 128, 32), 128, 0, s>>>(neq, t->nnz, t->IA, t->sbe, t->ri_ptr,
			t->ri, t->ke, t->fe, t->vert, t->node_type, t->upresc, t->A, t->F, &t->st->err);
		FG_TRY(cudaGetLastError());
		return fg_sell_refresh(t);
	} else if (t->o.scheme == FEMGPU_EDE) {
		k_assemble_ede<<<fg_grid(t->nedge + 1LL), FG_TPB, 0, s>>>(t->nedge, t->ec_ptr, t->ec, t->order,
			t->ke, t->A);
		k_assemble_F<<<fg_grid(neq), FG_TPB, 0, s>>>(neq, t->ri_ptr, t->ri, t->ke, t->fe, t->vert,
			t->node_type, t->upresc, t->F);
	} else {
		k_assemble_F<<<fg_grid(neq), FG_TPB, 0, s>>>(neq, t->ri_ptr, t->ri, t->A, t->fe, t->vert,
			t->node_type, t->upresc, t->F);
	}
	return (int)cudaGetLastError();
}
