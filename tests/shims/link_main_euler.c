/*
 * Test infrastructure: the reference's own Predictor_Old.c (the time loop of
 * the Euler driver) with femgpu_shim_euler.c installed in its function
 * pointers.  Built only where the reference tree exists (tests/test_shims.py);
 * without a GPU the first Build fails and the shim prints and exits.
 */
#include "EulerEquations.h"
#include "../../../00_CommonFiles/Time_Integration/time_integration.h"

void femgpu_shim_euler_install(FemFunctionsType *, FemOtherFunctionsType *);

static double gam(double x, double y) { (void)x; (void)y; return 1.4; }
static double one(double x, double y) { (void)x; (void)y; return 1.0; }
static int init(ParametersType *P, NodeType *N, double *u) { (void)N; memset(u, 0, sizeof(double) * P->neq); return 0; }
static int stop_corr(ParametersType *P, double a, double b, int i) { (void)a; (void)b; return i >= P->NonLinearMaxIter; }
static int stop_time(ParametersType *P, double *u, double *uo, double t) { (void)P; (void)u; (void)uo; return t > 0.0; }
static int noscale(ParametersType *P, MatrixDataType *M, FemStructsType *FS) { (void)P; (void)M; (void)FS; return 0; }
static int nounscale(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *x)
{
	(void)P; (void)M; (void)FS; (void)x;
	return 0;
}

int main(void)
{
	static NodeType node[4];
	static ElementType el[2] = { {{0, 1, 2}, -1}, {{0, 2, 3}, -1} };
	static double u[5], F[5];
	ParametersType P;
	MatrixDataType M;
	FemStructsType FS;
	FemFunctionsType FF;
	FemOtherFunctionsType FOF;
	int I, k;
	memset(&P, 0, sizeof P); memset(&M, 0, sizeof M); memset(&FS, 0, sizeof FS);
	memset(&FF, 0, sizeof FF); memset(&FOF, 0, sizeof FOF);
	for (I = 0; I < 4; I++) {
		node[I].x = (I == 1 || I == 2); node[I].y = (I >= 2);
		for (k = 0; k < 4; k++) node[I].id[k] = I == 2 ? k : -1;
	}
	strcpy(P.MatrixVectorProductScheme, "EBE"); strcpy(P.StabilizationForm, "SUPG");
	strcpy(P.ShockCapture, "CAU"); strcpy(P.Preconditioner, "BlockDiag"); strcpy(P.Dimensionless, "NO");
	strcpy(P.Scaling, "NOT");
	P.SolverTolerance = 1e-8; P.StabilizationTolerance = 1e-6; P.Mach = 1.0; P.Alpha = 0.5; P.DeltaT = 1e-3;
	P.KrylovBasisVectorsQuantity = 10; P.LinearMaxIter = 10; P.NonLinearMaxIter = 2;
	P.nnodes = 4; P.nel = 2; P.neq = 4;
	FS.Node = node; FS.Element = el; FS.u = u; FS.F = F;
	FF.gamma = gam; FF.rhopresc = one; FF.v1presc = one; FF.v2presc = one; FF.epresc = one;
	FF.InitialSolution = init; FF.StopCriteria = stop_corr; FF.StopTimeIntegration = stop_time;
	FF.scaling = noscale; FF.unscaling = nounscale;
	femgpu_shim_euler_install(&FF, &FOF);
	return Predictor_Old(&P, &M, &FS, &FF, &FOF);
}
