/*
 * Test infrastructure: a steady-transport driver made of the reference's own
 * Process.c (its Picard loop) with femgpu_shim_transport.c installed in
 * place of the reference's set*.c assignments -- what a maintainer's edit of
 * setStabilizationForm.c would do.  Built only where the reference tree
 * exists (tests/test_shims.py); run without a GPU it exercises the shim's
 * error path (print and exit, as the reference does on a failure).
 */
#include "SSTranspEquation.h"

void femgpu_shim_transport_install(FemFunctionsType *, FemOtherFunctionsType *);

static double cond(void) { return 1e-4; }
static double reac(void) { return 0.0; }
static void vel(double x, double y, double B[]) { (void)x; (void)y; B[0] = 0.8660254037844387; B[1] = 0.5; }
static double font(double x, double y, double k, double g, double bx, double by)
{
	(void)x; (void)y; (void)k; (void)g; (void)bx; (void)by;
	return 0.0;
}
static double upresc(double x, double y) { return (x == 0.0 && y > 0.3) ? 1.0 : 0.0; }
static double hflux(double x, double y) { (void)x; (void)y; return 0.0; }

int setProblem(ParametersType *P, FemFunctionsType *FF)
{
	(void)P;
	FF->Condutivity = cond; FF->Reaction = reac; FF->Velocity = vel; FF->Font = font; FF->upresc = upresc;
	FF->hflux = hflux;
	return 0;
}
int setMatrixVectorProductType(ParametersType *P, FemFunctionsType *FF) { (void)P; (void)FF; return 0; }
int setSolver(ParametersType *P, FemOtherFunctionsType *FOF) { (void)P; (void)FOF; return 0; }
int setScaling(ParametersType *P, FemFunctionsType *FF) { (void)P; (void)FF; return 0; }
int setPreconditioner(ParametersType *P, FemFunctionsType *FF) { (void)P; (void)FF; return 0; }
int setStabilizationForm(ParametersType *P, FemFunctionsType *FF, FemOtherFunctionsType *FOF)
{
	(void)P;
	femgpu_shim_transport_install(FF, FOF);
	return 0;
}

int main(void)
{
	/* two cells of the unit square, the inflow edges prescribed */
	static NodeType node[6] = { {0, 0, 0, -1}, {0.5, 0, 0, -1}, {1, 0, 0, -1},
	                            {0, 1, 0, -1}, {0.5, 1, 1, 0}, {1, 1, 1, 1} };
	static ElementType el[4] = { {{0, 1, 4}, -1}, {{0, 4, 3}, -1}, {{1, 2, 5}, -1}, {{1, 5, 4}, -1} };
	static double u[3], F[3];
	ParametersType P;
	MatrixDataType M;
	FemStructsType FS;
	FemFunctionsType FF;
	FemOtherFunctionsType FOF;
	memset(&P, 0, sizeof P); memset(&M, 0, sizeof M); memset(&FS, 0, sizeof FS);
	memset(&FF, 0, sizeof FF); memset(&FOF, 0, sizeof FOF);
	strcpy(P.Solver, "GMRES"); strcpy(P.Preconditioner, "NOT"); strcpy(P.Scaling, "NOT");
	strcpy(P.reordering, "NOT"); strcpy(P.MatrixVectorProductScheme, "CSR");
	strcpy(P.StabilizationForm, "SUPG"); strcpy(P.ShockCapture, "CAU"); strcpy(P.h_Shock, "2sqrtArea");
	strcpy(P.OutputFlow, "NO");
	P.SolverTolerance = 1e-8; P.NonLinearTolerance = 1e-6; P.KrylovBasisVectorsQuantity = 10;
	P.SolverMaxIter = 10; P.nnodes = 6; P.nel = 4; P.neq = 2;
	FS.Node = node; FS.Element = el; FS.u = u; FS.F = F;
	return Process(&P, &M, &FS, &FF, &FOF);
}
