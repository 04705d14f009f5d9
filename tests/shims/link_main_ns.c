/*
 * Test infrastructure: the reference's own steady Navier-Stokes Process.c
 * (the damped Newton loop with eta_newton.c's forcing terms) with
 * femgpu_shim_ns.c installed where the driver's set*.c files assign the
 * pointers.  Built (linked, not run) only where the reference tree exists.
 */
#include "SSNavierStokesEquations.h"

void femgpu_shim_ns_install(FemFunctionsType *, FemOtherFunctionsType *);

static double zero(double x, double y) { (void)x; (void)y; return 0.0; }

int setProblem(ParametersType *P, FemFunctionsType *FF)
{
	(void)P;
	FF->v1presc = zero; FF->v2presc = zero; FF->ppresc = zero; FF->f1ext = zero; FF->f2ext = zero;
	return 0;
}
int setMatrixVectorProductType(ParametersType *P, FemFunctionsType *FF) { (void)P; (void)FF; return 0; }
int setSolver(ParametersType *P, FemOtherFunctionsType *FOF) { (void)P; (void)FOF; return 0; }
int setPreconditioner(ParametersType *P, FemFunctionsType *FF) { (void)P; (void)FF; return 0; }
int setStabilizationForm(ParametersType *P, FemFunctionsType *FF, FemOtherFunctionsType *FOF)
{
	(void)P;
	femgpu_shim_ns_install(FF, FOF);
	return 0;
}

int main(void)
{
	ParametersType P;
	MatrixDataType M;
	FemStructsType FS;
	FemFunctionsType FF;
	FemOtherFunctionsType FOF;
	memset(&P, 0, sizeof P); memset(&M, 0, sizeof M); memset(&FS, 0, sizeof FS);
	memset(&FF, 0, sizeof FF); memset(&FOF, 0, sizeof FOF);
	return Process(&P, &M, &FS, &FF, &FOF);
}
