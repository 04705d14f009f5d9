/*
 * Test infrastructure: drives femgpu_shim_euler.c the way Predictor_Old.c:
 * 46-126 does (predict u += (1 - alpha) dt a, a = 0; per corrector Build,
 * scaling, precond_setup, the 6-argument solver, a += Da, u += alpha dt Da) through the
 * reference's struct layout (shim_types_euler.h), with the REFLETIDO
 * plug-ins: inflow x = 0 (1, 2.9, 0, 5.990715), top (1.7, 4.452878,
 * -0.860744, 9.870181681), rho v = 0 on the bottom wall, gamma 1.4.
 */
#include "shim_types_euler.h"
#include "femgpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

void femgpu_shim_euler_install(FemFunctionsType *, FemOtherFunctionsType *);
void femgpu_shim_euler_set_abort(int);
int femgpu_shim_euler_error(void);
void femgpu_shim_euler_release(void);

static double gam(double x, double y) { (void)x; (void)y; return 1.4; }
static int left(double x) { return fabs(x) <= 1e-15; }
static double rhop(double x, double y) { (void)y; return left(x) ? 1.0 : 1.7; }
static double v1p(double x, double y) { (void)y; return left(x) ? 2.9 : 4.452878; }
static double v2p(double x, double y) { return (left(x) || fabs(y) <= 1e-15) ? 0.0 : -0.860744; }
static double ep(double x, double y) { (void)y; return left(x) ? 5.990715 : 9.870181681; }

static int g_scaling;
/* on != 0: Scaling "BlockScaling", FemFunctions->scaling called after each
 * Build as Predictor_Old.c:73 does */
void drive_euler_set_scaling(int on) { g_scaling = on; }

/* nsteps time steps of ncorr correctors from u0 [neq+1]; uhist
 * [nsteps*(neq+1)], iters [nsteps*ncorr].  Returns 0 or a negative code. */
int drive_euler(int nnodes, const double *x, const double *y, int nel, const int *vert, const int *node_id, int neq,
                const double *u0, double alpha, double dt, double stab_tol, int kmax, int lmax, double tol,
                int nsteps, int ncorr, double *uhist, int *iters)
{
	ParametersType P;
	MatrixDataType M;
	FemStructsType FS;
	FemFunctionsType FF;
	FemOtherFunctionsType FOF;
	NodeType *node = calloc((size_t)nnodes, sizeof(NodeType));
	ElementType *el = calloc((size_t)nel, sizeof(ElementType));
	size_t n1 = (size_t)neq + 1;
	double *a = calloc(n1, sizeof(double)), *Da = calloc(n1, sizeof(double));
	int I, E, k, step, c, rc = 0;
	memset(&P, 0, sizeof P); memset(&M, 0, sizeof M); memset(&FS, 0, sizeof FS);
	memset(&FF, 0, sizeof FF); memset(&FOF, 0, sizeof FOF);
	strcpy(P.Solver, "GMRES");
	strcpy(P.TimeIntegration, "Predictor1");
	strcpy(P.MatrixVectorProductScheme, "EBE");
	strcpy(P.StabilizationForm, "SUPG");
	strcpy(P.ShockCapture, "CAU");
	strcpy(P.Preconditioner, "BlockDiag");
	strcpy(P.Scaling, g_scaling ? "BlockScaling" : "NOT");
	strcpy(P.StopMulticorrection, "ITERATION");
	strcpy(P.reordering, "NOT");
	strcpy(P.Dimensionless, "NO");
	strcpy(P.StopAtSteadyState, "NOT");
	P.SolverTolerance = tol;
	P.StabilizationTolerance = stab_tol;
	P.Mach = 1.0;
	P.Alpha = alpha; P.Alpha_Build = alpha;
	P.DeltaT = dt; P.DeltaT_Build = dt;
	P.KrylovBasisVectorsQuantity = kmax;
	P.LinearMaxIter = lmax;
	P.NonLinearMaxIter = ncorr;
	for (I = 0; I < nnodes; I++) {
		node[I].x = x[I];
		node[I].y = y[I];
		for (k = 0; k < 4; k++) node[I].id[k] = node_id[4 * I + k];
	}
	for (E = 0; E < nel; E++) {
		for (k = 0; k < 3; k++) el[E].Vertex[k] = vert[3 * E + k];
		el[E].Type = -1;
	}
	P.nnodes = nnodes; P.nel = nel; P.neq = neq;
	FS.Node = node; FS.Element = el;
	FS.u = calloc(n1, sizeof(double));
	FS.F = calloc(n1, sizeof(double));
	FS.du = a;
	memcpy(FS.u, u0, sizeof(double) * n1);
	FF.gamma = gam; FF.rhopresc = rhop; FF.v1presc = v1p; FF.v2presc = v2p; FF.epresc = ep;
	femgpu_shim_euler_set_abort(0);
	femgpu_shim_euler_install(&FF, &FOF);
	for (step = 0; step < nsteps && !rc; step++) {
		for (I = 0; I < neq; I++) {
			FS.u[I] += (1.0 - alpha) * dt * a[I];
			a[I] = 0.0;
		}
		for (c = 0; c < ncorr && !rc; c++) {
			int before = P.iterations;
			rc = FOF.Build(&P, &M, &FS, &FF);
			if (!rc) rc = FF.scaling(&P, &M, &FS);
			if (!rc) rc = FF.precond_setup(&P, &M, &FS, 1, FS.F);
			if (!rc) rc = FOF.solver(&P, &M, &FS, &FF, FS.F, Da);
			iters[step * ncorr + c] = P.iterations - before;
			for (I = 0; I < neq; I++) a[I] += 1 * Da[I];
			for (I = 0; I < neq; I++) FS.u[I] += alpha * dt * Da[I];
		}
		memcpy(uhist + (size_t)step * n1, FS.u, sizeof(double) * n1);
	}
	femgpu_shim_euler_release();
	free(node); free(el); free(FS.u); free(FS.F); free(a); free(Da);
	return rc;
}
