/*
 * Test infrastructure: drives femgpu_shim_transport.c the way the steady-
 * transport driver's Process.c:33-70 does -- Build, precond_setup (the call
 * Process.c:53 comments out, restored as the golden harness restores it),
 * the 4-argument solver -- through the reference's struct layout
 * (shim_types_transport.h), with the SKEW problem's plug-ins: constant k,
 * gamma and velocity, no source, u = 1 on x = 0 for y > 0.3.
 */
#include "shim_types_transport.h"
#include "femgpu.h"

#include <stdlib.h>
#include <string.h>

void femgpu_shim_transport_install(FemFunctionsType *, FemOtherFunctionsType *);
void femgpu_shim_transport_set_abort(int);
int femgpu_shim_transport_error(void);
void femgpu_shim_transport_release(void);

static double g_k, g_gamma, g_bx, g_by;
static double cond(void) { return g_k; }
static double reac(void) { return g_gamma; }
static void vel(double x, double y, double B[]) { (void)x; (void)y; B[0] = g_bx; B[1] = g_by; }
static double font(double x, double y, double k, double g, double bx, double by)
{
	(void)x; (void)y; (void)k; (void)g; (void)bx; (void)by;
	return 0.0;
}
static double upresc(double x, double y) { return (x == 0.0 && y > 0.3) ? 1.0 : 0.0; }
static double hflux(double x, double y) { (void)x; (void)y; return 0.0; }

/* npicard Picard steps from u = 0; F1 [neq+1] receives F after the first
 * Build, uhist [npicard*(neq+1)] u after each solve, iters the GMRES
 * iterations of each.  Returns the number of equations or a negative code. */
int drive_transport(int nnodes, const double *x, const double *y, const int *type, int nel, const int *vert,
                    double k, double gamma, double bx, double by, const char *scheme, const char *reord,
                    const char *precond, int kmax, int lmax, double tol, int npicard, double *F1, double *uhist,
                    int *iters)
{
	ParametersType P;
	MatrixDataType M;
	FemStructsType FS;
	FemFunctionsType FF;
	FemOtherFunctionsType FOF;
	NodeType *node = calloc((size_t)nnodes, sizeof(NodeType));
	ElementType *el = calloc((size_t)nel, sizeof(ElementType));
	int I, E, neq = 0, i, rc = 0;
	memset(&P, 0, sizeof P); memset(&M, 0, sizeof M); memset(&FS, 0, sizeof FS);
	memset(&FF, 0, sizeof FF); memset(&FOF, 0, sizeof FOF);
	strcpy(P.Solver, "GMRES");
	strncpy(P.Preconditioner, precond, sizeof P.Preconditioner - 1);
	strcpy(P.Scaling, "NOT");
	strncpy(P.reordering, reord, sizeof P.reordering - 1);
	strncpy(P.MatrixVectorProductScheme, scheme, sizeof P.MatrixVectorProductScheme - 1);
	strcpy(P.StabilizationForm, "SUPG");
	strcpy(P.ShockCapture, "CAU");
	strcpy(P.h_Shock, "2sqrtArea");
	strcpy(P.OutputFlow, "NO");
	P.SolverTolerance = tol;
	P.NonLinearTolerance = 0.0;
	P.KrylovBasisVectorsQuantity = kmax;
	P.SolverMaxIter = lmax;
	for (I = 0; I < nnodes; I++) {               /* Preprocess.c:73-81 */
		node[I].x = x[I];
		node[I].y = y[I];
		node[I].Type = type[I];
		node[I].id = type[I] >= 1 ? neq++ : -1;
	}
	for (E = 0; E < nel; E++) {
		for (i = 0; i < 3; i++) el[E].Vertex[i] = vert[3 * E + i];
		el[E].Type = -1;
	}
	P.nnodes = nnodes; P.nel = nel; P.neq = neq;
	FS.Node = node; FS.Element = el;
	FS.u = calloc((size_t)neq + 1, sizeof(double));
	FS.F = calloc((size_t)neq + 1, sizeof(double));
	g_k = k; g_gamma = gamma; g_bx = bx; g_by = by;
	FF.Condutivity = cond; FF.Reaction = reac; FF.Velocity = vel; FF.Font = font; FF.upresc = upresc;
	FF.hflux = hflux;
	femgpu_shim_transport_set_abort(0);
	femgpu_shim_transport_install(&FF, &FOF);
	for (i = 1; i <= npicard && !rc; i++) {
		int before = P.SolverIterations;
		rc = FOF.Build(&P, &M, &FS, &FF);
		if (!rc && i == 1) memcpy(F1, FS.F, sizeof(double) * ((size_t)neq + 1));
		if (!rc) rc = FF.precond_setup(&P, &M, &FS, i, FS.F);
		if (!rc) rc = FOF.solver(&P, &M, &FS, &FF);
		iters[i - 1] = P.SolverIterations - before;
		memcpy(uhist + (size_t)(i - 1) * ((size_t)neq + 1), FS.u, sizeof(double) * ((size_t)neq + 1));
	}
	femgpu_shim_transport_release();
	free(node); free(el); free(FS.u); free(FS.F);
	return rc ? rc : neq;
}
