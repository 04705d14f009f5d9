/*
 * femgpu_shim_ns.c -- binds libfemgpu into the steady Navier-Stokes driver
 * (04_SS_NavierStokes_Equations/2D) through the reference's own function
 * pointers (FemFunctionsType / FemOtherFunctionsType,
 * SSNavierStokesEquations.h:130-156): the VMS build (Build_K_F_MS), its
 * precond_setup and the 6-argument solver that the damped-Newton Process
 * (Process.c:62-194) calls, with EBE storage and BlockDiag (3x3 nodal
 * blocks) or CSR storage and ILU(0) or the DPA AMG ("AMG 2 NCL beta omega nr").
 *
 * Build, inside the driver's 01_CommonFiles (its own header):
 *     gcc -DSSNavierStokesEquations2D -I. -I<repo>/include -c femgpu_shim_ns.c
 * and link the driver with -lfemgpu -lcudart; without the reference tree,
 * -DFEMGPU_SHIM_OWN_TYPES takes the struct layout from shim_types_ns.h.
 * Call femgpu_shim_ns_install(FemFunctions, FemOtherFunctions) after the
 * driver's set*.c files, femgpu_shim_ns_release() in Postprocess.
 *
 * The first Build creates the device context from the nodes (Fill_ID.c
 * equation numbers, -1 prescribed), the elements, the prescribed values
 * v1presc / v2presc / ppresc and the body force f1ext / f2ext at every node,
 * ReynoldsNumber and VelMax.  The per-element stabilisation state
 * (delta_old, normres_old of Build_K_F_MS.c:260-265) lives on the device
 * between builds, starting from the first-call branch.  The solver reads the
 * driver's current forcing term (Parameters->SolverTolerance, which Process
 * updates through eta_newton.c) at every call.
 *
 * Errors: as femgpu_shim_transport.c (print and exit by default;
 * femgpu_shim_ns_set_abort(0) records and returns the code).
 */
#ifdef FEMGPU_SHIM_OWN_TYPES
#include "shim_types_ns.h"
#else
#include "SSNavierStokesEquations.h"
#endif
#include "femgpu.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

static femgpu_ns *g_ns;
static femgpu_amg *g_amg;

/* The deck's "AMG 2 NCL beta omega nr" (amg_precond.c:26-40): the DPA form
 * only; 0 on success. */
static int amg_of(const char *spec)
{
	int type = 0, ncl = 0, nr = 0;
	double beta = 0.0, omega = 0.0;
	if (g_amg) return 0;
	if (sscanf(spec, "AMG %d %d %lf %lf %d", &type, &ncl, &beta, &omega, &nr) != 5 || type != 2)
		return FEMGPU_E_ARG;
	return femgpu_amg_create(&g_amg, ncl, beta, omega, nr);
}
static int g_abort = 1, g_err, g_copy_matrix, g_fgmres;

/* A solve that reached its iteration limit is not a failure: the reference's
 * pgmres returns there too (pgmres.c:184), so it is only recorded. */
static int fail(const char *what, int rc)
{
	g_err = rc;
	if (g_abort && rc != FEMGPU_E_NOT_CONVERGED) {
		fprintf(stderr, "femgpu shim: %s failed (%d): %s\n", what, rc, femgpu_last_error());
		exit(1);
	}
	return rc;
}

void femgpu_shim_ns_set_abort(int on) { g_abort = on; }
int femgpu_shim_ns_error(void) { return g_err; }
femgpu_ns *femgpu_shim_ns_context(void) { return g_ns; }
/* copy != 0: every Build also copies the 9x9 element matrices into
 * MatrixData->Aaux (EBE storage); by default they stay on the device. */
void femgpu_shim_ns_copy_matrix(int copy) { g_copy_matrix = copy; }
/* fgmres != 0: flexible GMRES on the unpreconditioned residual. */
void femgpu_shim_ns_use_fgmres(int fgmres) { g_fgmres = fgmres; }

static int ns_of(ParametersType *P, FemStructsType *FS, FemFunctionsType *FF)
{
	int nn = P->nnodes, ne = P->nel, I, E, k, rc;
	femgpu_ns_opts o;
	double *x, *y, *up, *f;
	int *nid, *vert;
	if (g_ns) return 0;
	femgpu_ns_default_opts(&o);
	if (!strcasecmp(P->MatrixVectorProductScheme, "EBE")) o.scheme = FEMGPU_EBE;
	else if (!strcasecmp(P->MatrixVectorProductScheme, "CSR")) o.scheme = FEMGPU_CSR;
	else return FEMGPU_E_ARG;
	if (!strcasecmp(P->Preconditioner, "NOT")) o.precond = FEMGPU_PREC_NOT;
	else if (!strcasecmp(P->Preconditioner, "BlockDiag")) o.precond = FEMGPU_PREC_BLOCKDIAG;
	else if (!strcasecmp(P->Preconditioner, "ILU0") || !strcasecmp(P->Preconditioner, "ILU"))
		o.precond = FEMGPU_PREC_ILU0;
	else if (!strncmp(P->Preconditioner, "AMG", 3)) {
		if ((rc = amg_of(P->Preconditioner))) return rc;
		o.precond = FEMGPU_PREC_AMG;
	}
	else return FEMGPU_E_ARG;
	if (strcasecmp(P->StabilizationForm, "MS") != 0) return FEMGPU_E_ARG;
	o.re = P->ReynoldsNumber;
	o.velmax = P->VelMax;
	o.solver = g_fgmres ? FEMGPU_FGMRES : FEMGPU_PGMRES;
	o.kmax = P->KrylovBasisVectorsQuantity;
	o.lmax = P->LinearMaxIter;
	o.eta0 = P->SolverTolerance;
	o.eta_case = P->SolverToleranceCase;
	o.tol_nl = P->SolverToleranceNonLin;
	x = malloc(sizeof(double) * (size_t)nn);
	y = malloc(sizeof(double) * (size_t)nn);
	up = malloc(sizeof(double) * 3 * (size_t)nn);
	f = malloc(sizeof(double) * 2 * (size_t)nn);
	nid = malloc(sizeof(int) * 3 * (size_t)nn);
	vert = malloc(sizeof(int) * 3 * (size_t)ne);
	if (!x || !y || !up || !f || !nid || !vert) { rc = FEMGPU_E_NOMEM; goto out; }
	for (I = 0; I < nn; I++) {
		double xi = FS->Node[I].x, yi = FS->Node[I].y;
		x[I] = xi;
		y[I] = yi;
		for (k = 0; k < 3; k++) nid[3 * I + k] = FS->Node[I].id[k];
		up[3 * I] = FF->v1presc(xi, yi);
		up[3 * I + 1] = FF->v2presc(xi, yi);
		up[3 * I + 2] = FF->ppresc(xi, yi);
		f[2 * I] = FF->f1ext(xi, yi);
		f[2 * I + 1] = FF->f2ext(xi, yi);
	}
	for (E = 0; E < ne; E++)
		for (k = 0; k < 3; k++) vert[3 * E + k] = FS->Element[E].Vertex[k];
	rc = femgpu_ns_create(&g_ns, &o, nn, x, y, ne, vert, nid, P->neq, up, f);
	if (!rc && o.precond == FEMGPU_PREC_AMG) rc = femgpu_ns_set_amg(g_ns, g_amg);
out:
	free(x); free(y); free(up); free(f); free(nid); free(vert);
	return rc;
}

/* FemOtherFunctions->Build (Build_K_F_MS.c:8): element matrices and the
 * residual from FS->u, the residual into FS->F. */
int femgpu_shim_ns_Build(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF)
{
	int rc = ns_of(P, FS, FF);
	if (rc) return fail("Build (context)", rc);
	rc = femgpu_ns_build(g_ns, FS->u, g_copy_matrix && !strcasecmp(P->MatrixVectorProductScheme, "EBE")
	                                      ? M->Aaux : NULL, FS->F);
	return rc ? fail("Build", rc) : 0;
}

/* FemFunctions->precond_setup (BlockDiagDOF3_precond_EBE_setup.c or
 * ILUp_precond_setup.c): F := M^-1 F. */
int femgpu_shim_ns_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *FS, int tag, double *F)
{
	int rc;
	(void)P; (void)M; (void)FS; (void)tag;
	if (!g_ns) return fail("precond_setup", FEMGPU_E_NOT_BUILT);
	rc = femgpu_ns_precond_setup(g_ns, F);
	return rc ? fail("precond_setup", rc) : 0;
}

/* FemOtherFunctions->solver (SSNavierStokesEquations.h:152): A X = B to the
 * driver's current forcing term; the inner iterations are added to
 * Parameters->iterations. */
int femgpu_shim_ns_solver(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF,
                          double *B, double *X)
{
	int it = 0, rc;
	(void)M; (void)FS; (void)FF;
	if (!g_ns) return fail("solver", FEMGPU_E_NOT_BUILT);
	if ((rc = femgpu_ns_set_tol(g_ns, P->SolverTolerance))) return fail("solver (tolerance)", rc);
	rc = femgpu_ns_solve(g_ns, B, X, &it);
	P->iterations += it;
	return rc ? fail("solver", rc) : 0;
}

void femgpu_shim_ns_install(FemFunctionsType *FF, FemOtherFunctionsType *FOF)
{
	FF->precond_setup = femgpu_shim_ns_precond_setup;
	FOF->solver = femgpu_shim_ns_solver;
	FOF->Build = femgpu_shim_ns_Build;
}

void femgpu_shim_ns_release(void)
{
	if (g_ns) femgpu_ns_destroy(g_ns);
	if (g_amg) femgpu_amg_destroy(g_amg);
	g_ns = NULL;
	g_amg = NULL;
}
