/*
 * femgpu_shim_transport.c -- binds libfemgpu into the steady-transport
 * driver (01_SS_Transport_Equation/2D) through the reference's own function
 * pointers (FemFunctionsType / FemOtherFunctionsType,
 * 01_SS_Transport_Equation/2D/01_CommonFiles/SSTranspEquation.h:97-121).
 *
 * Build, inside the driver's 01_CommonFiles (its own header):
 *     gcc -DSSTranspEquation2D -I. -I<repo>/include -c femgpu_shim_transport.c
 * and link the driver with -lfemgpu -lcudart; without the reference tree,
 * -DFEMGPU_SHIM_OWN_TYPES takes the same struct layout from
 * shim_types_transport.h.  Then, where the driver's set*.c files assign the
 * pointers (after them, e.g. at the end of setStabilizationForm), call
 * femgpu_shim_transport_install(FemFunctions, FemOtherFunctions), and
 * femgpu_shim_transport_release() in Postprocess.
 *
 * The first Build creates the device context from the driver's structs:
 * node coordinates and types, element vertices, and the problem plug-ins
 * evaluated the way Build_K_F_SUPG.c:39-84 evaluates them (velocity at each
 * element's centroid, source at its vertices, prescribed value at every
 * node); options come from the parameter deck strings (Preprocess.c:44-62).
 * Host arrays stay authoritative: each call copies its vectors across.
 *
 * Errors: every function returns 0 or a negative FEMGPU_E_* code.  The
 * drivers ignore return values and the reference itself prints and exits on
 * failure (setPreconditioner.c:41-94, ILUp_precond_setup.c:161-162), so by
 * default a failing call does the same (message on stderr, exit(1));
 * femgpu_shim_transport_set_abort(0) makes it only record the code
 * (femgpu_shim_transport_error) and return it.
 */
#ifdef FEMGPU_SHIM_OWN_TYPES
#include "shim_types_transport.h"
#else
#include "SSTranspEquation.h"
#endif
#include "femgpu.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

static femgpu_transport *g_ctx;
static femgpu_transport_opts g_over;
static int g_have_over, g_abort = 1, g_err, g_copy_matrix;

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

void femgpu_shim_transport_set_abort(int on) { g_abort = on; }
int femgpu_shim_transport_error(void) { return g_err; }
femgpu_transport *femgpu_shim_transport_context(void) { return g_ctx; }

/* Options that the deck cannot express (FGMRES with the true-residual stop,
 * block ILU(0), mixed precision): taken instead of the deck-derived ones at
 * the context's creation; the deck still gives scheme, reordering,
 * preconditioner, shock capture, Krylov sizes and tolerances. */
void femgpu_shim_transport_set_options(const femgpu_transport_opts *o)
{
	if (o) { g_over = *o; g_have_over = 1; }
	else g_have_over = 0;
}

/* copy != 0: every Build also copies the matrix storage back into the
 * driver's arrays (MatrixData->AA for CSR, MatrixData->Aaux for EBE/EDE), for
 * drivers that read them; by default the matrix stays on the device. */
void femgpu_shim_transport_copy_matrix(int copy) { g_copy_matrix = copy; }

/* The deck's "ILU<p>" (setPreconditioner.c:80, ILUp_precond_setup.c:15):
 * level of fill p, or -1. */
static int ilu_level(const char *s)
{
	if (strncmp(s, "ILU", 3) != 0) return -1;
	return s[3] ? atoi(s + 3) : 0;
}

static int deck_options(const ParametersType *P, femgpu_transport_opts *o)
{
	femgpu_transport_default_opts(o);
	if (!strcasecmp(P->MatrixVectorProductScheme, "CSR")) o->scheme = FEMGPU_CSR;
	else if (!strcasecmp(P->MatrixVectorProductScheme, "EDE")) o->scheme = FEMGPU_EDE;
	else if (!strcasecmp(P->MatrixVectorProductScheme, "EBE")) o->scheme = FEMGPU_EBE;
	else return FEMGPU_E_ARG;
	o->reorder = !strcasecmp(P->reordering, "SYMRCM") ? FEMGPU_REORDER_SYMRCM : FEMGPU_REORDER_NOT;
	if (!strcasecmp(P->Preconditioner, "NOT")) o->precond = FEMGPU_PREC_NOT;
	else if (!strcasecmp(P->Preconditioner, "Diag")) o->precond = FEMGPU_PREC_DIAG;
	else if (ilu_level(P->Preconditioner) >= 0) {
		o->precond = FEMGPU_PREC_ILU0;
		o->ilu_level = ilu_level(P->Preconditioner);
	}
	else return FEMGPU_E_ARG;                   /* LU, SGS, SOR: not provided */
	if (strcasecmp(P->StabilizationForm, "SUPG") != 0) return FEMGPU_E_ARG;   /* DD: not provided */
	o->shock = !strcasecmp(P->ShockCapture, "YZBeta") ? FEMGPU_SHOCK_YZBETA : FEMGPU_SHOCK_CAU;
	if (!strcasecmp(P->h_Shock, "sqrtArea")) o->hshock = FEMGPU_H_SQRTAREA;
	else if (!strcasecmp(P->h_Shock, "Option1")) o->hshock = FEMGPU_H_OPTION1;
	else if (!strcasecmp(P->h_Shock, "Option2")) o->hshock = FEMGPU_H_OPTION2;
	else if (!strcasecmp(P->h_Shock, "2sqrtArea")) o->hshock = FEMGPU_H_2SQRTAREA;
	else return FEMGPU_E_ARG;                   /* "NOT" leaves the reference's pointer NULL */
	o->outflow = !strcasecmp(P->OutputFlow, "YES");
	o->kmax = P->KrylovBasisVectorsQuantity;
	o->lmax = P->SolverMaxIter;
	o->tol = P->SolverTolerance;
	o->nonlin_tol = P->NonLinearTolerance;
	return 0;
}

static int ctx_of(ParametersType *P, FemStructsType *FS, FemFunctionsType *FF)
{
	const double third = 1.0 / 3.0;
	int nn = P->nnodes, ne = P->nel, I, E, rc;
	femgpu_transport_opts o, deck;
	double *x, *y, *beta, *fsrc, *up, k, gamma;
	int *type, *vert;
	if (g_ctx) return 0;
	if ((rc = deck_options(P, &deck))) return rc;
	o = deck;
	if (g_have_over) {
		o = g_over;
		o.scheme = deck.scheme; o.reorder = deck.reorder; o.precond = deck.precond; o.shock = deck.shock;
		o.hshock = deck.hshock; o.outflow = deck.outflow; o.kmax = deck.kmax; o.lmax = deck.lmax;
		o.tol = deck.tol; o.nonlin_tol = deck.nonlin_tol; o.ilu_level = deck.ilu_level;
	}
	x = malloc(sizeof(double) * (size_t)nn);
	y = malloc(sizeof(double) * (size_t)nn);
	up = malloc(sizeof(double) * (size_t)nn);
	type = malloc(sizeof(int) * (size_t)nn);
	vert = malloc(sizeof(int) * 3 * (size_t)ne);
	beta = malloc(sizeof(double) * 2 * (size_t)ne);
	fsrc = malloc(sizeof(double) * 3 * (size_t)ne);
	if (!x || !y || !up || !type || !vert || !beta || !fsrc) { rc = FEMGPU_E_NOMEM; goto out; }
	k = FF->Condutivity();
	gamma = FF->Reaction();
	for (I = 0; I < nn; I++) {
		x[I] = FS->Node[I].x;
		y[I] = FS->Node[I].y;
		type[I] = FS->Node[I].Type;
		up[I] = FF->upresc(x[I], y[I]);
	}
	for (E = 0; E < ne; E++) {
		double X[3], Y[3], B[2];
		int a;
		for (a = 0; a < 3; a++) {
			vert[3 * E + a] = FS->Element[E].Vertex[a];
			X[a] = FS->Node[vert[3 * E + a]].x;
			Y[a] = FS->Node[vert[3 * E + a]].y;
		}
		FF->Velocity(third * (X[0] + X[1] + X[2]), third * (Y[0] + Y[1] + Y[2]), B);
		beta[2 * E] = B[0];
		beta[2 * E + 1] = B[1];
		for (a = 0; a < 3; a++) fsrc[3 * E + a] = FF->Font(X[a], Y[a], k, gamma, B[0], B[1]);
	}
	rc = femgpu_transport_create(&g_ctx, &o, nn, x, y, type, ne, vert, k, gamma, beta, NULL, fsrc, up);
out:
	free(x); free(y); free(up); free(type); free(vert); free(beta); free(fsrc);
	return rc;
}

/* FemOtherFunctions->Build (Build_K_F_SUPG.c:5): element matrices and RHS
 * from FS->u into the device storage and FS->F. */
int femgpu_shim_transport_Build(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF)
{
	double *A = NULL;
	int rc = ctx_of(P, FS, FF);
	if (rc) return fail("Build (context)", rc);
	if (g_copy_matrix) A = !strcasecmp(P->MatrixVectorProductScheme, "CSR") ? M->AA : M->Aaux;
	rc = femgpu_transport_build(g_ctx, FS->u, FS->F, A);
	return rc ? fail("Build", rc) : 0;
}

/* FemFunctions->precond_setup (ILUp_precond_setup.c:8-60, Diag_precond_*_setup):
 * factor, then F := M^-1 F. */
int femgpu_shim_transport_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *FS, int tag,
                                        double *F)
{
	int rc;
	(void)P; (void)M; (void)FS;
	if (!g_ctx) return fail("precond_setup", FEMGPU_E_NOT_BUILT);
	rc = femgpu_transport_precond_setup(g_ctx, tag, F);
	return rc ? fail("precond_setup", rc) : 0;
}

/* FemFunctions->precond (ILUp_precond.c, Diag_precond.c): z = M^-1 p, p == z allowed. */
int femgpu_shim_transport_precond(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *p, double *z)
{
	int rc;
	(void)P; (void)M; (void)FS;
	if (!g_ctx) return fail("precond", FEMGPU_E_NOT_BUILT);
	rc = femgpu_transport_precond(g_ctx, p, z);
	return rc ? fail("precond", rc) : 0;
}

/* FemFunctions->ProductMatrixVector (csrmv.c / ebemv.c / edemv.c): Q = A P. */
int femgpu_shim_transport_mv(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *Pv, double *Q)
{
	int rc;
	(void)P; (void)M; (void)FS;
	if (!g_ctx) return fail("ProductMatrixVector", FEMGPU_E_NOT_BUILT);
	rc = femgpu_transport_matvec(g_ctx, Pv, Q);
	return rc ? fail("ProductMatrixVector", rc) : 0;
}

/* FemOtherFunctions->solver, the 4-argument pgmres (pgmres.c:4-19): B =
 * FS->F (preconditioned by precond_setup), X = FS->u; the inner iterations
 * are added to SolverIterations (pgmres.c:191). */
int femgpu_shim_transport_solver(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF)
{
	int it = 0, rc;
	(void)M; (void)FF;
	if (!g_ctx) return fail("solver", FEMGPU_E_NOT_BUILT);
	rc = femgpu_transport_solve_bx(g_ctx, FS->F, FS->u, &it);
	P->SolverIterations += it;
	return rc ? fail("solver", rc) : 0;
}

void femgpu_shim_transport_install(FemFunctionsType *FF, FemOtherFunctionsType *FOF)
{
	FF->ProductMatrixVector = femgpu_shim_transport_mv;
	FF->precond = femgpu_shim_transport_precond;
	FF->precond_setup = femgpu_shim_transport_precond_setup;
	FOF->solver = femgpu_shim_transport_solver;
	FOF->Build = femgpu_shim_transport_Build;
}

void femgpu_shim_transport_release(void)
{
	if (g_ctx) femgpu_transport_destroy(g_ctx);
	g_ctx = NULL;
}
