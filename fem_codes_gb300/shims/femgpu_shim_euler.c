/*
 * femgpu_shim_euler.c -- binds libfemgpu into the 2D Euler driver
 * (03_Euler_Equations/2D) through the reference's own function pointers
 * (FemFunctionsType / FemOtherFunctionsType, EulerEquations.h:136-170), for
 * EBE storage with the nodal block-diagonal preconditioner or CSR storage
 * (reordering NOT) with ILU(0) or the DPA AMG, and the predictor-multicorrector
 * (Predictor_Old.c) that calls Build, precond_setup and the 6-argument
 * solver once per corrector.
 *
 * Build, inside the driver's 01_CommonFiles (its own header):
 *     gcc -DEulerEquations2D -I. -I<repo>/include -c femgpu_shim_euler.c
 * and link the driver with -lfemgpu -lcudart; without the reference tree,
 * -DFEMGPU_SHIM_OWN_TYPES takes the struct layout from shim_types_euler.h.
 * Call femgpu_shim_euler_install(FemFunctions, FemOtherFunctions) after the
 * driver's set*.c files have assigned their pointers, and
 * femgpu_shim_euler_release() in Postprocess.
 *
 * The first Build creates the device context: node coordinates, element
 * vertices, the equation numbers of Fill_ID.c (Node[I].id[k], -1 prescribed)
 * and the prescribed values rhopresc / v1presc / v2presc / epresc at every
 * node (as eval_U_dU.c:27-90 evaluates them); gamma (constant in every
 * problem plug-in), Alpha, DeltaT, StabilizationTolerance, Mach and
 * Dimensionless are read from the deck at that call.
 *
 * Errors: as femgpu_shim_transport.c -- by default a failing call prints and
 * exits, as the reference does; femgpu_shim_euler_set_abort(0) only records
 * and returns the code.
 */
#ifdef FEMGPU_SHIM_OWN_TYPES
#include "shim_types_euler.h"
#else
#include "EulerEquations.h"
#endif
#include "femgpu.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

static femgpu_euler *g_eu;
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

void femgpu_shim_euler_set_abort(int on) { g_abort = on; }
int femgpu_shim_euler_error(void) { return g_err; }
femgpu_euler *femgpu_shim_euler_context(void) { return g_eu; }
/* copy != 0: every Build also copies the matrix storage back -- the 12x12
 * element matrices into MatrixData->Aaux (EBE layout A[e][144]) or the CSR
 * values into MatrixData->AA; by default they stay on the device. */
void femgpu_shim_euler_copy_matrix(int copy) { g_copy_matrix = copy; }
/* fgmres != 0: flexible GMRES accepted on the unpreconditioned residual (and
 * precond_setup leaves R unpreconditioned) instead of the reference's pgmres. */
void femgpu_shim_euler_use_fgmres(int fgmres) { g_fgmres = fgmres; }

static int eu_of(ParametersType *P, FemStructsType *FS, FemFunctionsType *FF)
{
	int nn = P->nnodes, ne = P->nel, I, E, k, rc;
	femgpu_euler_opts o;
	double *x, *y, *up;
	int *nid, *vert;
	if (g_eu) return 0;
	femgpu_euler_default_opts(&o);
	/* setStabilizationForm.c:6-75: SUPG (CAU, YZBeta) or DD (CAUDD, YZBeta) */
	if (!strcasecmp(P->StabilizationForm, "DD")) o.stab = FEMGPU_STAB_DD;
	else if (strcasecmp(P->StabilizationForm, "SUPG") != 0) return FEMGPU_E_ARG;
	if (!strcasecmp(P->ShockCapture, "YZBeta")) o.shock = FEMGPU_SHOCK_YZBETA;
	else if (o.stab == FEMGPU_STAB_DD && !strcasecmp(P->ShockCapture, "CAUDD")) o.shock = FEMGPU_SHOCK_CAUDD;
	else if (o.stab != FEMGPU_STAB_SUPG || strcasecmp(P->ShockCapture, "CAU") != 0) return FEMGPU_E_ARG;
	for (k = 0; k < 4; k++) o.invY[k] = P->invY[k];
	if (!strcasecmp(P->MatrixVectorProductScheme, "EBE")) o.scheme = FEMGPU_EBE;
	else if (!strcasecmp(P->MatrixVectorProductScheme, "CSR") && !strcasecmp(P->reordering, "NOT"))
		o.scheme = FEMGPU_CSR;
	else return FEMGPU_E_ARG;
	if (!strcasecmp(P->Preconditioner, "NOT")) o.precond = FEMGPU_PREC_NOT;
	else if (!strcasecmp(P->Preconditioner, "BlockDiag") && o.scheme == FEMGPU_EBE) o.precond = FEMGPU_PREC_BLOCKDIAG;
	else if (!strncmp(P->Preconditioner, "ILU", 3) && (!P->Preconditioner[3] || atoi(P->Preconditioner + 3) == 0) &&
	         o.scheme == FEMGPU_CSR) o.precond = FEMGPU_PREC_ILU0;
	else if (!strncmp(P->Preconditioner, "AMG", 3) && o.scheme == FEMGPU_CSR) {
		if ((rc = amg_of(P->Preconditioner))) return rc;
		o.precond = FEMGPU_PREC_AMG;
	}
	else return FEMGPU_E_ARG;
	o.gamma = FF->gamma(FS->Node[0].x, FS->Node[0].y);
	o.mach = P->Mach;
	o.dimensionless = !strcasecmp(P->Dimensionless, "YES");
	o.alpha = P->Alpha;
	o.dt = P->DeltaT;
	o.stab_tol = P->StabilizationTolerance;
	o.solver = g_fgmres ? FEMGPU_FGMRES : FEMGPU_PGMRES;
	o.kmax = P->KrylovBasisVectorsQuantity;
	o.lmax = P->LinearMaxIter;
	o.tol = P->SolverTolerance;
	o.ncorr = P->NonLinearMaxIter;
	x = malloc(sizeof(double) * (size_t)nn);
	y = malloc(sizeof(double) * (size_t)nn);
	up = malloc(sizeof(double) * 4 * (size_t)nn);
	nid = malloc(sizeof(int) * 4 * (size_t)nn);
	vert = malloc(sizeof(int) * 3 * (size_t)ne);
	if (!x || !y || !up || !nid || !vert) { rc = FEMGPU_E_NOMEM; goto out; }
	for (I = 0; I < nn; I++) {
		double xi = FS->Node[I].x, yi = FS->Node[I].y;
		x[I] = xi;
		y[I] = yi;
		for (k = 0; k < 4; k++) nid[4 * I + k] = FS->Node[I].id[k];
		up[4 * I] = FF->rhopresc(xi, yi);
		up[4 * I + 1] = FF->v1presc(xi, yi);
		up[4 * I + 2] = FF->v2presc(xi, yi);
		up[4 * I + 3] = FF->epresc(xi, yi);
	}
	for (E = 0; E < ne; E++)
		for (k = 0; k < 3; k++) vert[3 * E + k] = FS->Element[E].Vertex[k];
	rc = femgpu_euler_create(&g_eu, &o, nn, x, y, ne, vert, nid, P->neq, up);
	if (!rc && o.precond == FEMGPU_PREC_AMG) rc = femgpu_euler_set_amg(g_eu, g_amg);
	/* slip walls: the nodes with v1Type == -1, rotated by BC_theta as
	 * Build_M_K_F_SUPG.c:1044-1056 and rotation.c:6-7 do */
	if (!rc) {
		int nslip = 0, *slip = calloc((size_t)nn, sizeof(int));
		double *cs = malloc(sizeof(double) * (size_t)nn), *sn = malloc(sizeof(double) * (size_t)nn);
		if (!slip || !cs || !sn) rc = FEMGPU_E_NOMEM;
		for (I = 0; !rc && I < nn; I++) {
			cs[I] = 1.0;
			sn[I] = 0.0;
			if (FS->Node[I].v1Type == -1) {
				double th = FF->BC_theta(FS->Node[I].x, FS->Node[I].y);
				slip[I] = 1;
				cs[I] = cos(th);
				sn[I] = sin(th);
				nslip++;
			}
		}
		if (!rc && nslip) rc = femgpu_euler_set_slip(g_eu, slip, cs, sn);
		free(slip); free(cs); free(sn);
	}
out:
	free(x); free(y); free(up); free(nid); free(vert);
	return rc;
}

/* FemOtherFunctions->Build (Build_M_K_F_SUPG.c:6): Ae = Me + alpha dt Ke and
 * R = -(Me du + Ke u) from FS->u and FS->du, R into FS->F (CSR storage: the
 * element matrices assembled into the pattern, csr_assembly.c). */
int femgpu_shim_euler_Build(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF)
{
	const int csr = !strcasecmp(P->MatrixVectorProductScheme, "CSR");
	int rc = eu_of(P, FS, FF);
	if (rc) return fail("Build (context)", rc);
	/* the time loop's Alpha_Build / DeltaT_Build (Build_M_K_F_SUPG.c:19-20) */
	if (P->DeltaT_Build > 0.0) rc = femgpu_euler_set_build_params(g_eu, P->Alpha_Build, P->DeltaT_Build);
	if (!rc) rc = femgpu_euler_build(g_eu, FS->u, FS->du, g_copy_matrix && !csr ? M->Aaux : NULL, FS->F);
	if (!rc && g_copy_matrix && csr) {
		int nn[2];
		rc = femgpu_euler_csr(g_eu, nn, NULL, NULL, NULL, M->AA);
	}
	return rc ? fail("Build", rc) : 0;
}

/* FemFunctions->precond_setup (BlockDiag_precond_EBE_setup.c:6-86): the
 * nodal 4x4 blocks, their inverses, then F := D^-1 F. */
int femgpu_shim_euler_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *FS, int tag, double *F)
{
	int rc;
	(void)P; (void)M; (void)FS; (void)tag;
	if (!g_eu) return fail("precond_setup", FEMGPU_E_NOT_BUILT);
	rc = femgpu_euler_precond_setup(g_eu, F);
	return rc ? fail("precond_setup", rc) : 0;
}

/* FemFunctions->mv (ebemvNDOF4.c:5-112): Q = A P (EBE storage). */
int femgpu_shim_euler_mv(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *Pv, double *Q)
{
	int rc;
	(void)M; (void)FS;
	if (!g_eu) return fail("mv", FEMGPU_E_NOT_BUILT);
	if (strcasecmp(P->MatrixVectorProductScheme, "EBE") != 0) return fail("mv (CSR storage)", FEMGPU_E_ARG);
	rc = femgpu_ebe_matvec(femgpu_euler_ebe(g_eu), Pv, Q);
	return rc ? fail("mv", rc) : 0;
}

/* FemFunctions->precond (BlockDiag_precond.c): z = D^-1 p, p == z allowed
 * (EBE storage). */
int femgpu_shim_euler_precond(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *p, double *z)
{
	int rc;
	(void)M; (void)FS;
	if (!g_eu) return fail("precond", FEMGPU_E_NOT_BUILT);
	if (strcasecmp(P->Preconditioner, "BlockDiag") != 0) return fail("precond (not BlockDiag)", FEMGPU_E_ARG);
	rc = femgpu_ebe_blockdiag_apply(femgpu_euler_ebe(g_eu), p, z);
	return rc ? fail("precond", rc) : 0;
}

/* FemFunctions->scaling = Block_scaling_EBE (Block_scaling.c:7-49, chosen by
 * setScaling.c:10-13 for Scaling "BlockScaling"): the element matrices
 * scaled by the inverse nodal blocks on the device and F := D^-1 F; with
 * femgpu_shim_euler_copy_matrix the scaled matrices are copied to Aaux.
 * Scaling "NOT" does nothing, as NO_scaling (scaling.c) does. */
int femgpu_shim_euler_scaling(ParametersType *P, MatrixDataType *M, FemStructsType *FS)
{
	int rc;
	if (!strcasecmp(P->Scaling, "NOT")) return 0;
	if (strcasecmp(P->Scaling, "BlockScaling") != 0) return fail("scaling (unknown Scaling)", FEMGPU_E_ARG);
	if (!g_eu) return fail("scaling", FEMGPU_E_NOT_BUILT);
	if (strcasecmp(P->MatrixVectorProductScheme, "EBE") != 0) return fail("scaling (CSR storage)", FEMGPU_E_ARG);
	rc = femgpu_euler_scale(g_eu, FS->F, g_copy_matrix ? M->Aaux : NULL);
	return rc ? fail("scaling", rc) : 0;
}

/* FemOtherFunctions->solver (EulerEquations.h:168): A X = B by the
 * reference's pgmres (or FGMRES, femgpu_shim_euler_use_fgmres); the inner
 * iterations are added to Parameters->iterations. */
int femgpu_shim_euler_solver(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF,
                             double *B, double *X)
{
	int it = 0, rc;
	(void)M; (void)FS; (void)FF;
	if (!g_eu) return fail("solver", FEMGPU_E_NOT_BUILT);
	rc = femgpu_euler_solve(g_eu, B, X, &it);
	P->iterations += it;
	return rc ? fail("solver", rc) : 0;
}

void femgpu_shim_euler_install(FemFunctionsType *FF, FemOtherFunctionsType *FOF)
{
	FF->mv = femgpu_shim_euler_mv;
	FF->precond = femgpu_shim_euler_precond;
	FF->precond_setup = femgpu_shim_euler_precond_setup;
	FF->scaling = femgpu_shim_euler_scaling;
	FOF->solver = femgpu_shim_euler_solver;
	FOF->Build = femgpu_shim_euler_Build;
}

void femgpu_shim_euler_release(void)
{
	if (g_eu) femgpu_euler_destroy(g_eu);
	if (g_amg) femgpu_amg_destroy(g_amg);
	g_eu = NULL;
	g_amg = NULL;
}
