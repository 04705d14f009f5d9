/*
 * Test infrastructure only: drives the reference's AMG preconditioner
 * (00_CommonFiles/Solvers_and_Preconditioners/amg_precond.c with the
 * CSR/AMG sources: the double pairwise aggregation "DPA" hierarchy of
 * amg_dpa.c with either the counting-sort matching (matching_c) or the
 * BootCMatch half-approximate matching (bcm_linmatch.c), and its V-cycle with
 * SOR_relax / SOR_relax_rev), compiled from the reference's sources by
 * oracle/Makefile.  The CSR matrix, the deck's "AMG ..." string and the
 * vectors are given as arrays.
 */
#include "SSNavierStokesEquations.h"

void *mycalloc(char *, int, int);
int AMG_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int AMG_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int csrmv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);

#include "ref_gmres6.h"

static ParametersType *g_P;
static MatrixDataType *g_M;
static FemStructsType *g_FS;

/* AMG_precond_setup on (IA, JA, AA) (n rows, nnz entries) with the deck
 * string `spec` ("AMG 2 NCL beta omega nr"); F [n] in/out (F := M^-1 F).
 * info[0] = levels (matrices in the hierarchy). */
int ref_amg_setup(int n, const int *IA, const int *JA, const double *AA, const char *spec, double *F, int *info)
{
	g_P = mycalloc("P", 1, sizeof(ParametersType));
	g_M = mycalloc("M", 1, sizeof(MatrixDataType));
	g_FS = mycalloc("FS", 1, sizeof(FemStructsType));
	g_P->neq = n;
	g_P->nnzero = IA[n];
	strcpy(g_P->Preconditioner, spec);
	g_M->IA = mycalloc("IA", n + 1, sizeof(int));
	g_M->JA = mycalloc("JA", IA[n], sizeof(int));
	g_M->AA = mycalloc("AA", IA[n] + 1, sizeof(double));
	memcpy(g_M->IA, IA, sizeof(int) * (n + 1));
	memcpy(g_M->JA, JA, sizeof(int) * IA[n]);
	memcpy(g_M->AA, AA, sizeof(double) * IA[n]);
	AMG_precond_setup(g_P, g_M, g_FS, 1, F);
	info[0] = 2 * g_M->amg_precond_data->NCL + 1;
	return 0;
}

/* Level l of the hierarchy: sizes (n, nnz) and, when the arrays are given,
 * its CSR and (l < levels-1) the pairwise matching rmatch [n+1]. */
int ref_amg_level(int l, int *n_nnz, int *IA, int *JA, double *AA, int *rmatch)
{
	AMG_precond_data *d = g_M->amg_precond_data;
	matrix *A = d->A[l];
	n_nnz[0] = A->n;
	n_nnz[1] = A->nnz;
	if (IA) memcpy(IA, A->row_ptr, sizeof(int) * (A->n + 1));
	if (JA) memcpy(JA, A->col_ind, sizeof(int) * A->nnz);
	if (AA) memcpy(AA, A->val, sizeof(double) * A->nnz);
	if (rmatch && l < 2 * d->NCL) memcpy(rmatch, d->DPA_data->match[l], sizeof(int) * (A->n + 1));
	return 0;
}

/* pgmres (left preconditioned, the ref_gmres6.h adapter of pgmres.c:4-211)
 * with csrmv (MatrixVector_Operations/CSR/csrmv.c) and AMG_precond on the
 * system set up by ref_amg_setup: B [n] (already M^-1 F), X [n] out.
 * Returns the inner iterations. */
int ref_amg_gmres(int kmax, int lmax, double tol, double *B, double *X)
{
	FemFunctionsType *FF = mycalloc("FF", 1, sizeof(FemFunctionsType));
	g_P->KrylovBasisVectorsQuantity = kmax;
	g_P->LinearMaxIter = lmax;
	g_P->SolverTolerance = tol;
	g_P->iterations = 0;
	g_M->Aaux = NULL;
	FF->mv = csrmv;
	FF->precond = AMG_precond;
	gmres6(g_P, g_M, g_FS, FF, B, X);
	return g_P->iterations;
}

/* z = M^-1 p (one V-cycle, AMG_precond). */
int ref_amg_apply(const double *p, double *z)
{
	double *pp = mycalloc("p", g_P->neq + 1, sizeof(double));
	memcpy(pp, p, sizeof(double) * g_P->neq);
	AMG_precond(g_P, g_M, g_FS, pp, z);
	return 0;
}
