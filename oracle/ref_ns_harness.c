/*
 * Test infrastructure only: drives the reference's steady Navier-Stokes VMS
 * (NSGS) element build (04_SS_NavierStokes_Equations/2D/01_CommonFiles/
 * Build_K_F_MS.c with eval_U.c, ebe_assembly.c and the CAVITY plug-ins) and
 * its damped-Newton loop (Process.c:62-194 control flow with eta_newton.c),
 * on in-memory arrays, with EBE storage and BlockDiagDOF3 preconditioning, or
 * CSR storage (csr_Initialization.c, csr_assembly.c, reordering NOT) with
 * ILU(0) (ILUp_precond_setup.c / ILUp_precond.c) and csrmv -- the drivers'
 * two configurations -- and the 6-argument GMRES adapter of ref_gmres6.h;
 * compiled from the reference's sources by oracle/Makefile with
 * -DSSNavierStokesEquations2D.
 *
 * Build_K_F_MS keeps a file-scope counter of its calls (varglobal, :6) that
 * switches the first build's delta update: load a fresh copy of this library
 * for every independent run.
 */
#include "SSNavierStokesEquations.h"

void *mycalloc(char *, int, int);
int ebemvNDOF3(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int BlockDiagDOF3_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int BlockDiagDOF3_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
double CAVITY_v1presc(double, double);
double CAVITY_v2presc(double, double);
double CAVITY_ppresc(double, double);
double CAVITY_f1ext(double, double);
double CAVITY_f2ext(double, double);
int daxpy(int, double, double *, double *);
int dcopy(int, double *, double *);
int csrmv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int ILUp_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int ILUp_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);

#include "ref_gmres6.h"

/* csr != 0: CSR storage with ILU(0), as Preprocess.c:138-160 sets it up. */
static void setup(int csr, int nnodes, const double *x, const double *y, const int *node_id, int nel,
                  const int *vert, int neq, double Re, double velmax, ParametersType **Po, MatrixDataType **Mo,
                  FemStructsType **FSo, FemFunctionsType **FFo)
{
	int I, k;
	ParametersType *P = mycalloc("P", 1, sizeof(ParametersType));
	MatrixDataType *M = mycalloc("M", 1, sizeof(MatrixDataType));
	FemStructsType *FS = mycalloc("FS", 1, sizeof(FemStructsType));
	FemFunctionsType *FF = mycalloc("FF", 1, sizeof(FemFunctionsType));
	NodeType *Node = mycalloc("Node", nnodes, sizeof(NodeType));
	ElementType *El = mycalloc("El", nel, sizeof(ElementType));
	int **lm = mycalloc("lm", nel, sizeof(int *)), *lmaux = mycalloc("lmaux", nel * 9, sizeof(int));
	double **A = mycalloc("A", nel, sizeof(double *)), *Aaux = mycalloc("Aaux", nel * 81, sizeof(double));
	P->nnodes = nnodes; P->nel = nel; P->neq = neq;
	P->ReynoldsNumber = Re; P->VelMax = velmax;
	strcpy(P->MatrixVectorProductScheme, csr ? "CSR" : "EBE");
	strcpy(P->Preconditioner, csr ? "ILU0" : "BlockDiag");
	strcpy(P->reordering, "NOT");
	for (I = 0; I < nnodes; I++) {
		Node[I].x = x[I]; Node[I].y = y[I];
		for (k = 0; k < 3; k++) Node[I].id[k] = node_id[3 * I + k];
	}
	for (I = 0; I < nel; I++) {
		for (k = 0; k < 3; k++) El[I].Vertex[k] = vert[3 * I + k];
		lm[I] = lmaux + 9 * I;
		A[I] = Aaux + 81 * I;
	}
	Fill_LM(neq, nel, lm, Node, El);
	M->A = A; M->Aaux = Aaux;
	if (csr) {
		int *IA, *JA, *perm, *invperm, **sbe;
		csr_Initialization(P, Node, &JA, &IA, &perm, &invperm, &lm, &lmaux, &sbe);
		M->AA = mycalloc("AA", P->nnzero + 1, sizeof(double));
		M->IA = IA; M->JA = JA; M->Scheme_by_Element = sbe; M->Perm = perm; M->invPerm = invperm;
	}
	FS->lm = lm; FS->Node = Node; FS->Element = El;
	FS->F = mycalloc("F", neq + 1, sizeof(double));
	FS->u = mycalloc("u", neq + 1, sizeof(double));
	FS->delta_old = mycalloc("delta_old", nel, sizeof(double));
	FS->normres_old = mycalloc("normres_old", nel, sizeof(double));
	FF->v1presc = CAVITY_v1presc; FF->v2presc = CAVITY_v2presc; FF->ppresc = CAVITY_ppresc;
	FF->f1ext = CAVITY_f1ext; FF->f2ext = CAVITY_f2ext;
	FF->assembly = csr ? csr_assembly : ebe_assembly;
	FF->mv = csr ? csrmv : ebemvNDOF3;
	FF->precond = csr ? ILUp_precond : BlockDiagDOF3_precond;
	FF->precond_setup = csr ? ILUp_precond_setup : BlockDiagDOF3_precond_EBE_setup;
	*Po = P; *Mo = M; *FSo = FS; *FFo = FF;
}

/* nbuild consecutive Builds on the states u[b] (each [neq+1]); element
 * matrices Ae[b] [nel*81], residuals F[b] [neq+1] and the stabilisation state
 * (delta_old, normres_old [nel]) after the last build. */
int ref_ns_builds(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                  int neq, double Re, double velmax, int nbuild, const double *u, double *Ae, double *F,
                  double *delta_old, double *normres_old)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	int b;
	size_t n1 = (size_t)neq + 1;
	setup(0, nnodes, x, y, node_id, nel, vert, neq, Re, velmax, &P, &M, &FS, &FF);
	for (b = 0; b < nbuild; b++) {
		memcpy(FS->u, u + b * n1, sizeof(double) * n1);
		Build_K_F_MS(P, M, FS, FF);
		memcpy(Ae + (size_t)b * 81 * nel, M->Aaux, sizeof(double) * 81 * nel);
		memcpy(F + b * n1, FS->F, sizeof(double) * n1);
	}
	memcpy(delta_old, FS->delta_old, sizeof(double) * nel);
	memcpy(normres_old, FS->normres_old, sizeof(double) * nel);
	return 0;
}

/* Process.c:62-194 (damped Newton with backtracking on ||F||, F the
 * block-diagonally preconditioned residual, forcing term eta_newton case
 * `ecase`) for at most maxit Newton iterations.  Outputs: u after each
 * iteration uhist [maxit*(neq+1)], ||F|| after it normF [maxit], damping
 * factor used w [maxit], GMRES iterations gmres [maxit]; returns the number
 * of Newton iterations done. */
static int newton(int csr, int nnodes, const double *x, const double *y, const int *node_id, int nel,
                  const int *vert, int neq, double Re, double velmax, int kmax, int lmax, double eta0, int ecase,
                  double tolnl, int maxit, double *uhist, double *normF, double *wout, int *gmres)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	size_t n1 = (size_t)neq + 1;
	int i, it, iter, iterold, pricek, fd, cont, nit = 0;
	double norm_F, norm_Fold, epsilon, etaold, w_old;
	double w_min = 0.05, w_max = 1.00, c1 = 1.001, c2 = 1.1, c3 = 1.001, c4 = 0.9, c5 = 0.5, w = w_max;
	double *s, *Fold, *u, *F;
	setup(csr, nnodes, x, y, node_id, nel, vert, neq, Re, velmax, &P, &M, &FS, &FF);
	P->KrylovBasisVectorsQuantity = kmax; P->LinearMaxIter = lmax; P->SolverTolerance = eta0;
	P->SolverToleranceCase = ecase; P->SolverToleranceNonLin = tolnl;
	u = FS->u; F = FS->F;
	s = calloc(n1, sizeof(double)); Fold = calloc(n1, sizeof(double));
	Build_K_F_MS(P, M, FS, FF);
	it = 1;
	FF->precond_setup(P, M, FS, it, F);
	norm_F = sqrt(ddot(neq, F, F));
	epsilon = tolnl * norm_F;
	iter = 0;
	pricek = 1;
	dcopy(neq, F, Fold);
	while (norm_F > epsilon && it < 2000 && nit < maxit) {
		it++;
		iterold = iter;
		norm_Fold = sqrt(ddot(neq, Fold, Fold));
		gmres6(P, M, FS, FF, F, s);
		iter = P->iterations;
		pricek = iter - iterold + 1;
		fd = 1; cont = 1; w_old = 0.0;
		do {
			w_old = w;
			daxpy(neq, w, s, u);
			Build_K_F_MS(P, M, FS, FF);
			FF->precond_setup(P, M, FS, it, F);
			etaold = P->SolverTolerance;
			P->SolverTolerance = eta_newton(Fold, F, etaold, pricek, it, epsilon, eta0, P);
			norm_F = sqrt(ddot(neq, F, F));
			if (norm_F < norm_Fold || w < c1 * w_min) {
				if (norm_F < norm_Fold && fd == 1) {
					w_max = (1.0 < c3 * w_max) ? 1.0 : c3 * w_max;
					w = (w_max < c2 * w) ? w_max : c2 * w;
				}
				cont = 0;
			} else {
				w = (w_min > c5 * w) ? w_min : c5 * w;
				if (fd == 1) {
					w_max = (w_min > c4 * w_max) ? w_min : c4 * w_max;
					fd = 0;
				}
				daxpy(neq, -1. * w_old, s, u);
			}
		} while (cont == 1);
		dcopy(neq, F, Fold);
		memcpy(uhist + (size_t)nit * n1, u, sizeof(double) * n1);
		normF[nit] = norm_F;
		wout[nit] = w_old;
		gmres[nit] = pricek - 1;
		nit++;
	}
	free(s); free(Fold);
	(void)i;
	return nit;
}

int ref_ns_newton(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                  int neq, double Re, double velmax, int kmax, int lmax, double eta0, int ecase, double tolnl,
                  int maxit, double *uhist, double *normF, double *wout, int *gmres)
{
	return newton(0, nnodes, x, y, node_id, nel, vert, neq, Re, velmax, kmax, lmax, eta0, ecase, tolnl, maxit,
	              uhist, normF, wout, gmres);
}

/* The same Newton loop with CSR storage and ILU(0). */
int ref_ns_newton_csr(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                      int neq, double Re, double velmax, int kmax, int lmax, double eta0, int ecase, double tolnl,
                      int maxit, double *uhist, double *normF, double *wout, int *gmres)
{
	return newton(1, nnodes, x, y, node_id, nel, vert, neq, Re, velmax, kmax, lmax, eta0, ecase, tolnl, maxit,
	              uhist, normF, wout, gmres);
}

/* CSR set-up and nbuild consecutive builds with CSR assembly: pattern IA
 * [neq+1], JA [nnz_cap], the assembled values AA [nbuild][nnz_cap+1], the
 * residuals F [nbuild][neq+1], F after precond_setup (ILU(0), F := M^-1 F) of
 * the last build Fp [neq+1], and one ILU(0) application z = M^-1 p [neq+1].
 * Returns nnz (or -1 when nnz_cap is too small). */
int ref_ns_builds_csr(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                      int neq, double Re, double velmax, int nbuild, const double *u, int nnz_cap, int *IA, int *JA,
                      double *AA, double *F, double *Fp, const double *p, double *z)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	int b, nnz;
	size_t n1 = (size_t)neq + 1;
	setup(1, nnodes, x, y, node_id, nel, vert, neq, Re, velmax, &P, &M, &FS, &FF);
	nnz = P->nnzero;
	if (nnz > nnz_cap) return -1;
	memcpy(IA, M->IA, sizeof(int) * n1);
	memcpy(JA, M->JA, sizeof(int) * (size_t)nnz);
	for (b = 0; b < nbuild; b++) {
		memcpy(FS->u, u + b * n1, sizeof(double) * n1);
		Build_K_F_MS(P, M, FS, FF);
		memcpy(AA + (size_t)b * (nnz_cap + 1), M->AA, sizeof(double) * ((size_t)nnz + 1));
		memcpy(F + b * n1, FS->F, sizeof(double) * n1);
	}
	memcpy(Fp, FS->F, sizeof(double) * n1);
	FF->precond_setup(P, M, FS, 1, Fp);
	{
		double *pp = mycalloc("p", n1, sizeof(double));
		memcpy(pp, p, sizeof(double) * n1);
		FF->precond(P, M, FS, pp, z);
	}
	return nnz;
}
