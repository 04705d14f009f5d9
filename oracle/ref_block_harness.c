/*
 * Test infrastructure only: drives the reference's block (multi-dof) EBE
 * operators, compiled from the reference's own sources by oracle/Makefile:
 *   -DEulerEquations2D:          ebemvNDOF4, ebe2mvNDOF4, BlockDiag_precond_EBE_setup,
 *                                BlockDiag_precond, BlockDiag2_precond, NOBlockDiag2_precond
 *   -DSSNavierStokesEquations2D: ebemvNDOF3, BlockDiagDOF3_precond_EBE_setup,
 *                                BlockDiagDOF3_precond
 * with the mesh, the node numbering and the element matrices given as arrays.
 */
#ifdef EulerEquations2D
#include "EulerEquations.h"
#define BLK_NDOF 4
int ebemvNDOF4(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int ebe2mvNDOF4(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int BlockDiag_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int BlockDiag_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
#define MV ebemvNDOF4
#define BD_SETUP BlockDiag_precond_EBE_setup
#define BD_APPLY BlockDiag_precond
#else
#include "SSNavierStokesEquations.h"
#define BLK_NDOF 3
int ebemvNDOF3(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int BlockDiagDOF3_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int BlockDiagDOF3_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
#define MV ebemvNDOF3
#define BD_SETUP BlockDiagDOF3_precond_EBE_setup
#define BD_APPLY BlockDiagDOF3_precond
#endif

void *mycalloc(char *, int, int);

/* Q = A P; Q2 = ebe2mvNDOF4 with BlockDiag2 (Euler only), Q2no = with
 * NOBlockDiag2; F in/out: F := invBD F; BD, invBD: the assembled blocks;
 * Z = invBD p. All vectors length neq+1. */
int ref_block_run(int nnodes, int nel, const int *vert, const int *node_id, int neq, const double *A,
                  const double *P, double *Q, double *Q2, double *Q2no, double *F, double *BD,
                  double *invBD, const double *p, double *Z)
{
	int m = 3 * BLK_NDOF, m2 = m * m, e, i, k;
	ParametersType *Pa = mycalloc("P", 1, sizeof(ParametersType));
	MatrixDataType *M = mycalloc("M", 1, sizeof(MatrixDataType));
	FemStructsType *FS = mycalloc("FS", 1, sizeof(FemStructsType));
	NodeType *Node = mycalloc("Node", nnodes, sizeof(NodeType));
	ElementType *El = mycalloc("El", nel, sizeof(ElementType));
	int **lm = mycalloc("lm", nel, sizeof(int *));
	double **Ap = mycalloc("A", nel, sizeof(double *));
	double *Aaux = mycalloc("Aaux", nel * m2, sizeof(double));
	double *tmp = mycalloc("tmp", neq + 1, sizeof(double));
	Pa->neq = neq; Pa->nel = nel; Pa->nnodes = nnodes;
	strcpy(Pa->Preconditioner, "BlockDiag");
	for (i = 0; i < nnodes; i++) for (k = 0; k < BLK_NDOF; k++) Node[i].id[k] = node_id[BLK_NDOF * i + k];
	for (e = 0; e < nel; e++) {
		for (i = 0; i < 3; i++) El[e].Vertex[i] = vert[3 * e + i];
		lm[e] = mycalloc("lm", m, sizeof(int));
	}
	Fill_LM(neq, nel, lm, Node, El);
	for (e = 0; e < nel; e++) { Ap[e] = Aaux + (size_t)e * m2; memcpy(Ap[e], A + (size_t)e * m2, sizeof(double) * m2); }
	M->A = Ap; M->Aaux = Aaux;
	FS->lm = lm; FS->Node = Node; FS->Element = El;

	memcpy(tmp, P, sizeof(double) * (neq + 1));
	MV(Pa, M, FS, tmp, Q);
	BD_SETUP(Pa, M, FS, 1, F);
	for (i = 0; i < nnodes; i++) for (k = 0; k < BLK_NDOF * BLK_NDOF; k++) {
		BD[i * BLK_NDOF * BLK_NDOF + k] = M->BlockDiag[i][k];
		invBD[i * BLK_NDOF * BLK_NDOF + k] = M->invBlockDiag[i][k];
	}
	memcpy(tmp, p, sizeof(double) * (neq + 1));
	memcpy(Z, p, sizeof(double) * (neq + 1));
	BD_APPLY(Pa, M, FS, tmp, Z);
#ifdef EulerEquations2D
	memcpy(tmp, P, sizeof(double) * (neq + 1));
	ebe2mvNDOF4(Pa, M, FS, tmp, Q2);
	strcpy(Pa->Preconditioner, "NOT");
	memcpy(tmp, P, sizeof(double) * (neq + 1));
	ebe2mvNDOF4(Pa, M, FS, tmp, Q2no);
#else
	(void)Q2; (void)Q2no;
#endif
	return 0;
}
