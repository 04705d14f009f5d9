/*
 * shim_types_ns.h -- the layout of the steady Navier-Stokes driver's structs
 * (04_SS_NavierStokes_Equations/2D/01_CommonFiles/SSNavierStokesEquations.h:
 * 17-156), restated so that femgpu_shim_ns.c compiles where the reference
 * tree is not present (-DFEMGPU_SHIM_OWN_TYPES).  Field order, types and
 * sizes must stay those of that header; tests/test_shims.py checks them field
 * by field wherever the reference tree exists.  ILU(p) and AMG data are
 * opaque pointers.
 *
 * SHIM_T(name) names every type (default: the reference's own name).
 */
#ifndef FEMGPU_SHIM_TYPES_NS_H
#define FEMGPU_SHIM_TYPES_NS_H

#ifndef SHIM_T
#define SHIM_T(n) n
#endif

typedef struct {
	double x, y;
	int v1Type, v2Type, pType;
	int id[3];
} SHIM_T(NodeType);

typedef struct { int Vertex[3]; int Type; } SHIM_T(ElementType);

typedef struct {
	char ProblemTitle[250];
	char Solver[200];
	char TimeIntegration[200];
	char MatrixVectorProductScheme[200];
	char StabilizationForm[200];
	char ShockCapture[200];
	char Preconditioner[200];
	char Experiments[200];
	char StopMulticorrection[200];
	double ReynoldsNumber, VelMax;
	char reordering[200];
	double SolverTolerance;
	int SolverToleranceCase;
	double SolverToleranceNonLin, CorrectionTolerance, TimeIntegrationTolerance, CoefficientTolerance;
	double Alpha, DeltaT, FinalT;
	double invY[4];
	double normu, normv, normp;
	int KrylovBasisVectorsQuantity;
	int nnodes, nel, neq, nedge, nnzero;
	int iterations, gmres, NLiterations, LinearMaxIter, NumberCorrection;
	int bandwidth_bef, bandwidth_aft;
} SHIM_T(ParametersType);

typedef struct {
	double **A;
	double *Aaux, *AA;
	int *JA, *IA;
	double *D, *Diag, *invDiag;
	double **BlockDiag;
	double *BlockDiagAux;
	double **invBlockDiag;
	double *invBlockDiagAux;
	int **Id;
	int *IdAux;
	int **Scheme_by_Element;
	int **order;
	void *ILUp, *mat, *Ailu;          /* SparILU *, SparMAT *, MAT * (ilup.h) */
	int *Perm, *invPerm;
	void *amg_precond_data;           /* AMG_precond_data * (amg_precond.h) */
} SHIM_T(MatrixDataType);

typedef struct {
	double **M2, **R1, **R2, *invN2;
	double tolerance;
} SHIM_T(AuxBuildStructuresType);

typedef struct {
	int **lm;
	int *lmaux;
	int **lm2;
	int *lm2aux;
	int *eqrho;
	SHIM_T(NodeType) *Node;
	SHIM_T(ElementType) *Element;
	double *F, *u, *du, *delta_old, *normres_old, *uB, *duB;
	SHIM_T(AuxBuildStructuresType) *AuxBuild;
} SHIM_T(FemStructsType);

typedef struct {
	double (*v1presc)(double, double);
	double (*v2presc)(double, double);
	double (*ppresc)(double, double);
	double (*f1ext)(double, double);
	double (*f2ext)(double, double);
	void (*assembly)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, int,
	                 double (*)[9]);
	int (*mv)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *, double *);
	int (*precond)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *,
	               double *);
	int (*precondR)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *,
	                double *);
	int (*precond_setup)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, int,
	                     double *);
} SHIM_T(FemFunctionsType);

typedef struct {
	int (*solver)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *,
	              SHIM_T(FemFunctionsType) *, double *, double *);
	int (*Build)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *,
	             SHIM_T(FemFunctionsType) *);
} SHIM_T(FemOtherFunctionsType);

#endif
