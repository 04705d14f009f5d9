/*
 * shim_types_euler.h -- the layout of the 2D Euler driver's structs
 * (03_Euler_Equations/2D/01_CommonFiles/EulerEquations.h:17-170), restated so
 * that femgpu_shim_euler.c compiles where the reference tree is not present
 * (-DFEMGPU_SHIM_OWN_TYPES).  Field order, types and sizes must stay those
 * of that header; tests/test_shims.py checks them field by field wherever
 * the reference tree exists.  Structures the shim never dereferences
 * (ILU(p) and AMG data) are opaque pointers; the callbacks the shim never
 * calls keep their slots with generic pointer types of the same size.
 *
 * SHIM_T(name) names every type (default: the reference's own name).
 */
#ifndef FEMGPU_SHIM_TYPES_EULER_H
#define FEMGPU_SHIM_TYPES_EULER_H

#ifndef SHIM_T
#define SHIM_T(n) n
#endif

typedef struct {
	double x, y;
	int rhoType, v1Type, v2Type, eType;
	int id[4];
} SHIM_T(NodeType);

typedef struct { int Vertex[3]; int Type; } SHIM_T(ElementType);

typedef struct {
	char ProblemTitle[300];
	char Solver[200];
	char TimeIntegration[200];
	char MatrixVectorProductScheme[200];
	char StabilizationForm[200];
	char ShockCapture[200];
	char Preconditioner[1000];
	char Scaling[200];
	char Experiments[200];
	char StopMulticorrection[200];
	char reordering[200];
	char Dimensionless[200];
	char StopAtSteadyState[200];
	double SolverTolerance, NonLinearTolerance, TimeIntegrationTolerance, StabilizationTolerance;
	double Mach, Alpha, Alpha_Build, DeltaT, DeltaT_Build, FinalTime, CurrentTime;
	double invY[4];
	int KrylovBasisVectorsQuantity;
	int nnodes, nonpnodes, nel, neq, neqrho, nedge, nnzero;
	int iterations, LinearMaxIter, NonLinearMaxIter;
	int bandwidth_bef, bandwidth_aft;
} SHIM_T(ParametersType);

typedef struct {
	double **A;
	double *Aaux;
	double **BlockDiag;
	double *BlockDiagAux;
	double **invBlockDiag;
	double *invBlockDiagAux;
	double **invDe;
	double *invDeaux;
	double **LUe;
	double *LUeaux;
	int **Id;
	int *IdAux;
	int **Scheme_by_Element;
	int **order;
	double *AA, *Diag, *invDiag;
	int *JA, *IA;
	void *ILUp, *mat, *Ailu;          /* SparILU *, SparMAT *, MAT * (ilup.h) */
	int *Perm, *invPerm;
	void *amg_precond_data;           /* AMG_precond_data * (amg_precond.h) */
} SHIM_T(MatrixDataType);

typedef struct {
	double **M2, **R2, *invN2, *delta_old_NMV;
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
	double *F, *u, *du, *delta_old, *uB, *duB;
	SHIM_T(AuxBuildStructuresType) *AuxBuild;
} SHIM_T(FemStructsType);

typedef struct {
	double (*gamma)(double, double);
	double (*cv)(double, double);
	double (*rhopresc)(double, double);
	double (*v1presc)(double, double);
	double (*v2presc)(double, double);
	double (*epresc)(double, double);
	int (*InitialSolution)(SHIM_T(ParametersType) *, SHIM_T(NodeType) *, double *);
	void (*ShockCapture)(void);       /* slots the shim never calls */
	void (*Ax_Ay_calculations)(void);
	double (*BC_theta)(double, double);
	void (*BC_no_penetrability)(void);
	void (*BC_General_theta)(void);
	int (*StopCriteria)(SHIM_T(ParametersType) *, double, double, int);
	int (*StopTimeIntegration)(SHIM_T(ParametersType) *, double *, double *, double);
	void (*assembly)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, int,
	                 double (*)[12]);
	int (*mv)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *, double *);
	int (*precond)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *,
	               double *);
	int (*precondR)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *,
	                double *);
	int (*precond_setup)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, int,
	                     double *);
	int (*scaling)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *);
	int (*unscaling)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, double *);
} SHIM_T(FemFunctionsType);

typedef struct {
	int (*solver)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *,
	              SHIM_T(FemFunctionsType) *, double *, double *);
	int (*Build)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *,
	             SHIM_T(FemFunctionsType) *);
} SHIM_T(FemOtherFunctionsType);

#endif
