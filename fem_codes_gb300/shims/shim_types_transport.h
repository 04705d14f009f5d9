/*
 * shim_types_transport.h -- the layout of the steady-transport driver's
 * structs (01_SS_Transport_Equation/2D/01_CommonFiles/SSTranspEquation.h:17-121),
 * restated so that femgpu_shim_transport.c compiles where the reference tree
 * is not present (build with -DFEMGPU_SHIM_OWN_TYPES).  A driver built from
 * the reference tree includes SSTranspEquation.h instead; the field order,
 * types and sizes here must stay those of that header, which
 * tests/test_shims.py checks field by field (offsetof / sizeof) wherever the
 * reference tree exists.  Types the shim never dereferences (the ILU(p) data
 * of ilup.h) are kept as opaque pointers.
 *
 * SHIM_T(name) names every type (default: the reference's own name), so a
 * checker can include this header beside the reference's with its own prefix.
 */
#ifndef FEMGPU_SHIM_TYPES_TRANSPORT_H
#define FEMGPU_SHIM_TYPES_TRANSPORT_H

#ifndef SHIM_T
#define SHIM_T(n) n
#endif

typedef struct { double x, y; int Type; int id; } SHIM_T(NodeType);
typedef struct { int Vertex[3]; int Type; } SHIM_T(ElementType);

typedef struct {
	char Experiments[50];
	char ProblemTitle[50];
	char Solver[10];
	char Preconditioner[50];
	char Scaling[50];
	char reordering[50];
	char MatrixVectorProductScheme[10];
	char StabilizationForm[50];
	char ShockCapture[50];
	char h_Shock[50];
	char OutputFlow[10];
	double SolverTolerance, NonLinearTolerance;
	int KrylovBasisVectorsQuantity;
	int nnodes, nel, neq, nedge, nnzero;
	int SolverIterations, SolverMaxIter;
	int bandwidth_bef, bandwidth_aft;
} SHIM_T(ParametersType);

typedef struct {
	double **A;
	double *Aaux, *AA, *Diag, *invDiag;
	double **invDe;
	double *invDeaux;
	double **LUe;
	double *LUeaux;
	int **Scheme_by_Element;
	int **order;
	int *JA, *IA;
	void *ILUp, *mat, *Ailu;          /* SparILU *, SparMAT *, MAT * (ilup.h) */
	int *Perm;
} SHIM_T(MatrixDataType);

typedef struct {
	int **lm;
	int *lmaux;
	int **lm2;
	int *lm2aux;
	SHIM_T(NodeType) *Node;
	SHIM_T(ElementType) *Element;
	double *u, *F, *CbOld;
} SHIM_T(FemStructsType);

typedef struct {
	double (*Condutivity)(void);
	double (*Font)(double, double, double, double, double, double);
	double (*Reaction)(void);
	void (*Velocity)(double, double, double[]);
	double (*upresc)(double, double);
	double (*hflux)(double, double);
	double (*h_shock)(SHIM_T(ParametersType) *, SHIM_T(ElementType) *, int, double, double, double, double,
	                  double, double, double, double, double, double, double, double);
	double (*ShockCapture)(double, double, double, double, double, double, double, double, double, double,
	                       double, double, double, double, double, double, double, double, double *, int);
	void (*assembly)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *, int,
	                 double (*)[3]);
	int (*ProductMatrixVector)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *,
	                           double *, double *);
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
	              SHIM_T(FemFunctionsType) *);
	int (*Build)(SHIM_T(ParametersType) *, SHIM_T(MatrixDataType) *, SHIM_T(FemStructsType) *,
	             SHIM_T(FemFunctionsType) *);
} SHIM_T(FemOtherFunctionsType);

#endif
