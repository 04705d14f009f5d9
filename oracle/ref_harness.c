/*
 * Test infrastructure only: a driver for the reference's own steady-transport
 * C sources (mod-comp-ufes/FEM_CODES, 01_SS_Transport_Equation/2D), compiled
 * from where they lie by oracle/Makefile into oracle/_ref/libfemref.so.
 *
 * It replaces the reference's file-reading Preprocess and its Process loop
 * with a function that takes the mesh as arrays, so golden vectors can be
 * produced without mesh files. Everything numeric is done by the reference's
 * own functions: Fill_LM, csr_Initialization (+ reordering/SYMRCM),
 * ede_Initialization, Build_K_F_SUPG, the assembly pointers, csrmv / ebemv /
 * edemv, ILUp_precond_setup / ILUp_precond, Diag_precond*, pgmres.
 *
 * Two documented fixes are applied here, not in the reference tree:
 *   - precond_setup is called after every Build, as the commented-out line
 *     01_SS_Transport_Equation/2D/01_CommonFiles/Process.c:53 intends (without
 *     it the ILU path dereferences an unset factor);
 *   - hflux is set to a function returning 0 for every problem (F_assembly.c:32
 *     calls it unconditionally; its contribution is multiplied by the integer
 *     constant 1/6 == 0 at F_assembly.c:31 anyway).
 * The config-1 problem ("SKEW": k=1e-4, beta=(cos30, sin30), f=0, gamma=0,
 * u=1 on x=0 for y>0.3, else 0 on x=0 or y=0) is defined here as a plug-in with
 * the reference's five-callback shape (e.g. CONVECTION/CONVECTION_Velocity.c).
 */
#include "SSTranspEquation.h"
#include <math.h>

int Fill_LM(int, int, int **, NodeType *, ElementType *);
int pgmres(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *);
int csrmv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int ebemv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int edemv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int NO_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int NO_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int ILUp_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int ILUp_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int Diag_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int Diag_precond_CSR_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int Diag_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int Diag_precond_EDE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);

/* --- problem plug-ins ---------------------------------------------------- */
double CONVECTION_Condutivity(void);
double CONVECTION_Font(double, double, double, double, double, double);
double CONVECTION_Reaction(void);
void CONVECTION_Velocity(double, double, double[]);
double CONVECTION_upresc(double, double);
double REACTION_Condutivity(void);
double REACTION_Font(double, double, double, double, double, double);
double REACTION_Reaction(void);
void REACTION_Velocity(double, double, double[]);
double REACTION_upresc(double, double);
double HEMKER_Condutivity(void);
double HEMKER_Font(double, double, double, double, double, double);
double HEMKER_Reaction(void);
void HEMKER_Velocity(double, double, double[]);
double HEMKER_upresc(double, double);
double VALIDACAO_Condutivity(void);
double VALIDACAO_Font(double, double, double, double, double, double);
double VALIDACAO_Reaction(void);
void VALIDACAO_Velocity(double, double, double[]);
double VALIDACAO_upresc(double, double);

#define SKEW_BX 0.86602540378443865
#define SKEW_BY 0.5
static double SKEW_Condutivity(void) { return 1e-4; }
static double SKEW_Font(double x, double y, double k, double g, double bx, double by) { return 0.0; }
static double SKEW_Reaction(void) { return 0.0; }
static void SKEW_Velocity(double x, double y, double b[]) { b[0] = SKEW_BX; b[1] = SKEW_BY; }
static double SKEW_upresc(double x, double y) { return (x == 0.0 && y > 0.3) ? 1.0 : 0.0; }
static double zero_hflux(double x, double y) { return 0.0; }

static void set_problem(int problem, FemFunctionsType *FF)
{
	FF->hflux = zero_hflux;
	switch (problem) {
	case 1:
		FF->Condutivity = CONVECTION_Condutivity; FF->Font = CONVECTION_Font;
		FF->Reaction = CONVECTION_Reaction; FF->Velocity = CONVECTION_Velocity;
		FF->upresc = CONVECTION_upresc; break;
	case 2:
		FF->Condutivity = REACTION_Condutivity; FF->Font = REACTION_Font;
		FF->Reaction = REACTION_Reaction; FF->Velocity = REACTION_Velocity;
		FF->upresc = REACTION_upresc; break;
	case 3:
		FF->Condutivity = HEMKER_Condutivity; FF->Font = HEMKER_Font;
		FF->Reaction = HEMKER_Reaction; FF->Velocity = HEMKER_Velocity;
		FF->upresc = HEMKER_upresc; break;
	case 4:
		FF->Condutivity = VALIDACAO_Condutivity; FF->Font = VALIDACAO_Font;
		FF->Reaction = VALIDACAO_Reaction; FF->Velocity = VALIDACAO_Velocity;
		FF->upresc = VALIDACAO_upresc; break;
	default:
		FF->Condutivity = SKEW_Condutivity; FF->Font = SKEW_Font;
		FF->Reaction = SKEW_Reaction; FF->Velocity = SKEW_Velocity;
		FF->upresc = SKEW_upresc; break;
	}
}

/* Element boundary classification, same rule as
 * 01_SS_Transport_Equation/2D/01_CommonFiles/Preprocess.c:108-152. */
static int classify_element(const NodeType *Node, const int v[3])
{
	int c1 = 0, c2 = 0, c3 = 0, c4 = 0, j;
	for (j = 0; j < 3; j++) {
		const NodeType *p = &Node[v[j]];
		if (p->x == 0.0) c1++;
		if (p->y == 0.0) c2++;
		if (p->x == 1.0) c3++;
		if (p->y == 1.0) c4++;
	}
	if (c1 == 2) return (c1 == c2) ? 5 : (c1 == c4) ? 8 : 1;
	if (c2 == 2) return (c2 == c3) ? 6 : 2;
	if (c3 == 2) return (c3 == c4) ? 7 : 3;
	if (c4 == 2) return 4;
	return -1;
}

/* Run the reference steady-transport path on an in-memory mesh.
 * Outputs (caller-allocated, upper-bounded sizes):
 *   info[0..3]   = neq, nnzero, nedge, bandwidth after reordering
 *   node_id      [nnodes]           Node[].id after csr_Initialization
 *   etype        [nel]              reclassified element Type
 *   beta,fsrc    [2*nel],[3*nel]    velocity at centroid / source at vertices
 *   upresc       [nnodes]           upresc(x,y) at every node
 *   IA,JA,sbe    CSR pattern and CSR_by_Element (CSR) or
 *                lm2 (2*nedge) and EDGE_by_Element (3*nel) + order (3*nel) (EDE)
 *   Afirst       matrix storage after the first Build (EBE 9*nel, EDE 4*(nedge+1), CSR nnz+1)
 *   Ffirst       F after the first Build, Fprec F after the first precond_setup
 *   Pin/Qmv      Qmv = ProductMatrixVector(Pin) after the first Build
 *   Zpc          Zpc = precond(Pin) after the first precond_setup
 *   uhist        [npicard*(neq+1)]  u after each Picard solve
 *   iters        [npicard]          GMRES iterations of each solve
 * Returns the number of Picard iterations run. */
int ref_transport_run(int nnodes, const double *x, const double *y, const int *ntype,
		int nel, const int *vert, int problem,
		const char *scheme, const char *reord, const char *precond,
		const char *shock, const char *hshock, const char *outflow,
		int kmax, int lmax, double tol, int npicard, double nonlin_tol,
		int *info, int *node_id, int *etype, double *beta, double *fsrc, double *upresc,
		int *IA_out, int *JA_out, int *sbe_out, int *order_out,
		double *Afirst, double *Ffirst, double *Fprec,
		double *Pin, double *Qmv, double *Zpc,
		double *uhist, int *iters)
{
	int I, J, neq;
	ParametersType *P = mycalloc("P", 1, sizeof(ParametersType));
	MatrixDataType *M = mycalloc("M", 1, sizeof(MatrixDataType));
	FemStructsType *FS = mycalloc("FS", 1, sizeof(FemStructsType));
	FemFunctionsType *FF = mycalloc("FF", 1, sizeof(FemFunctionsType));
	FemOtherFunctionsType *FOF = mycalloc("FOF", 1, sizeof(FemOtherFunctionsType));

	strcpy(P->ProblemTitle, "HARNESS");
	strcpy(P->Solver, "GMRES");
	strcpy(P->Preconditioner, precond);
	strcpy(P->Scaling, "NOT");
	strcpy(P->reordering, reord);
	strcpy(P->MatrixVectorProductScheme, scheme);
	strcpy(P->StabilizationForm, "SUPG");
	strcpy(P->ShockCapture, shock);
	strcpy(P->h_Shock, hshock);
	strcpy(P->OutputFlow, outflow);
	P->SolverTolerance = tol;
	P->NonLinearTolerance = nonlin_tol;
	P->SolverMaxIter = lmax;
	P->KrylovBasisVectorsQuantity = kmax;
	P->nnodes = nnodes;
	P->nel = nel;

	NodeType *Node = mycalloc("Node", nnodes, sizeof(NodeType));
	for (I = 0, neq = 0; I < nnodes; I++) {
		Node[I].x = x[I];
		Node[I].y = y[I];
		Node[I].Type = ntype[I];
		Node[I].id = (ntype[I] >= 1) ? neq++ : -1;
	}
	ElementType *Element = mycalloc("Element", nel, sizeof(ElementType));
	for (I = 0; I < nel; I++) {
		for (J = 0; J < 3; J++) Element[I].Vertex[J] = vert[3*I+J];
		Element[I].Type = classify_element(Node, Element[I].Vertex);
		etype[I] = Element[I].Type;
	}

	double *F = mycalloc("F", neq+1, sizeof(double));
	double *u = mycalloc("u", neq+1, sizeof(double));
	double *Diag = mycalloc("Diag", neq+1, sizeof(double));
	double *invDiag = mycalloc("invDiag", neq+1, sizeof(double));
	int **lm = mycalloc("lm", nel, sizeof(int*));
	int *lmaux = mycalloc("lmaux", nel*3, sizeof(int));
	for (I = 0; I < nel; I++) lm[I] = &lmaux[3*I];
	FS->u = u; FS->F = F;
	Fill_LM(neq, nel, lm, Node, Element);
	FS->lm = lm; FS->lmaux = lmaux;
	P->neq = neq;

	if (strcasecmp(scheme, "EBE") == 0) {
		double **K = mycalloc("K", nel, sizeof(double*));
		double *Kaux = mycalloc("Kaux", nel*9, sizeof(double));
		for (I = 0; I < nel; I++) K[I] = &Kaux[9*I];
		M->A = K; M->Aaux = Kaux;
		FF->assembly = ebe_assembly; FF->ProductMatrixVector = ebemv;
	} else if (strcasecmp(scheme, "EDE") == 0) {
		int **order = mycalloc("order", nel, sizeof(int*)), **EBE;
		for (I = 0; I < nel; I++) order[I] = mycalloc("order", 3, sizeof(int));
		ede_Initialization(P, order, &lm, &lmaux, &EBE);
		int nedge = P->nedge;
		double **K = mycalloc("K", nedge+1, sizeof(double*));
		double *Kaux = mycalloc("Kaux", (nedge+1)*4, sizeof(double));
		for (I = 0; I < nedge+1; I++) K[I] = &Kaux[4*I];
		FS->lm2 = lm; FS->lm2aux = lmaux;
		M->A = K; M->Aaux = Kaux; M->Scheme_by_Element = EBE; M->order = order;
		for (I = 0; I < nedge; I++) { JA_out[2*I] = lm[I][0]; JA_out[2*I+1] = lm[I][1]; }
		for (I = 0; I < nel; I++) for (J = 0; J < 3; J++) {
			sbe_out[3*I+J] = EBE[I][J];
			order_out[3*I+J] = order[I][J];
		}
		FF->assembly = ede_assembly; FF->ProductMatrixVector = edemv;
	} else {
		int *IA, *JA, *perm, *invperm, **CBE;
		csr_Initialization(P, Node, &JA, &IA, &perm, &invperm, &lm, &lmaux, &CBE);
		M->AA = mycalloc("AA", P->nnzero+1, sizeof(double));
		M->IA = IA; M->JA = JA; M->Scheme_by_Element = CBE; M->Perm = perm;
		for (I = 0; I <= neq; I++) IA_out[I] = IA[I];
		for (I = 0; I < P->nnzero; I++) JA_out[I] = JA[I];
		for (I = 0; I < nel; I++) for (J = 0; J < 9; J++) sbe_out[9*I+J] = CBE[I][J];
		FF->assembly = csr_assembly; FF->ProductMatrixVector = csrmv;
	}
	FS->Node = Node; FS->Element = Element;
	M->Diag = Diag; M->invDiag = invDiag;
	info[0] = neq; info[1] = P->nnzero; info[2] = P->nedge; info[3] = P->bandwidth_aft;
	for (I = 0; I < nnodes; I++) node_id[I] = Node[I].id;

	/* Function pointers, as set*.c would set them. */
	set_problem(problem, FF);
	if (strcasecmp(precond, "NOT") == 0) {
		FF->precond = NO_precond; FF->precond_setup = NO_precond_setup;
	} else if (strcasecmp(precond, "Diag") == 0) {
		FF->precond = Diag_precond;
		FF->precond_setup = (strcasecmp(scheme, "EBE") == 0) ? Diag_precond_EBE_setup :
			(strcasecmp(scheme, "EDE") == 0) ? Diag_precond_EDE_setup : Diag_precond_CSR_setup;
	} else {
		FF->precond = ILUp_precond; FF->precond_setup = ILUp_precond_setup;
	}
	FF->precondR = NO_precond;
	FOF->solver = pgmres;
	FOF->Build = Build_K_F_SUPG;
	FF->ShockCapture = (strcasecmp(shock, "YZBeta") == 0) ? YZBeta_ShockCapture : CAU_ShockCapture;
	if (strcasecmp(hshock, "sqrtArea") == 0) FF->h_shock = h_shock_sqrtArea;
	else if (strcasecmp(hshock, "Option1") == 0) FF->h_shock = h_shock_Option1;
	else if (strcasecmp(hshock, "Option2") == 0) FF->h_shock = h_shock_Option2;
	else FF->h_shock = h_shock_2sqrtArea;

	/* Coefficients exactly as Build_K_F_SUPG.c:61-84 evaluates them. */
	{
		double third = 1.0/3.0, k = FF->Condutivity(), g = FF->Reaction(), b[2];
		for (I = 0; I < nel; I++) {
			int *v = Element[I].Vertex;
			double XB = third*(Node[v[0]].x + Node[v[1]].x + Node[v[2]].x);
			double YB = third*(Node[v[0]].y + Node[v[1]].y + Node[v[2]].y);
			FF->Velocity(XB, YB, b);
			beta[2*I] = b[0]; beta[2*I+1] = b[1];
			for (J = 0; J < 3; J++)
				fsrc[3*I+J] = FF->Font(Node[v[J]].x, Node[v[J]].y, k, g, b[0], b[1]);
		}
		for (I = 0; I < nnodes; I++) upresc[I] = FF->upresc(Node[I].x, Node[I].y);
	}

	/* Process loop: Process.c:276-335 with the precond_setup call restored. */
	double *CbOld = mycalloc("CbOld", nel, sizeof(double));
	FS->CbOld = CbOld;
	dzero(neq+1, u);
	double *uold = mycalloc("uold", neq+1, sizeof(double));
	double error = 100.0;
	int it = 0;
	while (it < npicard && (nonlin_tol <= 0 || error > nonlin_tol)) {
		it++;
		dcopy(neq, u, uold);
		FOF->Build(P, M, FS, FF);
		if (it == 1) {
			for (I = 0; I <= neq; I++) Ffirst[I] = F[I];
			if (strcasecmp(scheme, "EBE") == 0) memcpy(Afirst, M->Aaux, sizeof(double)*9*nel);
			else if (strcasecmp(scheme, "EDE") == 0) memcpy(Afirst, M->Aaux, sizeof(double)*4*(P->nedge+1));
			else memcpy(Afirst, M->AA, sizeof(double)*(P->nnzero+1));
			double *tmp = mycalloc("tmp", neq+1, sizeof(double));
			memcpy(tmp, Pin, sizeof(double)*(neq+1));
			FF->ProductMatrixVector(P, M, FS, tmp, Qmv);
			free(tmp);
		}
		FF->precond_setup(P, M, FS, it, F);
		if (it == 1) {
			for (I = 0; I <= neq; I++) Fprec[I] = F[I];
			double *tmp = mycalloc("tmp", neq+1, sizeof(double));
			memcpy(tmp, Pin, sizeof(double)*(neq+1));
			memcpy(Zpc, Pin, sizeof(double)*(neq+1));
			FF->precond(P, M, FS, tmp, Zpc);
			free(tmp);
		}
		int before = P->SolverIterations;
		FOF->solver(P, M, FS, FF);
		iters[it-1] = P->SolverIterations - before;
		for (I = 0; I <= neq; I++) uhist[(size_t)(it-1)*(neq+1) + I] = u[I];
		error = 0.0;
		for (I = 0; I < neq; I++) {
			double d = fabs(u[I] - uold[I]);
			if (I == 0 || d > error) error = d;
		}
	}
	return it;
}

/* Paraview_Output.c on a given nodal numbering (node_id, -1 prescribed) and
 * solution u [neq+1] of a problem's plug-ins: the file goes where the
 * reference writes it, ../03_output/<names>.vtu relative to the working
 * directory. */
int Paraview_Output(ParametersType *, FemStructsType *, FemFunctionsType *);
int ref_transport_vtu(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                      int problem, int neq, const double *u)
{
	int I, J;
	ParametersType *P = mycalloc("P", 1, sizeof(ParametersType));
	FemStructsType *FS = mycalloc("FS", 1, sizeof(FemStructsType));
	FemFunctionsType *FF = mycalloc("FF", 1, sizeof(FemFunctionsType));
	NodeType *Node = mycalloc("Node", nnodes, sizeof(NodeType));
	ElementType *El = mycalloc("El", nel, sizeof(ElementType));
	strcpy(P->Experiments, "HARNESS"); strcpy(P->ProblemTitle, "VTU"); strcpy(P->StabilizationForm, "SUPG");
	strcpy(P->ShockCapture, "CAU"); strcpy(P->h_Shock, "2sqrtArea"); strcpy(P->MatrixVectorProductScheme, "CSR");
	strcpy(P->Preconditioner, "ILU0");
	P->nnodes = nnodes; P->nel = nel; P->neq = neq;
	for (I = 0; I < nnodes; I++) { Node[I].x = x[I]; Node[I].y = y[I]; Node[I].id = node_id[I]; }
	for (I = 0; I < nel; I++) for (J = 0; J < 3; J++) El[I].Vertex[J] = vert[3 * I + J];
	FS->Node = Node; FS->Element = El;
	FS->u = mycalloc("u", neq + 1, sizeof(double));
	memcpy(FS->u, u, sizeof(double) * (neq + 1));
	set_problem(problem, FF);
	return Paraview_Output(P, FS, FF);
}

/* The reference's own Preprocess (Preprocess.c:4-260) on a deck file, run in
 * the working directory (it opens ../02_mesh/<title>_<nnodes>_<nel>.dat):
 * the parameters it read (ints: nnodes, nel, neq, SolverMaxIter,
 * KrylovBasisVectorsQuantity, nnzero; doubles: SolverTolerance,
 * NonLinearTolerance; strings: the deck's 11 strings, 64 bytes apart), the
 * nodes (x, y, Type, id) and elements (vertices, Type) it built. */
int Preprocess(int, char **, ParametersType **, MatrixDataType **, FemStructsType **, FemFunctionsType **,
               FemOtherFunctionsType **);
int ref_transport_preprocess(const char *deck, int *iv, double *dv, char *sv, double *x, double *y, int *type,
                             int *id, int *vert, int *etype, int cap_nodes, int cap_el)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF; FemOtherFunctionsType *FOF;
	char *argv[2] = { "harness", (char *)deck };
	int I;
	const char *str[11];
	Preprocess(2, argv, &P, &M, &FS, &FF, &FOF);
	iv[0] = P->nnodes; iv[1] = P->nel; iv[2] = P->neq; iv[3] = P->SolverMaxIter;
	iv[4] = P->KrylovBasisVectorsQuantity; iv[5] = P->nnzero;
	dv[0] = P->SolverTolerance; dv[1] = P->NonLinearTolerance;
	str[0] = P->Experiments; str[1] = P->ProblemTitle; str[2] = P->Solver; str[3] = P->Preconditioner;
	str[4] = P->Scaling; str[5] = P->reordering; str[6] = P->MatrixVectorProductScheme;
	str[7] = P->StabilizationForm; str[8] = P->ShockCapture; str[9] = P->h_Shock; str[10] = P->OutputFlow;
	for (I = 0; I < 11; I++) strncpy(sv + 64 * I, str[I], 63);
	if (P->nnodes > cap_nodes || P->nel > cap_el) return -1;
	for (I = 0; I < P->nnodes; I++) {
		x[I] = FS->Node[I].x; y[I] = FS->Node[I].y; type[I] = FS->Node[I].Type; id[I] = FS->Node[I].id;
	}
	for (I = 0; I < P->nel; I++) {
		vert[3 * I] = FS->Element[I].Vertex[0]; vert[3 * I + 1] = FS->Element[I].Vertex[1];
		vert[3 * I + 2] = FS->Element[I].Vertex[2]; etype[I] = FS->Element[I].Type;
	}
	return 0;
}
