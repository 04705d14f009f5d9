/*
 * Test infrastructure only: drives the reference's transient scalar transport
 * (mod-comp-ufes/FEM_CODES, 02_Transport_Equation/2D) from in-memory arrays,
 * compiled from the reference's own sources by oracle/Makefile into
 * oracle/_ref/libfemref_transient.so with -DTranspEquation2D.
 *
 * Everything numeric is the reference's: Fill_LM, csr_Initialization (with
 * reordering/SYMRCM), ede_Initialization, Build_M_K_R_SUPG / Build_M_K_R_DD
 * with eval_U_dU and the CAU / CAU_DD / YZBeta shock capturing and the
 * h_shock options, the assembly pointers, csrmv / ebemv / edemv, the NOT /
 * Diag / ILU(0) preconditioners, the CONE / CONE2 / CARTOLA / PUDIM
 * plug-ins, and the time loops themselves: 00_CommonFiles/Time_Integration/
 * Predictor_Old.c, Predictor_Old_BDF.c, Predictor_Old_TRBDF2.c and
 * Predictor_New.c, Predictor_New_BDF.c and Predictor_New_TRBDF2.c (with
 * Build_M_F_DD.c, calculate_DaB.c, uB_InitialSolution.c)
 * with the stop criteria of Criteria.c.
 *
 * One documented adapter: the driver's solver pointer takes (B, X)
 * (TranspEquation.h: solver(P, M, FS, FF, B, X)), while the shipped pgmres.c
 * has only the steady-transport 4-argument form, so 02 does not link as
 * shipped; the 6-argument GMRES of ref_gmres6.h (pgmres.c's algorithm and
 * arithmetic with B and X as arguments) stands in.  Scaling is "NOT"
 * (setScaling.c: NO_scaling / NO_unscaling, which do nothing), restated here
 * as no-op functions because scaling.c does not compile against this
 * driver's header.
 */
#include "TranspEquation.h"
#include "time_integration.h"

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

#define PLUGIN(P) \
	double P##_Condutivity(void); double P##_Font(double, double, double, double, double, double); \
	double P##_Reaction(void); void P##_Velocity(double, double, double[]); double P##_upresc(double, double); \
	int P##_InitialSolution(ParametersType *, NodeType *, double *);
PLUGIN(CONE)
PLUGIN(CONE2)
PLUGIN(CARTOLA)
PLUGIN(PUDIM)

#include "ref_gmres6.h"

static void set_problem(int problem, FemFunctionsType *FF)
{
#define SETP(P) do { FF->Condutivity = P##_Condutivity; FF->Font = P##_Font; FF->Reaction = P##_Reaction; \
		FF->Velocity = P##_Velocity; FF->upresc = P##_upresc; FF->InitialSolution = P##_InitialSolution; } while (0)
	switch (problem) {
	case 1: SETP(CONE2); break;
	case 2: SETP(CARTOLA); break;
	case 3: SETP(PUDIM); break;
	default: SETP(CONE); break;
	}
#undef SETP
}

static int noscale(ParametersType *P, MatrixDataType *M, FemStructsType *FS) { return 0; }
static int nounscale(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *x) { return 0; }

/* Records of the time loop.  Every multicorrection loop (one per step, two
 * per TRBDF2 step -- a stage) ends when the reference's StopCriteria says
 * so: the wrapper stores the stage's u and correction count then.  The time
 * criterion is asked once per step of the time loop (not after BDF's first,
 * implicit step): the wrapper stores t then and stops at the step cap. */
static double *g_uhist, *g_thist;
static int *g_iters, *g_ncorr, g_stage, g_tcheck, g_maxsteps, g_corr, g_steady, g_norm, g_neq, g_cap;
static double *g_u;

static int record_stage(ParametersType *P, double norm_a, double norm_Da, int i)
{
	int stop = g_norm ? StopByNorm(P, norm_a, norm_Da, i) : StopByIterations(P, norm_a, norm_Da, i);
	if (stop) {
		if (g_stage < g_cap) {
			memcpy(g_uhist + (size_t)g_stage * (g_neq + 1), g_u, sizeof(double) * (g_neq + 1));
			g_ncorr[g_stage] = g_corr;
		}
		g_stage++;
		g_corr = 0;
	}
	return stop;
}

static int record_step(ParametersType *P, double *u, double *u_old, double t)
{
	int stop = g_steady ? StopBySteadyState(P, u, u_old, t) : StopByTime(P, u, u_old, t);
	g_thist[g_tcheck++] = t;
	return stop || g_tcheck >= g_maxsteps;
}

static int solver_rec(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF, double *B,
                      double *X)
{
	int before = P->iterations, rc = gmres6(P, M, FS, FF, B, X);
	if (g_stage < g_cap) g_iters[(size_t)g_stage * 64 + (g_corr < 63 ? g_corr : 63)] = P->iterations - before;
	g_corr++;
	return rc;
}

/* Transient transport on an in-memory mesh.
 *   problem: 0 CONE, 1 CONE2, 2 CARTOLA, 3 PUDIM; ntype: Node Type (1 free, 0 prescribed)
 *   stab "SUPG" | "DD"; shock "CAU" | "CAUDD" | "YZBeta"; hshock "2sqrtArea" | "Option1" | "Option2"
 *   stopmc "ITERATION" | "NORM"; steady "YES" | "NOT"
 *   tint "Predictor1" | "Predictor1_BDF" | "Predictor1_TRBDF2" | "Predictor2" | "Predictor2_BDF" |
 *   "Predictor2_TRBDF2" (setStabilizationForm.c:10-62; the Predictor2 forms run Predictor_New* with
 *   Build_M_F_DD)
 * Outputs:
 *   info [5] = neq, nnzero, nedge, bandwidth after reordering, (out) time checks; node_id [nnodes]
 *   beta [2*nel], fsrc [3*nel], upresc [nnodes]: the plug-ins as Build evaluates them
 *   u0 [neq+1]: the plug-in's initial solution
 *   IA/JA/sbe (CSR) or lm2 (JA, 2*nedge) / EDGE_by_Element (sbe, 3*nel) / order (3*nel) (EDE)
 *   two consecutive Builds on (ub, dub) (the DD builds keep per-element state; Build_M_F_DD also
 *   reads the element bubbles ubB, dubB [nel]):
 *   A1, R1 and A2, R2 (storage values EBE 9*nel / EDE 4*(nedge+1) / CSR nnz+1; R [neq+1])
 *   then the time loop from u0, stopped after maxsteps time checks: per stage (multicorrection
 *   loop) uhist [cap*(neq+1)], ncorr [cap], iters [cap*64] (GMRES iterations of each correction),
 *   cap = 2*maxsteps + 2; per time check thist [maxsteps].
 * Returns the number of stages recorded; info[4] = the number of time checks. */
int ref_transient_run(int nnodes, const double *x, const double *y, const int *ntype, int nel, const int *vert,
                      int problem, const char *scheme, const char *reord, const char *precond, const char *stab,
                      const char *shock, const char *hshock, const char *stopmc, const char *steady,
                      const char *tint, double alpha,
                      double dt, double final_time, double nonlin_tol, int max_corr, double time_tol, double stab_tol,
                      int kmax, int lmax, double tol, int *info, int *node_id, double *beta, double *fsrc,
                      double *upresc, double *u0, int *IA_out, int *JA_out, int *sbe_out, int *order_out,
                      const double *ub, const double *dub, const double *ubB, const double *dubB, double *A1,
                      double *R1, double *A2, double *R2, int maxsteps, double *uhist, double *thist, int *ncorr,
                      int *iters)
{
	int I, J, neq;
	ParametersType *P = mycalloc("P", 1, sizeof(ParametersType));
	MatrixDataType *M = mycalloc("M", 1, sizeof(MatrixDataType));
	FemStructsType *FS = mycalloc("FS", 1, sizeof(FemStructsType));
	FemFunctionsType *FF = mycalloc("FF", 1, sizeof(FemFunctionsType));
	FemOtherFunctionsType *FOF = mycalloc("FOF", 1, sizeof(FemOtherFunctionsType));
	int ebe = strcasecmp(scheme, "EBE") == 0, ede = strcasecmp(scheme, "EDE") == 0;
	size_t nA;

	strcpy(P->ProblemTitle, "HARNESS");
	strcpy(P->Solver, "GMRES");
	strcpy(P->Preconditioner, precond);
	strcpy(P->Scaling, "NOT");
	strcpy(P->reordering, reord);
	strcpy(P->MatrixVectorProductScheme, scheme);
	strcpy(P->StabilizationForm, stab);
	strcpy(P->ShockCapture, shock);
	strcpy(P->h_Shock, hshock);
	strcpy(P->TimeIntegration, tint);
	strcpy(P->StopMulticorrection, stopmc);
	strcpy(P->StopAtSteadyState, steady);
	P->SolverTolerance = tol;
	P->NonLinearTolerance = nonlin_tol;
	P->TimeIntegrationTolerance = time_tol;
	P->StabilizationTolerance = stab_tol;
	P->NonLinearMaxIter = max_corr;
	P->LinearMaxIter = lmax;
	P->KrylovBasisVectorsQuantity = kmax;
	P->Alpha = alpha;
	P->DeltaT = dt;
	P->FinalTime = final_time;
	P->nnodes = nnodes;
	P->nel = nel;

	/* Preprocess.c:77-98 */
	NodeType *Node = mycalloc("Node", nnodes, sizeof(NodeType));
	for (I = 0, neq = 0; I < nnodes; I++) {
		Node[I].x = x[I];
		Node[I].y = y[I];
		Node[I].Type = ntype[I];
		Node[I].id = (ntype[I] == 1) ? neq++ : -1;
	}
	ElementType *Element = mycalloc("Element", nel, sizeof(ElementType));
	for (I = 0; I < nel; I++)
		for (J = 0; J < 3; J++) Element[I].Vertex[J] = vert[3 * I + J];

	/* Preprocess.c:107-196 */
	double *F = mycalloc("F", neq + 1, sizeof(double));
	double *u = mycalloc("u", neq + 1, sizeof(double));
	double *du = mycalloc("du", neq + 1, sizeof(double));
	double *Diag = mycalloc("Diag", neq + 1, sizeof(double));
	double *invDiag = mycalloc("invDiag", neq + 1, sizeof(double));
	int **lm = mycalloc("lm", nel, sizeof(int *));
	int *lmaux = mycalloc("lmaux", nel * 3, sizeof(int));
	for (I = 0; I < nel; I++) lm[I] = &lmaux[3 * I];
	FS->u = u; FS->F = F; FS->du = du;
	Fill_LM(neq, nel, lm, Node, Element);
	FS->lm = lm; FS->lmaux = lmaux;
	P->neq = neq;
	if (ebe) {
		double **K = mycalloc("K", nel, sizeof(double *));
		double *Kaux = mycalloc("Kaux", nel * 9, sizeof(double));
		for (I = 0; I < nel; I++) K[I] = &Kaux[9 * I];
		M->A = K; M->Aaux = Kaux;
		FF->assembly = ebe_assembly; FF->mv = ebemv;
		nA = (size_t)9 * nel;
	} else if (ede) {
		int **order = mycalloc("order", nel, sizeof(int *)), **EBE;
		for (I = 0; I < nel; I++) order[I] = mycalloc("order", 3, sizeof(int));
		ede_Initialization(P, order, &lm, &lmaux, &EBE);
		double **K = mycalloc("K", P->nedge + 1, sizeof(double *));
		double *Kaux = mycalloc("Kaux", (P->nedge + 1) * 4, sizeof(double));
		for (I = 0; I < P->nedge + 1; I++) K[I] = &Kaux[4 * I];
		FS->lm2 = lm; FS->lm2aux = lmaux;
		M->A = K; M->Aaux = Kaux; M->Scheme_by_Element = EBE; M->order = order;
		for (I = 0; I < P->nedge; I++) { JA_out[2 * I] = lm[I][0]; JA_out[2 * I + 1] = lm[I][1]; }
		for (I = 0; I < nel; I++)
			for (J = 0; J < 3; J++) { sbe_out[3 * I + J] = EBE[I][J]; order_out[3 * I + J] = order[I][J]; }
		FF->assembly = ede_assembly; FF->mv = edemv;
		nA = (size_t)4 * (P->nedge + 1);
	} else {
		int *IA, *JA, *perm, *invperm, **CBE;
		csr_Initialization(P, Node, &JA, &IA, &perm, &invperm, &lm, &lmaux, &CBE);
		FS->lm = lm; FS->lmaux = lmaux;
		M->AA = mycalloc("AA", P->nnzero + 1, sizeof(double));
		M->IA = IA; M->JA = JA; M->Scheme_by_Element = CBE; M->Perm = perm;
		for (I = 0; I <= neq; I++) IA_out[I] = IA[I];
		for (I = 0; I < P->nnzero; I++) JA_out[I] = JA[I];
		for (I = 0; I < nel; I++) for (J = 0; J < 9; J++) sbe_out[9 * I + J] = CBE[I][J];
		FF->assembly = csr_assembly; FF->mv = csrmv;
		nA = (size_t)P->nnzero + 1;
	}
	FS->Node = Node; FS->Element = Element;
	M->Diag = Diag; M->invDiag = invDiag;
	info[0] = neq; info[1] = P->nnzero; info[2] = P->nedge; info[3] = P->bandwidth_aft;
	for (I = 0; I < nnodes; I++) node_id[I] = Node[I].id;

	/* Process.c: setProblem, setPreconditioner, setScaling, setStabilizationForm */
	set_problem(problem, FF);
	if (strcasecmp(precond, "NOT") == 0) {
		FF->precond = NO_precond; FF->precond_setup = NO_precond_setup;
	} else if (strcasecmp(precond, "Diag") == 0) {
		FF->precond = Diag_precond;
		FF->precond_setup = ebe ? Diag_precond_EBE_setup : ede ? Diag_precond_EDE_setup : Diag_precond_CSR_setup;
	} else {
		FF->precond = ILUp_precond; FF->precond_setup = ILUp_precond_setup;
	}
	FF->precondR = NO_precond;
	FF->scaling = noscale;
	FF->unscaling = nounscale;
	int predictor2 = strncasecmp(tint, "Predictor2", 10) == 0;
	FOF->Build = predictor2 ? Build_M_F_DD : strcasecmp(stab, "DD") == 0 ? Build_M_K_R_DD : Build_M_K_R_SUPG;
	FF->ShockCapture = strcasecmp(shock, "YZBeta") == 0 ? YZBeta_ShockCapture
	                 : strcasecmp(shock, "CAUDD") == 0 ? CAU_DD_ShockCapture : CAU_ShockCapture;
	FF->h_shock = strcasecmp(hshock, "Option1") == 0 ? h_shock_Option1
	            : strcasecmp(hshock, "Option2") == 0 ? h_shock_Option2 : h_shock_2sqrtArea;
	setStopCriteria(P, FF);

	/* the plug-ins as Build_M_K_R_*.c evaluate them */
	{
		double third = 1.0 / 3.0, k = FF->Condutivity(), g = FF->Reaction(), b[2];
		for (I = 0; I < nel; I++) {
			int *v = Element[I].Vertex;
			double XB = third * (Node[v[0]].x + Node[v[1]].x + Node[v[2]].x);
			double YB = third * (Node[v[0]].y + Node[v[1]].y + Node[v[2]].y);
			FF->Velocity(XB, YB, b);
			beta[2 * I] = b[0]; beta[2 * I + 1] = b[1];
			for (J = 0; J < 3; J++) fsrc[3 * I + J] = FF->Font(Node[v[J]].x, Node[v[J]].y, k, g, b[0], b[1]);
		}
		for (I = 0; I < nnodes; I++) upresc[I] = FF->upresc(Node[I].x, Node[I].y);
		memset(u0, 0, sizeof(double) * (neq + 1));
		FF->InitialSolution(P, Node, u0);
	}

	/* two Builds on (ub, dub) (and the bubbles (ubB, dubB) for Build_M_F_DD),
	 * fresh per-element state */
	{
		double *dold = mycalloc("delta_old", nel, sizeof(double));
		AuxBuildStructuresType *aux = mycalloc("aux", 1, sizeof(AuxBuildStructuresType));
		double **M2 = mycalloc("M2", nel, sizeof(double *)), *M2aux = mycalloc("M2aux", 3 * nel, sizeof(double));
		double **R2b = mycalloc("R2", nel, sizeof(double *)), *R2aux = mycalloc("R2aux", nel, sizeof(double));
		double *uBb = mycalloc("uB", nel, sizeof(double)), *duBb = mycalloc("duB", nel, sizeof(double));
		for (I = 0; I < nel; I++) { M2[I] = M2aux + 3 * I; R2b[I] = R2aux + I; }
		aux->tolerance = stab_tol;
		aux->M2 = M2; aux->R2 = R2b; aux->invN2 = mycalloc("invN2", nel, sizeof(double));
		if (predictor2) {
			memcpy(uBb, ubB, sizeof(double) * nel);
			memcpy(duBb, dubB, sizeof(double) * nel);
		}
		FS->uB = uBb; FS->duB = duBb;
		FS->AuxBuild = aux;
		FS->delta_old = dold;
		P->Alpha_Build = alpha;
		P->DeltaT_Build = dt;
		memcpy(u, ub, sizeof(double) * (neq + 1));
		memcpy(du, dub, sizeof(double) * (neq + 1));
		FOF->Build(P, M, FS, FF);
		memcpy(A1, ebe || ede ? M->Aaux : M->AA, sizeof(double) * nA);
		memcpy(R1, F, sizeof(double) * (neq + 1));
		FOF->Build(P, M, FS, FF);
		memcpy(A2, ebe || ede ? M->Aaux : M->AA, sizeof(double) * nA);
		memcpy(R2, F, sizeof(double) * (neq + 1));
		free(dold);
		free(aux->invN2); free(aux);
		free(M2); free(M2aux); free(R2b); free(R2aux); free(uBb); free(duBb);
		memset(u, 0, sizeof(double) * (neq + 1));
	}

	/* the reference's time loop */
	g_uhist = uhist; g_thist = thist; g_iters = iters; g_ncorr = ncorr; g_u = u; g_neq = neq;
	g_stage = 0; g_tcheck = 0; g_maxsteps = maxsteps; g_corr = 0; g_cap = 2 * maxsteps + 2;
	g_steady = strcasecmp(steady, "YES") == 0;
	g_norm = strcasecmp(stopmc, "NORM") == 0;
	FF->StopCriteria = record_stage;
	FF->StopTimeIntegration = record_step;
	FOF->solver = solver_rec;
	if (strcasecmp(tint, "Predictor1_BDF") == 0) Predictor_Old_BDF(P, M, FS, FF, FOF);
	else if (strcasecmp(tint, "Predictor1_TRBDF2") == 0) Predictor_Old_TRBDF2(P, M, FS, FF, FOF);
	else if (strcasecmp(tint, "Predictor2_BDF") == 0) Predictor_New_BDF(P, M, FS, FF, FOF);
	else if (strcasecmp(tint, "Predictor2_TRBDF2") == 0) Predictor_New_TRBDF2(P, M, FS, FF, FOF);
	else if (predictor2) Predictor_New(P, M, FS, FF, FOF);
	else Predictor_Old(P, M, FS, FF, FOF);
	info[4] = g_tcheck;
	return g_stage < g_cap ? g_stage : g_cap;
}

/* The transient driver's own Preprocess (Preprocess.c:5-180) on a deck (the
 * mesh file at ../../../../INPUT_DATA/<title>_<nnodes>_<nel>.dat from the
 * working directory): iv [7] = nnodes, nel, neq, NonLinearMaxIter,
 * LinearMaxIter, KrylovBasisVectorsQuantity, nnzero (CSR); dv [7] =
 * SolverTolerance, NonLinearTolerance, TimeIntegrationTolerance,
 * StabilizationTolerance, Alpha, DeltaT, FinalTime; sv [13 x 64] the
 * strings in reading order; per node x, y, Type, id; per element the
 * vertices and Type. */
int Preprocess(int, char **, ParametersType **, MatrixDataType **, FemStructsType **, FemFunctionsType **,
               FemOtherFunctionsType **);

int ref_transient_preprocess(const char *deck, int *iv, double *dv, char *sv, double *x, double *y, int *type,
                             int *id, int *vert, int *etype, int cap_nodes, int cap_el)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF; FemOtherFunctionsType *FOF;
	char *argv[2] = { "harness", (char *)deck };
	int I;
	const char *str[13];
	Preprocess(2, argv, &P, &M, &FS, &FF, &FOF);
	iv[0] = P->nnodes; iv[1] = P->nel; iv[2] = P->neq; iv[3] = P->NonLinearMaxIter; iv[4] = P->LinearMaxIter;
	iv[5] = P->KrylovBasisVectorsQuantity; iv[6] = P->nnzero;
	dv[0] = P->SolverTolerance; dv[1] = P->NonLinearTolerance; dv[2] = P->TimeIntegrationTolerance;
	dv[3] = P->StabilizationTolerance; dv[4] = P->Alpha; dv[5] = P->DeltaT; dv[6] = P->FinalTime;
	str[0] = P->ProblemTitle; str[1] = P->StopAtSteadyState; str[2] = P->Solver; str[3] = P->Preconditioner;
	str[4] = P->Scaling; str[5] = P->reordering; str[6] = P->MatrixVectorProductScheme;
	str[7] = P->StabilizationForm; str[8] = P->ShockCapture; str[9] = P->h_Shock; str[10] = P->TimeIntegration;
	str[11] = P->StopMulticorrection; str[12] = "";
	for (I = 0; I < 13; I++) strncpy(sv + 64 * I, str[I], 63);
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
