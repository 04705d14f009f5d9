/*
 * Test infrastructure only: drives the reference's 2D Euler SUPG+CAU element
 * build (03_Euler_Equations/2D/01_CommonFiles/Build_M_K_F_SUPG.c with
 * Delta_CAU.c, Ax_Ay_calculations.c, eval_U_dU.c, ebe_assembly.c, the
 * REFLETIDO plug-in) and its predictor-multicorrector (Predictor_Old.c:46-132
 * control flow) on in-memory arrays, compiled from the reference's sources by
 * oracle/Makefile with -DEulerEquations2D.
 *
 * The solver is the 6-argument GMRES adapter of ref_gmres6.h (the shipped
 * pgmres.c has only the steady-transport 4-argument form).
 *
 * CSR storage with ILU(0) (csr_Initialization.c and csr_assembly.c of the
 * Euler driver, reordering NOT, csrmv, ILUp_precond_setup.c /
 * ILUp_precond.c: setMatrixVectorProductType.c:24 and setPreconditioner.c:
 * 118-128) is the csr != 0 form of the set-up.
 */
#include "EulerEquations.h"

void *mycalloc(char *, int, int);
void myfree(void *);
int ebemvNDOF4(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int BlockDiag_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int BlockDiag_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int Block_scaling_EBE(ParametersType *, MatrixDataType *, FemStructsType *);
int Build_M_K_F_SUPG(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *);
double Delta_CAU(double, double *, double *, double *, double (*)[4], double (*)[4], double (*)[4],
                 double *, double, double, double, double, double, double, double, int, double *, double *);
double Delta_YZBeta(double, double *, double *, double *, double (*)[4], double (*)[4], double (*)[4],
                    double *, double, double, double, double, double, double, double, int, double *, double *);

/* Shock capturing of the builds below: 0 Delta_CAU, 1 Delta_YZBeta with the
 * deck's Y^-1 (the ShockCapture "YZBeta" of setStabilizationForm.c:27). */
static int g_yz, g_dd;
static double g_invY[4];
/* The element build of the predictor below: 0 Build_M_K_F_SUPG, 1 the DD
 * build Build_M_K_F_DD_Transiente (StabilizationForm "DD"; shock capturing
 * Delta_DD, or Delta_YZBeta after ref_euler_set_shock(1, ...)). */
void ref_euler_set_dd(int dd) { g_dd = dd; }
void ref_euler_set_shock(int yzbeta, const double *invY)
{
	int k;
	g_yz = yzbeta;
	for (k = 0; k < 4; k++) g_invY[k] = invY ? invY[k] : 1.0;
}
void dimensional_Ax_Ay_calculations(double, double, double *, double (*)[4], double (*)[4]);
int Build_M_K_F_DD_Transiente(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *);
double Delta_DD(double, double *, double *, double *, double (*)[4], double (*)[4], double (*)[4],
                double *, double, double, double, double, double, double, double, int, double *, double *);
double REFLETIDO_gamma(double, double);
double REFLETIDO_rhopresc(double, double);
double REFLETIDO_v1presc(double, double);
double REFLETIDO_v2presc(double, double);
double REFLETIDO_epresc(double, double);
static double zero_theta(double x, double y) { return 0.0; }
void csr_Initialization(ParametersType *, NodeType *, int **, int **, int **, int **, int ***, int **, int ***);
void csr_assembly(ParametersType *, MatrixDataType *, FemStructsType *, int, double (*)[12]);
int csrmv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int ILUp_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
int ILUp_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);

#include "ref_gmres6.h"

static void setup(int csr, int nnodes, const double *x, const double *y, const int *node_id, int nel,
                  const int *vert, int neq, double alpha, double dt, double stab_tol,
                  ParametersType **Po, MatrixDataType **Mo, FemStructsType **FSo, FemFunctionsType **FFo)
{
	int I, k;
	ParametersType *P = mycalloc("P", 1, sizeof(ParametersType));
	MatrixDataType *M = mycalloc("M", 1, sizeof(MatrixDataType));
	FemStructsType *FS = mycalloc("FS", 1, sizeof(FemStructsType));
	FemFunctionsType *FF = mycalloc("FF", 1, sizeof(FemFunctionsType));
	NodeType *Node = mycalloc("Node", nnodes, sizeof(NodeType));
	ElementType *El = mycalloc("El", nel, sizeof(ElementType));
	int **lm = mycalloc("lm", nel, sizeof(int *)), *lmaux = mycalloc("lmaux", nel * 12, sizeof(int));
	double **A = mycalloc("A", nel, sizeof(double *)), *Aaux = mycalloc("Aaux", nel * 144, sizeof(double));
	AuxBuildStructuresType *aux = mycalloc("aux", 1, sizeof(AuxBuildStructuresType));
	P->nnodes = nnodes; P->nel = nel; P->neq = neq;
	P->Alpha = alpha; P->Alpha_Build = alpha; P->DeltaT = dt; P->DeltaT_Build = dt;
	P->StabilizationTolerance = stab_tol;
	strcpy(P->MatrixVectorProductScheme, csr ? "CSR" : "EBE");
	strcpy(P->Preconditioner, csr ? "ILU0" : "BlockDiag");
	strcpy(P->reordering, "NOT");
	for (I = 0; I < nnodes; I++) {
		Node[I].x = x[I]; Node[I].y = y[I];
		Node[I].rhoType = Node[I].v1Type = Node[I].v2Type = Node[I].eType = 1;
		for (k = 0; k < 4; k++) Node[I].id[k] = node_id[4 * I + k];
	}
	for (I = 0; I < nel; I++) {
		for (k = 0; k < 3; k++) El[I].Vertex[k] = vert[3 * I + k];
		lm[I] = lmaux + 12 * I;
		A[I] = Aaux + 144 * I;
	}
	Fill_LM(neq, nel, lm, Node, El);
	M->A = A; M->Aaux = Aaux;
	if (csr) {
		int *IA, *JA, *perm, *invperm, **sbe;
		csr_Initialization(P, Node, &JA, &IA, &perm, &invperm, &lm, &lmaux, &sbe);
		M->AA = mycalloc("AA", P->nnzero + 1, sizeof(double));
		M->IA = IA; M->JA = JA; M->Scheme_by_Element = sbe; M->Perm = perm; M->invPerm = invperm;
	}
	aux->tolerance = stab_tol;
	FS->lm = lm; FS->Node = Node; FS->Element = El; FS->AuxBuild = aux;
	FS->F = mycalloc("F", neq + 1, sizeof(double));
	FS->u = mycalloc("u", neq + 1, sizeof(double));
	FS->du = mycalloc("du", neq + 1, sizeof(double));
	FS->delta_old = mycalloc("delta_old", nel, sizeof(double));
	FS->uB = mycalloc("uB", 4 * nel, sizeof(double));
	FF->gamma = REFLETIDO_gamma;
	FF->rhopresc = REFLETIDO_rhopresc; FF->v1presc = REFLETIDO_v1presc;
	FF->v2presc = REFLETIDO_v2presc; FF->epresc = REFLETIDO_epresc;
	FF->Ax_Ay_calculations = dimensional_Ax_Ay_calculations;
	FF->ShockCapture = g_yz ? Delta_YZBeta : g_dd ? Delta_DD : Delta_CAU;
	for (k = 0; k < 4; k++) P->invY[k] = g_invY[k];
	FF->BC_theta = zero_theta;
	FF->assembly = csr ? csr_assembly : ebe_assembly;
	FF->mv = csr ? csrmv : ebemvNDOF4;
	FF->precond = csr ? ILUp_precond : BlockDiag_precond;
	FF->precond_setup = csr ? ILUp_precond_setup : BlockDiag_precond_EBE_setup;
	*Po = P; *Mo = M; *FSo = FS; *FFo = FF;
}

/* Two consecutive Builds on the state (u, du) from a zero delta_old (the
 * second reads the first's per-element shock parameter: Delta_YZBeta keeps
 * one): Ae1, R1 and Ae2, R2, and delta_old after the second [nel]. */
int ref_euler_build2(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                     int neq, double alpha, double dt, double stab_tol, const double *u, const double *du,
                     double *Ae1, double *R1, double *Ae2, double *R2, double *dold)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	setup(0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	memcpy(FS->u, u, sizeof(double) * (neq + 1));
	memcpy(FS->du, du, sizeof(double) * (neq + 1));
	Build_M_K_F_SUPG(P, M, FS, FF);
	memcpy(Ae1, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R1, FS->F, sizeof(double) * (neq + 1));
	Build_M_K_F_SUPG(P, M, FS, FF);
	memcpy(Ae2, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R2, FS->F, sizeof(double) * (neq + 1));
	memcpy(dold, FS->delta_old, sizeof(double) * nel);
	return 0;
}

/* One Build on the state (u, du): element matrices Ae [nel*144] and R. */
int ref_euler_build(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                    int neq, double alpha, double dt, double stab_tol, const double *u, const double *du,
                    double *Ae, double *R)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	setup(0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	memcpy(FS->u, u, sizeof(double) * (neq + 1));
	memcpy(FS->du, du, sizeof(double) * (neq + 1));
	Build_M_K_F_SUPG(P, M, FS, FF);
	memcpy(Ae, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R, FS->F, sizeof(double) * (neq + 1));
	return 0;
}

/* One Build followed by the scaling Block_scaling_EBE (Block_scaling.c:7-49,
 * the Scaling "BlockScaling" of setScaling.c): scaled Ae [nel*144] and R. */
int ref_euler_build_scaled(int nnodes, const double *x, const double *y, const int *node_id, int nel,
                           const int *vert, int neq, double alpha, double dt, double stab_tol, const double *u,
                           const double *du, double *Ae, double *R)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	setup(0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	memcpy(FS->u, u, sizeof(double) * (neq + 1));
	memcpy(FS->du, du, sizeof(double) * (neq + 1));
	Build_M_K_F_SUPG(P, M, FS, FF);
	Block_scaling_EBE(P, M, FS);
	memcpy(Ae, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R, FS->F, sizeof(double) * (neq + 1));
	return 0;
}

/* A slip-wall angle with the shape of the reference's BC_theta plug-ins
 * (CYLINDER/CYLINDER_theta.c: atan(-x/y) about the cylinder's centre); here
 * about (2, -1), below the REFLETIDO domain, so it is defined on every wall
 * node. */
static double slip_theta(double x, double y) { return atan(-(x - 2.0) / (y + 1.0)); }

/* One Build with slip walls: nodes with slip[I] != 0 get v1Type = -1, so
 * Build_M_K_F_SUPG.c:1044-1056 rotates their rows and columns of Ae and their
 * Re by BC_theta (rotation.c:3-43).  Outputs Ae [nel*144], R, and the
 * cos / sin of each node's angle as rotation.c evaluates them (cs, sn
 * [nnodes], 1 / 0 off the wall). */
int ref_euler_build_slip(int nnodes, const double *x, const double *y, const int *node_id, const int *slip,
                         int nel, const int *vert, int neq, double alpha, double dt, double stab_tol,
                         const double *u, const double *du, double *Ae, double *R, double *cs, double *sn)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	int I;
	setup(0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	for (I = 0; I < nnodes; I++) {
		cs[I] = 1.0; sn[I] = 0.0;
		if (slip[I]) {
			double th = slip_theta(x[I], y[I]);
			FS->Node[I].v1Type = -1;
			cs[I] = cos(th); sn[I] = sin(th);
		}
	}
	FF->BC_theta = slip_theta;
	memcpy(FS->u, u, sizeof(double) * (neq + 1));
	memcpy(FS->du, du, sizeof(double) * (neq + 1));
	Build_M_K_F_SUPG(P, M, FS, FF);
	memcpy(Ae, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R, FS->F, sizeof(double) * (neq + 1));
	return 0;
}

/* Predictor_Old.c:46-132 with ncorr correctors per step (StopByIterations,
 * Criteria.c:25-31) and nsteps steps, BlockDiag + EBE + the GMRES above.
 * u in/out; ahist [nsteps*(neq+1)], uhist likewise; iters [nsteps*ncorr]. */
static int predictor(int csr, int scaling, int nnodes, const double *x, const double *y, const int *node_id, int nel,
                     const int *vert, int neq, double alpha, double dt, double stab_tol, int kmax,
                     int lmax, double tol, int nsteps, int ncorr, double *u_io, double *uhist, int *iters)
{
	int I, step, i, tag = 1;
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	setup(csr, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	P->KrylovBasisVectorsQuantity = kmax; P->LinearMaxIter = lmax; P->SolverTolerance = tol;
	double *u = FS->u, *a = FS->du, *R = FS->F, *Da = calloc(neq + 1, sizeof(double));
	memcpy(u, u_io, sizeof(double) * (neq + 1));
	for (step = 0; step < nsteps; step++) {
		for (I = 0; I < neq; I++) { u[I] += (1.0 - alpha)*dt*a[I]; a[I] = 0.0; }
		for (i = 0; i < ncorr; i++) {
			int before = P->iterations;
			if (g_dd) Build_M_K_F_DD_Transiente(P, M, FS, FF);
			else Build_M_K_F_SUPG(P, M, FS, FF);
			if (scaling) Block_scaling_EBE(P, M, FS);       /* Predictor_Old.c:73 */
			FF->precond_setup(P, M, FS, tag++, R);
			gmres6(P, M, FS, FF, R, Da);
			iters[step * ncorr + i] = P->iterations - before;
			for (I = 0; I < neq; I++) a[I] += 1 * Da[I];
			for (I = 0; I < neq; I++) u[I] += alpha*dt * Da[I];
		}
		memcpy(uhist + (size_t)step * (neq + 1), u, sizeof(double) * (neq + 1));
	}
	memcpy(u_io, u, sizeof(double) * (neq + 1));
	free(Da);
	return 0;
}

int ref_euler_predictor(int nnodes, const double *x, const double *y, const int *node_id, int nel,
                        const int *vert, int neq, double alpha, double dt, double stab_tol, int kmax,
                        int lmax, double tol, int nsteps, int ncorr, double *u_io, double *uhist, int *iters)
{
	return predictor(0, 0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, kmax, lmax, tol, nsteps, ncorr,
	                 u_io, uhist, iters);
}

/* The same predictor with Block_scaling_EBE after every Build. */
int ref_euler_predictor_scaled(int nnodes, const double *x, const double *y, const int *node_id, int nel,
                               const int *vert, int neq, double alpha, double dt, double stab_tol, int kmax,
                               int lmax, double tol, int nsteps, int ncorr, double *u_io, double *uhist, int *iters)
{
	return predictor(0, 1, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, kmax, lmax, tol, nsteps, ncorr,
	                 u_io, uhist, iters);
}

/* The same predictor with CSR storage and ILU(0). */
int ref_euler_predictor_csr(int nnodes, const double *x, const double *y, const int *node_id, int nel,
                            const int *vert, int neq, double alpha, double dt, double stab_tol, int kmax,
                            int lmax, double tol, int nsteps, int ncorr, double *u_io, double *uhist, int *iters)
{
	return predictor(1, 0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, kmax, lmax, tol, nsteps, ncorr,
	                 u_io, uhist, iters);
}

/* CSR set-up and one Build with CSR assembly on (u, du): pattern IA [neq+1],
 * JA [nnz_cap], CSR_by_Element sbe [nel*144], the assembled values AA
 * [nnz_cap+1], the residual R [neq+1], R after precond_setup (ILU(0),
 * R := M^-1 R) Rp [neq+1] and one ILU(0) application z = M^-1 p [neq+1].
 * Returns nnz (or -1 when nnz_cap is too small). */
int ref_euler_build_csr(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                        int neq, double alpha, double dt, double stab_tol, const double *u, const double *du,
                        int nnz_cap, int *IA, int *JA, int *sbe, double *AA, double *R, double *Rp, const double *p,
                        double *z)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	int nnz, e;
	size_t n1 = (size_t)neq + 1;
	setup(1, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	nnz = P->nnzero;
	if (nnz > nnz_cap) return -1;
	memcpy(IA, M->IA, sizeof(int) * n1);
	memcpy(JA, M->JA, sizeof(int) * (size_t)nnz);
	for (e = 0; e < nel; e++) memcpy(sbe + (size_t)144 * e, M->Scheme_by_Element[e], sizeof(int) * 144);
	memcpy(FS->u, u, sizeof(double) * n1);
	memcpy(FS->du, du, sizeof(double) * n1);
	Build_M_K_F_SUPG(P, M, FS, FF);
	memcpy(AA, M->AA, sizeof(double) * ((size_t)nnz + 1));
	memcpy(R, FS->F, sizeof(double) * n1);
	memcpy(Rp, FS->F, sizeof(double) * n1);
	FF->precond_setup(P, M, FS, 1, Rp);
	{
		double *pp = mycalloc("p", n1, sizeof(double));
		memcpy(pp, p, sizeof(double) * n1);
		FF->precond(P, M, FS, pp, z);
	}
	return nnz;
}

/* The reference's own Predictor_Old_BDF.c / Predictor_Old_TRBDF2.c
 * (00_CommonFiles/Time_Integration, TimeIntegration "Predictor1_BDF" /
 * "Predictor1_TRBDF2" of setStabilizationForm.c:12-17) on the EBE
 * BlockDiag set-up above: ncorr correctors per stage (StopByIterations) and
 * nsteps time checks (StopTimeIntegration).  Per stage (multicorrection
 * loop): uhist [cap*(neq+1)] u at its end, iters [cap*ncorr] the GMRES
 * iterations of its correctors.  Returns the number of stages. */
int Predictor_Old_BDF(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *,
                      FemOtherFunctionsType *);
int Predictor_Old_TRBDF2(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *,
                         FemOtherFunctionsType *);
static const double *g_u0;
static double *g_uh, *g_uc;
static int *g_it, g_stage, g_cap, g_ncorr, g_nchk, g_maxchk, g_neq1, g_corr;
static int tint_init(ParametersType *P, NodeType *N, double *u)
{
	(void)N;
	memcpy(u, g_u0, sizeof(double) * (P->neq + 1));
	return 0;
}
static int tint_stage(ParametersType *P, double na, double nda, int i)
{
	(void)na; (void)nda;
	if (i < g_ncorr) return 0;
	if (g_stage < g_cap) memcpy(g_uh + (size_t)g_stage * g_neq1, g_uc, sizeof(double) * g_neq1);
	g_stage++;
	g_corr = 0;
	return 1;
}
static int tint_time(ParametersType *P, double *u, double *uo, double t)
{
	(void)P; (void)u; (void)uo; (void)t;
	return ++g_nchk >= g_maxchk;
}
static int tint_solver(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF, double *B,
                       double *X)
{
	int before = P->iterations, rc = gmres6(P, M, FS, FF, B, X);
	if (g_stage < g_cap && g_corr < g_ncorr) g_it[(size_t)g_stage * g_ncorr + g_corr] = P->iterations - before;
	g_corr++;
	return rc;
}
static int tint_noscale(ParametersType *P, MatrixDataType *M, FemStructsType *FS) { return 0; }
static int tint_nounscale(ParametersType *P, MatrixDataType *M, FemStructsType *FS, double *x) { return 0; }

int ref_euler_predictor_tint(int trbdf2, int nnodes, const double *x, const double *y, const int *node_id, int nel,
                             const int *vert, int neq, double alpha, double dt, double stab_tol, int kmax, int lmax,
                             double tol, int nsteps, int ncorr, const double *u0, int cap, double *uhist, int *iters)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	FemOtherFunctionsType *FOF = mycalloc("FOF", 1, sizeof(FemOtherFunctionsType));
	setup(0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	P->KrylovBasisVectorsQuantity = kmax; P->LinearMaxIter = lmax; P->SolverTolerance = tol;
	P->NonLinearMaxIter = ncorr;
	FOF->Build = Build_M_K_F_SUPG;
	FOF->solver = tint_solver;
	FF->InitialSolution = tint_init;
	FF->StopCriteria = tint_stage;
	FF->StopTimeIntegration = tint_time;
	FF->scaling = tint_noscale;
	FF->unscaling = tint_nounscale;
	g_u0 = u0; g_uh = uhist; g_uc = FS->u; g_it = iters; g_stage = 0; g_cap = cap; g_ncorr = ncorr;
	g_nchk = 0; g_maxchk = nsteps; g_neq1 = neq + 1; g_corr = 0;
	if (trbdf2) Predictor_Old_TRBDF2(P, M, FS, FF, FOF);
	else Predictor_Old_BDF(P, M, FS, FF, FOF);
	return g_stage;
}

/* Two consecutive DD builds (Build_M_K_F_DD_Transiente.c:6-915, the
 * StabilizationForm "DD" of setStabilizationForm.c:33-46) on (u, du) from a
 * zero delta_old and the element bubbles uB0 [4*nel]: shock capturing Delta_DD
 * ("CAUDD"), or Delta_YZBeta after ref_euler_set_shock(1, ...).  Ae1, R1,
 * Ae2, R2 as ref_euler_build2; uB [4*nel] and delta_old [nel] after the
 * second build. */
int ref_euler_build_dd(int nnodes, const double *x, const double *y, const int *node_id, int nel, const int *vert,
                       int neq, double alpha, double dt, double stab_tol, const double *u, const double *du,
                       const double *uB0, double *Ae1, double *R1, double *Ae2, double *R2, double *uB, double *dold)
{
	ParametersType *P; MatrixDataType *M; FemStructsType *FS; FemFunctionsType *FF;
	setup(0, nnodes, x, y, node_id, nel, vert, neq, alpha, dt, stab_tol, &P, &M, &FS, &FF);
	if (!g_yz) FF->ShockCapture = Delta_DD;
	memcpy(FS->uB, uB0, sizeof(double) * 4 * nel);
	memcpy(FS->u, u, sizeof(double) * (neq + 1));
	memcpy(FS->du, du, sizeof(double) * (neq + 1));
	Build_M_K_F_DD_Transiente(P, M, FS, FF);
	memcpy(Ae1, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R1, FS->F, sizeof(double) * (neq + 1));
	Build_M_K_F_DD_Transiente(P, M, FS, FF);
	memcpy(Ae2, M->Aaux, sizeof(double) * nel * 144);
	memcpy(R2, FS->F, sizeof(double) * (neq + 1));
	memcpy(uB, FS->uB, sizeof(double) * 4 * nel);
	memcpy(dold, FS->delta_old, sizeof(double) * nel);
	return 0;
}
