/*
 * Parameter decks and mesh files of the three drivers: the reading half of
 * Preprocess (01_SS_Transport_Equation/2D/01_CommonFiles/Preprocess.c:44-99,
 * 03_Euler_Equations/2D/01_CommonFiles/Preprocess.c:45-102,
 * 04_SS_NavierStokes_Equations/2D/01_CommonFiles/Preprocess.c:45-88), so a
 * run can start from the reference's own input files.
 *
 * A deck is one "value<TAB>:label" line per parameter in a fixed order per
 * driver; it is read with the same conversions the drivers use (the
 * preconditioner string of the Euler and Navier-Stokes decks may hold
 * blanks, "AMG 2 3 -1 1.0 2").  A mesh file holds the node count, one line
 * per node (x, y and the driver's node types: 1 for transport, 4 for Euler,
 * 3 for Navier-Stokes), the element count and one line per element (three
 * vertices and the element type); it is parsed from one buffered read of the
 * file (at 2048x1024 cells the file has 6.3M lines).  Plain C.
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "femgpu.h"
#include "femgpu_host.h"

#define RD(fmt, ...) do { if (fscanf(f, fmt, __VA_ARGS__) < 1) { bad = 1; goto done; } } while (0)

int femgpu_deck_read(const char *path, int equation, femgpu_deck *d)
{
	char label[2048];
	FILE *f;
	int bad = 0;
	if (!path || !d || equation < FEMGPU_EQ_TRANSPORT || equation > FEMGPU_EQ_TRANSIENT) return FEMGPU_E_ARG;
	f = fopen(path, "r");
	if (!f) { fgh_set_error("deck %s: cannot open", path); return FEMGPU_E_ARG; }
	memset(d, 0, sizeof *d);
	d->equation = equation;
	if (equation == FEMGPU_EQ_TRANSPORT) {            /* Preprocess.c:44-61 */
		RD("%199s\t:%2047[^\n]\n", d->Experiments, label);
		RD("%299s\t:%2047[^\n]\n", d->ProblemTitle, label);
		RD("%lf\t:%2047[^\n]\n", &d->SolverTolerance, label);
		RD("%lf\t:%2047[^\n]\n", &d->NonLinearTolerance, label);
		RD("%d\t:%2047[^\n]\n", &d->SolverMaxIter, label);
		RD("%d\t:%2047[^\n]\n", &d->KrylovBasisVectorsQuantity, label);
		RD("%199s\t:%2047[^\n]\n", d->Solver, label);
		RD("%999s\t:%2047[^\n]\n", d->Preconditioner, label);
		RD("%199s\t:%2047[^\n]\n", d->Scaling, label);
		RD("%199s\t:%2047[^\n]\n", d->reordering, label);
		RD("%199s\t:%2047[^\n]\n", d->MatrixVectorProductScheme, label);
		RD("%199s\t:%2047[^\n]\n", d->StabilizationForm, label);
		RD("%199s\t:%2047[^\n]\n", d->ShockCapture, label);
		RD("%199s\t:%2047[^\n]\n", d->h_Shock, label);
		RD("%199s\t:%2047[^\n]\n", d->OutputFlow, label);
		RD("%d\t:%2047[^\n]\n", &d->nnodes, label);
		RD("%d\t:%2047[^\n]\n", &d->nel, label);
	} else if (equation == FEMGPU_EQ_TRANSIENT) {     /* 02_Transport_Equation Preprocess.c:42-66 */
		RD("%299s\t:%2047[^\n]\n", d->ProblemTitle, label);
		RD("%lf\t:%2047[^\n]\n", &d->SolverTolerance, label);
		RD("%lf\t:%2047[^\n]\n", &d->NonLinearTolerance, label);
		RD("%lf\t:%2047[^\n]", &d->TimeIntegrationTolerance, label);
		RD("%lf\t:%2047[^\n]", &d->StabilizationTolerance, label);
		RD("%d\t:%2047[^\n]\n", &d->NonLinearMaxIter, label);
		RD("%d\t:%2047[^\n]\n", &d->LinearMaxIter, label);
		RD("%199s\t:%2047[^\n]\n", d->StopAtSteadyState, label);
		RD("%d\t:%2047[^\n]\n", &d->KrylovBasisVectorsQuantity, label);
		RD("%199s\t:%2047[^\n]\n", d->Solver, label);
		RD("%999s\t:%2047[^\n]\n", d->Preconditioner, label);
		RD("%199s\t:%2047[^\n]\n", d->Scaling, label);
		RD("%199s\t:%2047[^\n]\n", d->reordering, label);
		RD("%199s\t:%2047[^\n]\n", d->MatrixVectorProductScheme, label);
		RD("%199s\t:%2047[^\n]\n", d->StabilizationForm, label);
		RD("%199s\t:%2047[^\n]\n", d->ShockCapture, label);
		RD("%199s\t:%2047[^\n]\n", d->h_Shock, label);
		RD("%199s\t:%2047[^\n]\n", d->TimeIntegration, label);
		RD("%lf\t:%2047[^\n]\n", &d->Alpha, label);
		RD("%lf\t:%2047[^\n]\n", &d->DeltaT, label);
		RD("%199s\t:%2047[^\n]", d->StopMulticorrection, label);
		RD("%lf\t:%2047[^\n]\n", &d->FinalTime, label);
		RD("%d\t:%2047[^\n]\n", &d->nnodes, label);
		RD("%d\t:%2047[^\n]\n", &d->nel, label);
	} else if (equation == FEMGPU_EQ_EULER) {         /* Preprocess.c:45-74 */
		RD("%199s\t:%2047[^\n]", d->Experiments, label);
		RD("%299s\t:%2047[^\n]", d->ProblemTitle, label);
		RD("%lf\t:%2047[^\n]", &d->SolverTolerance, label);
		RD("%lf\t:%2047[^\n]", &d->NonLinearTolerance, label);
		RD("%lf\t:%2047[^\n]", &d->TimeIntegrationTolerance, label);
		RD("%lf\t:%2047[^\n]", &d->StabilizationTolerance, label);
		RD("%d\t:%2047[^\n]", &d->LinearMaxIter, label);
		RD("%d\t:%2047[^\n]", &d->KrylovBasisVectorsQuantity, label);
		RD("%199s\t:%2047[^\n]", d->Solver, label);
		RD("\n%999[^\t]%2047[^\n]\n", d->Preconditioner, label);
		RD("%199s\t:%2047[^\n]\n", d->Scaling, label);
		RD("%199s\t:%2047[^\n]", d->reordering, label);
		RD("%199s\t:%2047[^\n]", d->TimeIntegration, label);
		RD("%199s\t:%2047[^\n]", d->StopAtSteadyState, label);
		RD("%lf\t:%2047[^\n]", &d->Alpha, label);
		RD("%lf\t:%2047[^\n]", &d->DeltaT, label);
		RD("%lf\t:%2047[^\n]", &d->FinalTime, label);
		RD("%199s\t:%2047[^\n]", d->Dimensionless, label);
		RD("%lf\t:%2047[^\n]", &d->Mach, label);
		RD("%d\t:%2047[^\n]", &d->NonLinearMaxIter, label);
		RD("%199s\t:%2047[^\n]", d->StopMulticorrection, label);
		RD("%199s\t:%2047[^\n]", d->MatrixVectorProductScheme, label);
		RD("%199s\t:%2047[^\n]", d->StabilizationForm, label);
		RD("%199s\t:%2047[^\n]", d->ShockCapture, label);
		RD("%lf\t:%2047[^\n]", &d->invY[0], label);
		RD("%lf\t:%2047[^\n]", &d->invY[1], label);
		RD("%lf\t:%2047[^\n]", &d->invY[2], label);
		RD("%lf\t:%2047[^\n]", &d->invY[3], label);
		RD("%d\t:%2047[^\n]", &d->nnodes, label);
		RD("%d\t:%2047[^\n]", &d->nel, label);
	} else {                                          /* Preprocess.c:45-60 */
		RD("%199s\t:%2047[^\n]", d->Experiments, label);
		RD("%299s\t:%2047[^\n]", d->ProblemTitle, label);
		RD("%lf\t:%2047[^\n]", &d->ReynoldsNumber, label);
		RD("%lf\t:%2047[^\n]", &d->VelMax, label);
		RD("%lf\t:%2047[^\n]", &d->SolverTolerance, label);
		RD("%d\t:%2047[^\n]", &d->SolverToleranceCase, label);
		RD("%lf\t:%2047[^\n]", &d->SolverToleranceNonLin, label);
		RD("%d\t:%2047[^\n]", &d->LinearMaxIter, label);
		RD("%d\t:%2047[^\n]", &d->KrylovBasisVectorsQuantity, label);
		RD("%199s\t:%2047[^\n]", d->Solver, label);
		RD("\n%999[^:]%2047[^\n]\n", d->Preconditioner, label);
		RD("%199s\t:%2047[^\n]", d->reordering, label);
		RD("%199s\t:%2047[^\n]", d->MatrixVectorProductScheme, label);
		RD("%199s\t:%2047[^\n]", d->StabilizationForm, label);
		RD("%d\t:%2047[^\n]", &d->nnodes, label);
		RD("%d\t:%2047[^\n]", &d->nel, label);
	}
done:
	fclose(f);
	if (bad) { fgh_set_error("deck %s: a parameter is missing or malformed", path); return FEMGPU_E_ARG; }
	/* the Euler/NS preconditioner string keeps its trailing blanks, as read */
	return 0;
}

int femgpu_deck_mesh_file(const femgpu_deck *d, const char *dir, char *path, int cap)
{
	int n;
	if (!d || !dir || !path || cap <= 0) return FEMGPU_E_ARG;
	n = snprintf(path, (size_t)cap, "%s/%s_%d_%d.dat", dir, d->ProblemTitle, d->nnodes, d->nel);
	return (n < 0 || n >= cap) ? FEMGPU_E_ARG : 0;
}

/* ---- mesh files ------------------------------------------------------- */
static char *skip_ws(char *p, const char *end)
{
	while (p < end && isspace((unsigned char)*p)) p++;
	return p;
}

static int next_int(char **p, const char *end, int *v)
{
	char *e;
	long x;
	*p = skip_ws(*p, end);
	if (*p >= end) return 0;
	x = strtol(*p, &e, 10);
	if (e == *p) return 0;
	*v = (int)x;
	*p = e;
	return 1;
}

static int next_double(char **p, const char *end, double *v)
{
	char *e;
	*p = skip_ws(*p, end);
	if (*p >= end) return 0;
	*v = strtod(*p, &e);
	if (e == *p) return 0;
	*p = e;
	return 1;
}

int femgpu_mesh_read(const char *path, int ntype, int *nnodes, int *nel, double *x, double *y, int *node_type,
                     int *vert, int *elem_type)
{
	FILE *f;
	char *buf = NULL, *p, *end;
	long len;
	int nn = 0, ne = 0, i, k, v, rc = 0, etype_col = !(ntype & FEMGPU_MESH_NO_ELEM_TYPE);
	ntype &= ~FEMGPU_MESH_NO_ELEM_TYPE;
	if (!path || !nnodes || !nel || ntype < 1 || ntype > 4) return FEMGPU_E_ARG;
	f = fopen(path, "rb");
	if (!f) { fgh_set_error("mesh %s: cannot open", path); return FEMGPU_E_ARG; }
	if (fseek(f, 0, SEEK_END) || (len = ftell(f)) < 0 || fseek(f, 0, SEEK_SET)) { fclose(f); return FEMGPU_E_ARG; }
	buf = malloc((size_t)len + 1);
	if (!buf) { fclose(f); return FEMGPU_E_NOMEM; }
	if (fread(buf, 1, (size_t)len, f) != (size_t)len) { fclose(f); free(buf); return FEMGPU_E_ARG; }
	fclose(f);
	buf[len] = 0;
	p = buf;
	end = buf + len;
	if (!next_int(&p, end, &nn) || nn <= 0) { rc = FEMGPU_E_MESH; goto out; }
	/* sizes only: skip the node block to the element count */
	for (i = 0; i < nn; i++) {
		double a, b;
		if (!next_double(&p, end, &a) || !next_double(&p, end, &b)) { rc = FEMGPU_E_MESH; goto out; }
		if (x) x[i] = a;
		if (y) y[i] = b;
		for (k = 0; k < ntype; k++) {
			if (!next_int(&p, end, &v)) { rc = FEMGPU_E_MESH; goto out; }
			if (node_type) node_type[(size_t)ntype * i + k] = v;
		}
	}
	if (!next_int(&p, end, &ne) || ne <= 0) { rc = FEMGPU_E_MESH; goto out; }
	if (vert || elem_type) {
		for (i = 0; i < ne; i++) {
			for (k = 0; k < 3; k++) {
				if (!next_int(&p, end, &v) || v < 0 || v >= nn) { rc = FEMGPU_E_MESH; goto out; }
				if (vert) vert[3 * (size_t)i + k] = v;
			}
			v = 0;
			if (etype_col && !next_int(&p, end, &v)) { rc = FEMGPU_E_MESH; goto out; }
			if (elem_type) elem_type[i] = v;
		}
	}
	*nnodes = nn;
	*nel = ne;
out:
	free(buf);
	if (rc) fgh_set_error("mesh %s: malformed (%d node types per node expected)", path, ntype);
	return rc;
}

int femgpu_mesh_side_types(int nnodes, const double *x, const double *y, int nel, const int *vert, int *elem_type)
{
	int e, j;
	if (nnodes <= 0 || nel <= 0 || !x || !y || !vert || !elem_type) return FEMGPU_E_ARG;
	for (e = 0; e < nel; e++) {
		int c[4] = { 0, 0, 0, 0 }, t = -1;
		for (j = 0; j < 3; j++) {
			const int v = vert[3 * (size_t)e + j];
			if (v < 0 || v >= nnodes) return FEMGPU_E_MESH;
			c[0] += x[v] == 0.0;
			c[1] += y[v] == 0.0;
			c[2] += x[v] == 1.0;
			c[3] += y[v] == 1.0;
		}
		/* the reference's test order: the first side holding two vertices
		 * decides, a corner only when the next side it is checked against
		 * holds two as well */
		if (c[0] == 2) t = c[1] == 2 ? 5 : c[3] == 2 ? 8 : 1;
		else if (c[1] == 2) t = c[2] == 2 ? 6 : 2;
		else if (c[2] == 2) t = c[3] == 2 ? 7 : 3;
		else if (c[3] == 2) t = 4;
		elem_type[e] = t;
	}
	return 0;
}

/* ---- deck strings -> options (setMatrixVectorProductType.c,
 * setPreconditioner.c, setStabilizationForm.c of each driver) ---------- */
static int ilu_level_of(const char *s)
{
	if (strncasecmp(s, "ILU", 3) != 0) return -1;
	return s[3] && !isspace((unsigned char)s[3]) ? atoi(s + 3) : 0;
}

int femgpu_deck_transport_opts(const femgpu_deck *d, femgpu_transport_opts *o)
{
	if (!d || !o || d->equation != FEMGPU_EQ_TRANSPORT) return FEMGPU_E_ARG;
	femgpu_transport_default_opts(o);
	if (!strcasecmp(d->MatrixVectorProductScheme, "CSR")) o->scheme = FEMGPU_CSR;
	else if (!strcasecmp(d->MatrixVectorProductScheme, "EDE")) o->scheme = FEMGPU_EDE;
	else if (!strcasecmp(d->MatrixVectorProductScheme, "EBE")) o->scheme = FEMGPU_EBE;
	else return FEMGPU_E_ARG;
	o->reorder = !strcasecmp(d->reordering, "SYMRCM") ? FEMGPU_REORDER_SYMRCM : FEMGPU_REORDER_NOT;
	if (!strcasecmp(d->Preconditioner, "NOT")) o->precond = FEMGPU_PREC_NOT;
	else if (!strcasecmp(d->Preconditioner, "Diag")) o->precond = FEMGPU_PREC_DIAG;
	else if (ilu_level_of(d->Preconditioner) >= 0) {
		o->precond = FEMGPU_PREC_ILU0;
		o->ilu_level = ilu_level_of(d->Preconditioner);
	} else return FEMGPU_E_ARG;
	if (strcasecmp(d->StabilizationForm, "SUPG") != 0) return FEMGPU_E_ARG;
	if (!strcasecmp(d->ShockCapture, "YZBeta")) o->shock = FEMGPU_SHOCK_YZBETA;
	else if (!strcasecmp(d->ShockCapture, "CAU")) o->shock = FEMGPU_SHOCK_CAU;
	else return FEMGPU_E_ARG;
	if (!strcasecmp(d->h_Shock, "sqrtArea")) o->hshock = FEMGPU_H_SQRTAREA;
	else if (!strcasecmp(d->h_Shock, "Option1")) o->hshock = FEMGPU_H_OPTION1;
	else if (!strcasecmp(d->h_Shock, "Option2")) o->hshock = FEMGPU_H_OPTION2;
	else if (!strcasecmp(d->h_Shock, "2sqrtArea")) o->hshock = FEMGPU_H_2SQRTAREA;
	else return FEMGPU_E_ARG;
	o->outflow = !strcasecmp(d->OutputFlow, "YES");
	o->kmax = d->KrylovBasisVectorsQuantity;
	o->lmax = d->SolverMaxIter;
	o->tol = d->SolverTolerance;
	o->nonlin_tol = d->NonLinearTolerance;
	return 0;
}

int femgpu_deck_transient_opts(const femgpu_deck *d, femgpu_transport_opts *o, femgpu_transient_opts *tr)
{
	static const char *const methods[] = { "Predictor1", "Predictor1_BDF", "Predictor1_TRBDF2", "Predictor2",
	                                       "Predictor2_BDF", "Predictor2_TRBDF2" };
	int m;
	if (!d || !o || !tr || d->equation != FEMGPU_EQ_TRANSIENT) return FEMGPU_E_ARG;
	femgpu_transport_default_opts(o);
	memset(tr, 0, sizeof *tr);
	if (!strcasecmp(d->MatrixVectorProductScheme, "CSR")) o->scheme = FEMGPU_CSR;
	else if (!strcasecmp(d->MatrixVectorProductScheme, "EDE")) o->scheme = FEMGPU_EDE;
	else if (!strcasecmp(d->MatrixVectorProductScheme, "EBE")) o->scheme = FEMGPU_EBE;
	else return FEMGPU_E_ARG;
	o->reorder = !strcasecmp(d->reordering, "SYMRCM") ? FEMGPU_REORDER_SYMRCM : FEMGPU_REORDER_NOT;
	if (strcasecmp(d->Scaling, "NOT") != 0 || strcasecmp(d->Solver, "GMRES") != 0) return FEMGPU_E_ARG;
	/* setPreconditioner.c:6-30, 79-89 */
	if (!strcasecmp(d->Preconditioner, "NOT")) o->precond = FEMGPU_PREC_NOT;
	else if (!strcasecmp(d->Preconditioner, "Diag")) o->precond = FEMGPU_PREC_DIAG;
	else if (ilu_level_of(d->Preconditioner) >= 0 && o->scheme == FEMGPU_CSR) {
		o->precond = FEMGPU_PREC_ILU0;
		o->ilu_level = ilu_level_of(d->Preconditioner);
	} else return FEMGPU_E_ARG;
	/* setStabilizationForm.c:6-98 */
	if (!strcasecmp(d->StabilizationForm, "SUPG")) tr->stab = FEMGPU_STAB_SUPG;
	else if (!strcasecmp(d->StabilizationForm, "DD")) tr->stab = FEMGPU_STAB_DD;
	else return FEMGPU_E_ARG;
	for (m = 0; m < 6 && strcasecmp(d->TimeIntegration, methods[m]) != 0; m++) {}
	if (m == 6 || (m >= FEMGPU_TI_PREDICTOR2 && tr->stab != FEMGPU_STAB_DD)) return FEMGPU_E_ARG;
	tr->method = m;
	if (!strcasecmp(d->ShockCapture, "CAU")) o->shock = FEMGPU_SHOCK_CAU;
	else if (!strcasecmp(d->ShockCapture, "YZBeta")) o->shock = FEMGPU_SHOCK_YZBETA;
	else if (!strcasecmp(d->ShockCapture, "CAUDD") && tr->stab == FEMGPU_STAB_DD) o->shock = FEMGPU_SHOCK_CAUDD;
	else return FEMGPU_E_ARG;
	if (!strcasecmp(d->h_Shock, "2sqrtArea")) o->hshock = FEMGPU_H_2SQRTAREA;
	else if (!strcasecmp(d->h_Shock, "Option1")) o->hshock = FEMGPU_H_OPTION1;
	else if (!strcasecmp(d->h_Shock, "Option2")) o->hshock = FEMGPU_H_OPTION2;
	else return FEMGPU_E_ARG;
	/* Criteria.c:3-20 */
	if (!strcasecmp(d->StopMulticorrection, "NORM")) tr->stop_norm = 1;
	else if (strcasecmp(d->StopMulticorrection, "ITERATION") != 0) return FEMGPU_E_ARG;
	if (!strcasecmp(d->StopAtSteadyState, "YES")) tr->steady_stop = 1;
	else if (strcasecmp(d->StopAtSteadyState, "NOT") != 0) return FEMGPU_E_ARG;
	o->kmax = d->KrylovBasisVectorsQuantity;
	o->lmax = d->LinearMaxIter;
	o->tol = d->SolverTolerance;
	o->nonlin_tol = d->NonLinearTolerance;
	tr->alpha = d->Alpha;
	tr->dt = d->DeltaT;
	tr->final_time = d->FinalTime;
	tr->max_corr = d->NonLinearMaxIter;
	tr->nonlin_tol = d->NonLinearTolerance;
	tr->time_tol = d->TimeIntegrationTolerance;
	return 0;
}

/* "AMG 2 NCL beta omega nr" -> the DPA parameters (amg_precond.c:26-40). */
int femgpu_deck_amg(const femgpu_deck *d, int *ncl, double *beta, double *omega, int *nr)
{
	int type = 0;
	if (!d || !ncl || !beta || !omega || !nr) return FEMGPU_E_ARG;
	if (sscanf(d->Preconditioner, "AMG %d %d %lf %lf %d", &type, ncl, beta, omega, nr) != 5 || type != 2)
		return FEMGPU_E_ARG;
	return 0;
}

static int trimmed_is(const char *s, const char *word)
{
	size_t n = strlen(word);
	if (strncasecmp(s, word, n) != 0) return 0;
	for (s += n; *s; s++) if (!isspace((unsigned char)*s)) return 0;
	return 1;
}

static int block_precond(const char *s, int csr, int *precond)
{
	if (trimmed_is(s, "NOT")) *precond = FEMGPU_PREC_NOT;
	else if (trimmed_is(s, "BlockDiag") && !csr) *precond = FEMGPU_PREC_BLOCKDIAG;
	else if (ilu_level_of(s) == 0 && csr) *precond = FEMGPU_PREC_ILU0;
	else if (!strncasecmp(s, "AMG", 3) && csr) *precond = FEMGPU_PREC_AMG;
	else return FEMGPU_E_ARG;
	return 0;
}

int femgpu_deck_euler_opts(const femgpu_deck *d, femgpu_euler_opts *o)
{
	if (!d || !o || d->equation != FEMGPU_EQ_EULER) return FEMGPU_E_ARG;
	femgpu_euler_default_opts(o);
	if (!strcasecmp(d->MatrixVectorProductScheme, "EBE")) o->scheme = FEMGPU_EBE;
	else if (!strcasecmp(d->MatrixVectorProductScheme, "CSR") && !strcasecmp(d->reordering, "NOT"))
		o->scheme = FEMGPU_CSR;
	else return FEMGPU_E_ARG;
	if (block_precond(d->Preconditioner, o->scheme == FEMGPU_CSR, &o->precond)) return FEMGPU_E_ARG;
	/* setStabilizationForm.c:6-75: SUPG with CAU or YZBeta, DD (with the
	 * Predictor1 loops: Build_M_K_F_DD_Transiente) with CAUDD or YZBeta;
	 * Y^-1 from the deck */
	if (!strcasecmp(d->StabilizationForm, "DD")) o->stab = FEMGPU_STAB_DD;
	else if (strcasecmp(d->StabilizationForm, "SUPG") != 0) return FEMGPU_E_ARG;
	if (!strcasecmp(d->ShockCapture, "YZBeta")) o->shock = FEMGPU_SHOCK_YZBETA;
	else if (o->stab == FEMGPU_STAB_DD && !strcasecmp(d->ShockCapture, "CAUDD")) o->shock = FEMGPU_SHOCK_CAUDD;
	else if (o->stab != FEMGPU_STAB_SUPG || strcasecmp(d->ShockCapture, "CAU") != 0) return FEMGPU_E_ARG;
	o->invY[0] = d->invY[0]; o->invY[1] = d->invY[1]; o->invY[2] = d->invY[2]; o->invY[3] = d->invY[3];
	/* setStabilizationForm.c:9-21: Predictor1, Predictor1_BDF, Predictor1_TRBDF2 */
	if (!strcasecmp(d->TimeIntegration, "Predictor1_BDF")) o->method = FEMGPU_TI_BDF;
	else if (!strcasecmp(d->TimeIntegration, "Predictor1_TRBDF2")) o->method = FEMGPU_TI_TRBDF2;
	else if (strcasecmp(d->TimeIntegration, "Predictor1") != 0) return FEMGPU_E_ARG;
	/* setScaling.c:6-27: "NOT", or "BlockScaling" with EBE storage only */
	if (!strcasecmp(d->Scaling, "BlockScaling") && o->scheme == FEMGPU_EBE) o->scaling = 1;
	else if (strcasecmp(d->Scaling, "NOT") != 0) return FEMGPU_E_ARG;
	o->dimensionless = !strcasecmp(d->Dimensionless, "YES");
	o->mach = d->Mach;
	o->alpha = d->Alpha;
	o->dt = d->DeltaT;
	o->stab_tol = d->StabilizationTolerance;
	o->kmax = d->KrylovBasisVectorsQuantity;
	o->lmax = d->LinearMaxIter;
	o->tol = d->SolverTolerance;
	o->ncorr = d->NonLinearMaxIter;
	return 0;
}

int femgpu_deck_ns_opts(const femgpu_deck *d, femgpu_ns_opts *o)
{
	if (!d || !o || d->equation != FEMGPU_EQ_NS) return FEMGPU_E_ARG;
	femgpu_ns_default_opts(o);
	if (!strcasecmp(d->MatrixVectorProductScheme, "EBE")) o->scheme = FEMGPU_EBE;
	else if (!strcasecmp(d->MatrixVectorProductScheme, "CSR")) o->scheme = FEMGPU_CSR;
	else return FEMGPU_E_ARG;
	if (block_precond(d->Preconditioner, o->scheme == FEMGPU_CSR, &o->precond)) return FEMGPU_E_ARG;
	if (strcasecmp(d->StabilizationForm, "MS") != 0) return FEMGPU_E_ARG;
	o->re = d->ReynoldsNumber;
	o->velmax = d->VelMax;
	o->kmax = d->KrylovBasisVectorsQuantity;
	o->lmax = d->LinearMaxIter;
	o->eta0 = d->SolverTolerance;
	o->eta_case = d->SolverToleranceCase;
	o->tol_nl = d->SolverToleranceNonLin;
	return 0;
}
