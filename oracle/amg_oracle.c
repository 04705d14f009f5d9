/*
 * Test infrastructure only -- the CPU oracle of the AMG V-cycle.
 *
 * dpa_Vcycle_precond (00_CommonFiles/Solvers_and_Preconditioners/CSR/AMG/
 * amg_dpa.c:485-506) over a given double-pairwise hierarchy, sequentially:
 * SOR_relax / SOR_relax_rev (amg_solvers.c:3-33), residual with mat_vec
 * (amg_util.c:44-48, amg_matrix.c:276-282), dpa_fine2coarse,
 * dpa_coarse2fine and dpa_coarse2fine_pure (amg_dpa.c:394-422).  Pinned
 * against the reference's own V-cycle on the golden fixtures
 * (tests/golden/amg_*.npz).
 */
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

static void sor(int n, const int *IA, const int *JA, const double *AA, const double *d, const double *f,
                double *u, double omega, int iter, int rev)
{
	for (int k = 0; k < iter; k++)
		for (int s = 0; s < n; s++) {
			int i = rev ? n - 1 - s : s;
			double sum = 0.0;
			for (int j = IA[i]; j < IA[i + 1]; j++)
				if (JA[j] != i) sum += AA[j] * u[JA[j]];
			u[i] += omega * ((f[i] - sum) / d[i] - u[i]);
		}
}

static void f2c(const int *m, const double *fine, int n, double *coarse)
{
	for (int i = 0, j = 0; i < n; i++)
		if (m[i] == -1) coarse[j++] = fine[i];
		else if (i < m[i]) coarse[j++] = fine[i] + fine[m[i]];
}

static void c2f(const int *m, const double *coarse, int n, double *fine, int pure)
{
	for (int i = 0, j = 0; i < n; i++)
		if (m[i] == -1) { if (pure) fine[i] = coarse[j++]; else fine[i] += coarse[j++]; }
		else if (i < m[i]) {
			if (pure) { fine[i] = coarse[j]; fine[m[i]] = coarse[j++]; }
			else { fine[i] += coarse[j]; fine[m[i]] += coarse[j++]; }
		}
}

int orc_amg_vcycle(int nlev, const int *n, const int *IA, const int *JA, const double *AA, const int *rm,
                   double omega, int nr, const double *q, double *z)
{
	const int **ia = calloc((size_t)nlev, sizeof(int *)), **ja = calloc((size_t)nlev, sizeof(int *));
	const int **m = calloc((size_t)nlev, sizeof(int *));
	const double **aa = calloc((size_t)nlev, sizeof(double *));
	double **f = calloc((size_t)nlev, sizeof(double *)), **u = calloc((size_t)nlev, sizeof(double *));
	double **d = calloc((size_t)nlev, sizeof(double *)), *r;
	size_t oi = 0, oj = 0, om = 0;
	int l, i;
	for (l = 0; l < nlev; l++) {
		ia[l] = IA + oi; ja[l] = JA + oj; aa[l] = AA + oj;
		oi += (size_t)n[l] + 1; oj += (size_t)ia[l][n[l]];
		if (l < nlev - 1) { m[l] = rm + om; om += (size_t)n[l] + 1; }
		f[l] = calloc((size_t)n[l] + 1, sizeof(double));
		u[l] = calloc((size_t)n[l] + 1, sizeof(double));
		d[l] = calloc((size_t)n[l] + 1, sizeof(double));
		for (i = 0; i < n[l]; i++)
			for (int k = ia[l][i]; k < ia[l][i + 1]; k++) if (ja[l][k] == i) d[l][i] = aa[l][k];
	}
	r = calloc((size_t)n[0] + 1, sizeof(double));
	memcpy(f[0], q, sizeof(double) * (size_t)n[0]);
	for (l = 0; l < nlev - 1; l += 2) {
		sor(n[l], ia[l], ja[l], aa[l], d[l], f[l], u[l], omega, nr, 0);
		for (i = 0; i < n[l]; i++) {
			double p = 0.0;
			for (int k = ia[l][i]; k < ia[l][i + 1]; k++) p += aa[l][k] * u[l][ja[l][k]];
			r[i] = p;
		}
		for (i = 0; i < n[l]; i++) r[i] = f[l][i] - r[i];
		f2c(m[l], r, n[l], f[l + 1]);
		f2c(m[l + 1], f[l + 1], n[l + 1], f[l + 2]);
		memset(u[l + 1], 0, sizeof(double) * (size_t)n[l + 1]);
		memset(u[l + 2], 0, sizeof(double) * (size_t)n[l + 2]);
	}
	sor(n[l], ia[l], ja[l], aa[l], d[l], f[l], u[l], omega, nr, 0);
	sor(n[l], ia[l], ja[l], aa[l], d[l], f[l], u[l], omega, nr, 1);
	for (; l > 0; l -= 2) {
		c2f(m[l - 1], u[l], n[l - 1], u[l - 1], 1);
		c2f(m[l - 2], u[l - 1], n[l - 2], u[l - 2], 0);
		sor(n[l - 2], ia[l - 2], ja[l - 2], aa[l - 2], d[l - 2], f[l - 2], u[l - 2], omega, nr, 1);
	}
	memcpy(z, u[0], sizeof(double) * (size_t)n[0]);
	for (l = 0; l < nlev; l++) { free(f[l]); free(u[l]); free(d[l]); }
	free(ia); free(ja); free(aa); free(m); free(f); free(u); free(d); free(r);
	return 0;
}

/* pgmres (pgmres.c:4-211) preconditioned by the V-cycle above, the way the
 * reference's drivers run it with "AMG 2 ...": AMG_precond_setup replaces F
 * by M^-1 F (amg_precond.c:92-97), csrmv is the product and AMG_precond the
 * preconditioner.  B [n] is overwritten by M^-1 B; returns the iterations. */
typedef struct {
	int nlev;
	const int *n, *IA, *JA, *rm;
	const double *AA;
	double omega;
	int nr;
} amg_ctx;

static void amg_mv(const void *c, double *in, double *out)
{
	const amg_ctx *a = c;
	for (int i = 0; i < a->n[0]; i++) {
		out[i] = 0;
		for (int j = a->IA[i]; j < a->IA[i + 1]; j++) out[i] += a->AA[j] * in[a->JA[j]];
	}
}

static void amg_pc(const void *c, double *in, double *out)
{
	const amg_ctx *a = c;
	double *t = malloc(sizeof(double) * ((size_t)a->n[0] + 1));
	memcpy(t, in, sizeof(double) * (size_t)a->n[0]);
	orc_amg_vcycle(a->nlev, a->n, a->IA, a->JA, a->AA, a->rm, a->omega, a->nr, t, out);
	free(t);
}

int orc_amg_gmres(int nlev, const int *n, const int *IA, const int *JA, const double *AA, const int *rm,
                  double omega, int nr, int kmax, int lmax, double tol, double *B, double *X)
{
	amg_ctx a = { nlev, n, IA, JA, rm, AA, omega, nr };
	amg_pc(&a, B, B);
	return orc_pgmres_cb(n[0], amg_mv, amg_pc, &a, kmax, lmax, tol, B, X);
}
