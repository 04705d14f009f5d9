/*
 * Symbolic ILU(p): the level-of-fill pattern of LEVEL_OF_FILL_lu
 * (00_CommonFiles/Solvers_and_Preconditioners/ilup.c:164-302), selected by
 * the deck's "ILU<p>" (CSR/ILUp_precond_setup.c:15).  Row i's entries are
 * found by a symbolic IKJ elimination: the matrix's own entries have level
 * 0; eliminating with pivot row k (lower entries taken leftmost first) adds
 * column c of U(k, :) at level lev(i, k) + lev(k, c) + 1 when that is at most
 * p, or lowers the level of an entry already present.
 *
 * The filled row is stored as the reference stores it: the lower part in
 * ascending columns (the leftmost-pivot selection sorts it), the diagonal,
 * then the upper part in the order the elimination found it -- the
 * matrix's own upper entries first, fill after.  The reference's backward
 * sweep (ILUp_precond.c:38-46) subtracts in that order, so the device sweep
 * programs, built from this layout, reproduce it bit for bit; the numeric
 * factorisation does not depend on the upper order (each entry of a row
 * receives at most one update per pivot row, pivots in ascending order).
 * Plain C.
 */
#include <stdlib.h>
#include <string.h>

#include "femgpu.h"
#include "femgpu_host.h"

int fgh_iluk_pattern(int n, const int *IA, const int *JA, int p, int **fIA_out, int **fJA_out, int **map_out)
{
	int *levls = malloc(sizeof(int) * (size_t)n), *jbuf = malloc(sizeof(int) * (size_t)n);
	int *iw = malloc(sizeof(int) * (size_t)n), *unz = calloc((size_t)n, sizeof(int));
	int **uja = calloc((size_t)n, sizeof(int *)), **ulvl = calloc((size_t)n, sizeof(int *));
	int *fIA = malloc(sizeof(int) * ((size_t)n + 1)), *fJA = NULL, *map = NULL;
	size_t cap = (size_t)IA[n] + (size_t)n + 16, nnz = 0;
	int i, j, rc = 0;
	fJA = malloc(sizeof(int) * cap);
	map = malloc(sizeof(int) * ((size_t)IA[n] + 1));
	if (!levls || !jbuf || !iw || !unz || !uja || !ulvl || !fIA || !fJA || !map) { rc = FEMGPU_E_NOMEM; goto out; }
	for (j = 0; j < n; j++) iw[j] = -1;
	fIA[0] = 0;
	for (i = 0; i < n; i++) {
		int incl = 0, incu = i, jpiv = -1, k, hasdiag = 0;
		for (j = IA[i]; j < IA[i + 1]; j++) {
			const int col = JA[j];
			if (col < i) { jbuf[incl] = col; levls[incl] = 0; iw[col] = incl++; }
			else if (col > i) { jbuf[incu] = col; levls[incu] = 0; iw[col] = incu++; }
			else hasdiag = 1;
		}
		if (!hasdiag) { rc = FEMGPU_E_ZERO_PIVOT; goto out; }
		while (++jpiv < incl) {
			int kmin, jmin = jpiv;
			k = jbuf[jpiv];
			kmin = k;
			for (j = jpiv + 1; j < incl; j++)
				if (jbuf[j] < kmin) { kmin = jbuf[j]; jmin = j; }
			if (jmin != jpiv) {                   /* leftmost pivot first */
				int t = levls[jpiv];
				jbuf[jpiv] = kmin; jbuf[jmin] = k;
				iw[kmin] = jpiv; iw[k] = jmin;
				levls[jpiv] = levls[jmin]; levls[jmin] = t;
				k = kmin;
			}
			for (j = 0; j < unz[k]; j++) {
				const int col = uja[k][j], it = ulvl[k][j] + levls[jpiv] + 1;
				int ip;
				if (it > p) continue;
				ip = iw[col];
				if (ip == -1) {
					if (col < i) { jbuf[incl] = col; levls[incl] = it; iw[col] = incl++; }
					else if (col > i) { jbuf[incu] = col; levls[incu] = it; iw[col] = incu++; }
				} else if (it < levls[ip]) levls[ip] = it;
			}
		}
		for (j = 0; j < incl; j++) iw[jbuf[j]] = -1;
		for (j = i; j < incu; j++) iw[jbuf[j]] = -1;
		/* this row's upper part and its levels, for the rows below */
		unz[i] = incu - i;
		if (unz[i]) {
			uja[i] = malloc(sizeof(int) * (size_t)unz[i]);
			ulvl[i] = malloc(sizeof(int) * (size_t)unz[i]);
			if (!uja[i] || !ulvl[i]) { rc = FEMGPU_E_NOMEM; goto out; }
			memcpy(uja[i], jbuf + i, sizeof(int) * (size_t)unz[i]);
			memcpy(ulvl[i], levls + i, sizeof(int) * (size_t)unz[i]);
		}
		/* the filled row: lower, diagonal, upper */
		if (nnz + (size_t)incl + 1 + (size_t)unz[i] > cap) {
			int *b;
			cap = 2 * cap + (size_t)incl + (size_t)unz[i] + 1;
			b = realloc(fJA, sizeof(int) * cap);
			if (!b) { rc = FEMGPU_E_NOMEM; goto out; }
			fJA = b;
		}
		memcpy(fJA + nnz, jbuf, sizeof(int) * (size_t)incl);
		nnz += (size_t)incl;
		fJA[nnz++] = i;
		memcpy(fJA + nnz, jbuf + i, sizeof(int) * (size_t)unz[i]);
		nnz += (size_t)unz[i];
		if (nnz > 0x7fffffff) { rc = FEMGPU_E_MESH; goto out; }
		fIA[i + 1] = (int)nnz;
		/* where each of the matrix's entries sits in the filled row */
		for (j = IA[i]; j < IA[i + 1]; j++) {
			int q;
			for (q = fIA[i]; q < fIA[i + 1] && fJA[q] != JA[j]; q++) ;
			map[j] = q;
		}
	}
out:
	if (uja) for (i = 0; i < n; i++) { free(uja[i]); free(ulvl[i]); }
	free(levls); free(jbuf); free(iw); free(unz); free(uja); free(ulvl);
	if (rc) { free(fIA); free(fJA); free(map); return rc; }
	*fIA_out = fIA;
	*fJA_out = fJA;
	*map_out = map;
	return 0;
}

int femgpu_iluk_pattern(int n, const int *IA, const int *JA, int p, int *fIA, int *fJA, int cap)
{
	int *a = NULL, *b = NULL, *m = NULL, rc, nnz;
	if (n <= 0 || !IA || !JA || p < 0 || IA[0] != 0) return FEMGPU_E_ARG;
	for (rc = 0; rc < n; rc++) {
		int k;
		if (IA[rc + 1] < IA[rc]) return FEMGPU_E_ARG;
		for (k = IA[rc]; k < IA[rc + 1]; k++) if (JA[k] < 0 || JA[k] >= n) return FEMGPU_E_ARG;
	}
	rc = fgh_iluk_pattern(n, IA, JA, p, &a, &b, &m);
	if (rc) return rc;
	nnz = a[n];
	if (fIA) memcpy(fIA, a, sizeof(int) * ((size_t)n + 1));
	if (fJA) {
		if (cap < nnz) { free(a); free(b); free(m); return FEMGPU_E_ARG; }
		memcpy(fJA, b, sizeof(int) * (size_t)nnz);
	}
	free(a); free(b); free(m);
	return nnz;
}
