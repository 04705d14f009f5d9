/*
 * Reverse Cuthill-McKee ordering of a structurally symmetric CSR pattern,
 * with the exact tie-breaking of the reference's SYMRCM
 * (00_CommonFiles/Reordering/symrcm.c:4-242): a pseudo-peripheral start node
 * found by repeated breadth-first sweeps (find_starting_node, :357-488),
 * unvisited neighbours of each dequeued node pushed in ascending index order
 * onto a binary min-heap keyed by degree and popped into the queue
 * (H_insert / H_remove_min, :510-572), components started at the lowest
 * unvisited index, and the final order reversed (:231-235).  The heap and
 * neighbour order decide ties between equal degrees, so they are kept step
 * for step; the data structures around them are this library's own.
 *
 * Host setup code: runs once per pattern, before the device solve.
 */
#include <stdlib.h>
#include <string.h>
#include "femgpu_host.h"

typedef struct { int id, deg, dist; } rcm_entry;

static void heap_push(rcm_entry *H, int *h, rcm_entry o)
{
	int i = (*h)++;
	H[i] = o;
	while (i > 0) {
		int p = (i - 1) >> 1;
		if (!(H[i].deg < H[p].deg)) break;
		rcm_entry t = H[i]; H[i] = H[p]; H[p] = t;
		i = p;
	}
}

static rcm_entry heap_pop(rcm_entry *H, int *h)
{
	rcm_entry top = H[0];
	int size = --(*h), j = 0;
	H[0] = H[size];
	for (;;) {
		int l = 2 * j + 1, r = l + 1, m = j;
		if (l < size && H[l].deg < H[m].deg) m = l;
		if (r < size && H[r].deg < H[m].deg) m = r;
		if (m == j) break;
		rcm_entry t = H[j]; H[j] = H[m]; H[m] = t;
		j = m;
	}
	return top;
}

/* Neighbours of i in A + A^T, ascending, each once. */
static int neighbours(int i, const int *IA, const int *JA, const int *IT, const int *JT, int *out)
{
	int a = IA[i], ae = IA[i + 1], b = IT[i], be = IT[i + 1], m = 0;
	while (a < ae || b < be) {
		int v;
		if (a == ae) v = JT[b++];
		else if (b == be) v = JA[a++];
		else if (JA[a] <= JT[b]) { v = JA[a]; if (JA[a] == JT[b]) b++; a++; }
		else v = JT[b++];
		out[m++] = v;
	}
	return m;
}

int fgh_symrcm(int n, const int *IA, const int *JA, int *perm)
{
	int nnz = IA[n], i, k, maxdeg = 0, maxrow = 1, c = -1, qh = 0, qt = 0;
	int *IT = calloc((size_t)n + 1, sizeof(int)), *JT = malloc(sizeof(int) * ((size_t)nnz + 1));
	int *deg = calloc((size_t)n + 1, sizeof(int)), *fill = calloc((size_t)n + 1, sizeof(int));
	int *seen = calloc((size_t)n + 1, sizeof(int)), *seen2 = calloc((size_t)n + 1, sizeof(int));
	int *nb;
	rcm_entry *heap, *Q, *Q2;
	if (!IT || !JT || !deg || !fill || !seen || !seen2) return FEMGPU_E_NOMEM;

	for (k = 0; k < nnz; k++) fill[JA[k]]++;
	for (i = 0; i < n; i++) { IT[i + 1] = IT[i] + fill[i]; fill[i] = IT[i]; }
	for (i = 0; i < n; i++)
		for (k = IA[i]; k < IA[i + 1]; k++) JT[fill[JA[k]]++] = i;

	/* degrees of the symmetrised pattern (calc_degrees, symrcm.c:310-355) */
	for (i = 0; i < n; i++)
		for (k = IA[i]; k < IA[i + 1]; k++) {
			int col = JA[k], l, found = 0;
			if (++deg[col] > maxdeg) maxdeg = deg[col];
			if (col == i) continue;
			for (l = IA[col]; l < IA[col + 1] && JA[l] <= i; l++)
				if (JA[l] == i) { found = 1; break; }
			if (!found && ++deg[i] > maxdeg) maxdeg = deg[i];
		}
	if (maxdeg == 0) {
		for (i = 0; i < n; i++) perm[i] = i;
		free(IT); free(JT); free(deg); free(fill); free(seen); free(seen2);
		return 0;
	}
	for (i = 0; i < n; i++) {
		int len = IA[i + 1] - IA[i] + IT[i + 1] - IT[i];
		if (len > maxrow) maxrow = len;
	}
	nb = malloc(sizeof(int) * (size_t)maxrow);
	heap = malloc(sizeof(rcm_entry) * (size_t)(maxdeg > maxrow ? maxdeg : maxrow));
	Q = malloc(sizeof(rcm_entry) * ((size_t)n + 1));
	Q2 = malloc(sizeof(rcm_entry) * ((size_t)n + 1));

	do {
		rcm_entry x, v;
		int start, eccentricity = 0, h2, t2;
		for (start = 0; start < n && seen[start]; start++) ;
		/* pseudo-peripheral node: BFS from x, move x to the last, widest
		 * node found, repeat while the eccentricity grows */
		x.id = start; x.deg = deg[start]; x.dist = 0;
		memset(seen2, 0, sizeof(int) * (size_t)n);
		h2 = t2 = 0;
		Q2[t2++] = x;
		seen2[start] = 1;
		for (;;) {
			while (h2 != t2) {
				rcm_entry u = Q2[h2++];
				int m = neighbours(u.id, IA, JA, IT, JT, nb), q;
				if (u.dist > x.dist || (u.id != x.id && u.deg > x.deg)) x = u;
				for (q = 0; q < m; q++) {
					int r = nb[q];
					if (seen2[r]) continue;
					seen2[r] = 1;
					Q2[t2].id = r; Q2[t2].deg = deg[r]; Q2[t2].dist = u.dist + 1; t2++;
				}
			}
			if (eccentricity >= x.dist) break;
			eccentricity = x.dist;
			memset(seen2, 0, sizeof(int) * (size_t)n);
			seen2[x.id] = 1;
			x.dist = 0;
			h2 = t2 = 0;
			Q2[t2++] = x;
		}
		v.id = x.id; v.deg = deg[x.id]; v.dist = 0;
		seen[v.id] = 1;
		Q[qt++] = v;
		while (qh != qt) {
			int m, q, hs = 0;
			v = Q[qh++];
			perm[++c] = v.id;
			m = neighbours(v.id, IA, JA, IT, JT, nb);
			for (q = 0; q < m; q++) {
				int r = nb[q];
				if (seen[r]) continue;
				rcm_entry w = { r, deg[r], v.dist + 1 };
				heap_push(heap, &hs, w);
				seen[r] = 1;
			}
			while (hs > 0) Q[qt++] = heap_pop(heap, &hs);
		}
	} while (c + 1 < n);

	for (i = 0, k = n - 1; i < n / 2; i++, k--) { int t = perm[i]; perm[i] = perm[k]; perm[k] = t; }
	free(IT); free(JT); free(deg); free(fill); free(seen); free(seen2);
	free(nb); free(heap); free(Q); free(Q2);
	return 0;
}

/* Half bandwidth of a CSR pattern (reordering.c:310-332). */
int fgh_bandwidth(int n, const int *IA, const int *JA)
{
	int i, bl = 0, br = 0;
	for (i = 0; i < n; i++) {
		int lo = i - JA[IA[i]], hi = JA[IA[i + 1] - 1] - i;
		if (abs(lo) > bl) bl = lo;
		if (abs(hi) > br) br = hi;
	}
	return bl > br ? bl : br;
}

/* Dependency levels of the lower (lower != 0) or upper triangle of a CSR
 * pattern, and level-aligned tasks of at most 32 rows: rows[] lists the rows
 * by (level, index) -- descending index within a level for the upper sweep is
 * not needed, any order within a level is independent. */
int fgh_levels(int n, const int *IA, const int *JA, int lower, int *rows, int **task_out,
               int *ntask_out, int *nlev_out)
{
	int *lev = malloc(sizeof(int) * ((size_t)n + 1)), *cnt, *pos, *task;
	int i, k, nlev = 0, ntask = 0;
	if (!lev) return FEMGPU_E_NOMEM;
	if (lower) {
		for (i = 0; i < n; i++) {
			int l = 0;
			for (k = IA[i]; k < IA[i + 1] && JA[k] < i; k++)
				if (lev[JA[k]] + 1 > l) l = lev[JA[k]] + 1;
			lev[i] = l;
			if (l + 1 > nlev) nlev = l + 1;
		}
	} else {
		for (i = n - 1; i >= 0; i--) {
			int l = 0;
			for (k = IA[i]; k < IA[i + 1]; k++)
				if (JA[k] > i && lev[JA[k]] + 1 > l) l = lev[JA[k]] + 1;
			lev[i] = l;
			if (l + 1 > nlev) nlev = l + 1;
		}
	}
	cnt = calloc((size_t)nlev + 1, sizeof(int));
	pos = calloc((size_t)nlev + 1, sizeof(int));
	for (i = 0; i < n; i++) cnt[lev[i]]++;
	for (k = 0; k < nlev; k++) { pos[k + 1] = pos[k] + cnt[k]; ntask += (cnt[k] + 31) / 32; }
	for (i = 0; i < n; i++) rows[pos[lev[i]]++] = i;
	task = malloc(sizeof(int) * ((size_t)ntask + 1));
	ntask = 0;
	{
		int off = 0;
		for (k = 0; k < nlev; k++) {
			int q;
			for (q = 0; q < cnt[k]; q += 32) task[ntask++] = off + q;
			off += cnt[k];
		}
		task[ntask] = off;
	}
	free(lev); free(cnt); free(pos);
	*task_out = task;
	*ntask_out = ntask;
	*nlev_out = nlev;
	return 0;
}
