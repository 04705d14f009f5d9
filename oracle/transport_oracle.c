/*
 * Test infrastructure only -- CPU oracle for the steady 2D transport path.
 * A restatement, in this project's own code, of the reference algorithm
 * (mod-comp-ufes/FEM_CODES); each function names the reference lines it
 * follows.  Floating-point expressions keep the reference's evaluation order
 * so that, compiled without contraction or reassociation, results are
 * bit-identical to the reference's own sources (checked against the golden
 * fixtures in tests/golden/).  Never linked into the product.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <time.h>

/* Wall-clock phases of the last orc_transport_run (seconds): set-up, then
 * build, precond_setup and solve summed over the Picard iterations. */
static double g_times[4];
#define ORC_MAX_STEPS 256
static double g_step[ORC_MAX_STEPS];    /* wall time of each Picard iteration */

/* To-solution variant of the CPU baseline (no reference counterpart): when
 * g_refine_to > 0, every Picard solve is followed by host-checked iterative
 * refinement with the reference's own solver -- r = F - A u in FP64, the
 * left-preconditioned correction system (M^-1 A) d = M^-1 r solved by the same
 * pgmres (at the loosest tolerance expected to reach the target, no tighter
 * than g_refine_tol), u += d -- until the true relative residual
 * ||F - A u|| / ||F|| is at most g_refine_to (or g_refine_max rounds).  The
 * reference's own stop (pgmres.c:49-53,184) bounds only the preconditioned
 * residual, which at 2048x1024 leaves a true residual near 0.5. */
static double g_refine_to = 0.0, g_refine_tol = 1e-12;
static int g_refine_max = 40;
/* Refinement starts at Picard step g_refine_from (0-based; earlier steps stop
 * where the reference stops), and once g_refine_budget seconds have gone into
 * refined steps the Picard loop ends after the current step (0: no bound). */
static int g_refine_from = 0;
static double g_refine_budget = 0.0;
static double g_refine_res[ORC_MAX_STEPS];   /* true residual after each Picard solve */
static int g_refine_its[ORC_MAX_STEPS];      /* refinement rounds of each Picard solve */

void orc_set_refine(double to, double tol, int maxrounds)
{
	g_refine_to = to;
	g_refine_tol = tol > 0 ? tol : 1e-12;
	g_refine_max = maxrounds > 0 ? maxrounds : 40;
	g_refine_from = 0;
	g_refine_budget = 0.0;
}

void orc_set_refine_window(int from, double budget_s)
{
	g_refine_from = from > 0 ? from : 0;
	g_refine_budget = budget_s > 0 ? budget_s : 0.0;
}

void orc_get_refine(double *res, int *rounds, int n)
{
	int i;
	for (i = 0; i < n && i < ORC_MAX_STEPS; i++) { res[i] = g_refine_res[i]; rounds[i] = g_refine_its[i]; }
}

static double now_s(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

void orc_get_times(double *t)
{
	int i;
	for (i = 0; i < 4; i++) t[i] = g_times[i];
}

void orc_get_step_times(double *t, int n)
{
	int i;
	for (i = 0; i < n && i < ORC_MAX_STEPS; i++) t[i] = g_step[i];
}

/* ------------------------------------------------------------------------ */
/* Numbering: Preprocess.c:73-81 (id = neq++ for Type >= 1), Fill_LM.c:7-19  */
/* (prescribed vertices map to the dump equation neq).                       */
int orc_fill_lm(int nnodes, const int *node_type, int nel, const int *vert,
                int *node_id, int *lm)
{
	int neq = 0, i, j;
	for (i = 0; i < nnodes; i++)
		node_id[i] = (node_type[i] >= 1) ? neq++ : -1;
	for (i = 0; i < nel; i++)
		for (j = 0; j < 3; j++) {
			int v = vert[3*i+j];
			lm[3*i+j] = (node_type[v] >= 1) ? node_id[v] : neq;
		}
	return neq;
}

/* Small helpers for per-row sorted unique column sets. */
static int cmp_int(const void *a, const void *b)
{
	int x = *(const int *)a, y = *(const int *)b;
	return (x > y) - (x < y);
}

static int sort_unique(int *v, int n)
{
	int i, m = 0;
	qsort(v, (size_t)n, sizeof(int), cmp_int);
	for (i = 0; i < n; i++)
		if (m == 0 || v[m-1] != v[i]) v[m++] = v[i];
	return m;
}

static int find_in_row(const int *JA, int lo, int hi, int col)
{
	while (lo < hi) {
		int mid = (lo + hi) >> 1;
		if (JA[mid] < col) lo = mid + 1; else hi = mid;
	}
	return lo;
}

/* ------------------------------------------------------------------------ */
/* csr_Initialization.c:18-123: row I holds every equation J sharing an      */
/* element with I (both unknown), ascending and unique (csr_List_insertA     */
/* keeps each row list sorted and drops duplicates); CSR_by_Element[K][3a+b] */
/* is the position of (lm[a], lm[b]) or nnzero when either is prescribed.    */
int orc_csr_pattern(int neq, int nel, const int *lm, int *IA, int *JA, int *sbe)
{
	int *cnt = calloc((size_t)neq + 1, sizeof(int));
	int *start, *buf, *ulen, i, a, b, K, nnz = 0;
	for (K = 0; K < nel; K++)
		for (a = 0; a < 3; a++)
			if (lm[3*K+a] != neq) cnt[lm[3*K+a]] += 3;
	start = malloc(((size_t)neq + 1) * sizeof(int));
	start[0] = 0;
	for (i = 0; i < neq; i++) start[i+1] = start[i] + cnt[i];
	buf = malloc((size_t)start[neq] * sizeof(int) + 1);
	memset(cnt, 0, ((size_t)neq + 1) * sizeof(int));
	for (K = 0; K < nel; K++)
		for (a = 0; a < 3; a++) {
			int I = lm[3*K+a];
			if (I == neq) continue;
			for (b = 0; b < 3; b++)
				if (lm[3*K+b] != neq) buf[start[I] + cnt[I]++] = lm[3*K+b];
		}
	ulen = malloc(((size_t)neq + 1) * sizeof(int));
	for (i = 0; i < neq; i++) {
		ulen[i] = sort_unique(buf + start[i], cnt[i]);
		nnz += ulen[i];
	}
	if (IA) {
		IA[0] = 0;
		for (i = 0; i < neq; i++) {
			IA[i+1] = IA[i] + ulen[i];
			memcpy(JA + IA[i], buf + start[i], (size_t)ulen[i] * sizeof(int));
		}
		for (K = 0; K < nel; K++)
			for (a = 0; a < 3; a++)
				for (b = 0; b < 3; b++) {
					int I = lm[3*K+a], J = lm[3*K+b];
					sbe[9*K+3*a+b] = (I == neq || J == neq) ? nnz :
						find_in_row(JA, IA[I], IA[I+1], J);
				}
	}
	free(cnt); free(start); free(buf); free(ulen);
	return nnz;
}

/* ------------------------------------------------------------------------ */
/* SYMRCM: symrcm.c:4-236 (Cuthill-McKee from a pseudo-peripheral node with  */
/* a degree-keyed binary min-heap for each node's unvisited neighbours, then */
/* reversal).  The heap operations and the neighbour visiting order (merge   */
/* of row i of A and of A^T, ascending) are kept as the reference has them,  */
/* because they decide ties between equal degrees.                           */
typedef struct { int id, deg, dist; } rcm_node;

static void heap_push(rcm_node *H, int *h, rcm_node o)      /* symrcm.c:510-531 */
{
	int i = (*h)++;
	H[i] = o;
	while (i > 0) {
		int p = (i - 1) >> 1;
		if (H[i].deg < H[p].deg) { rcm_node t = H[i]; H[i] = H[p]; H[p] = t; i = p; }
		else break;
	}
}

static rcm_node heap_pop(rcm_node *H, int *h)               /* symrcm.c:535-572 */
{
	rcm_node r = H[0];
	int j = 0, size;
	H[0] = H[--(*h)];
	size = *h;
	for (;;) {
		int l = 2*j + 1, rr = 2*j + 2, s;
		s = (l < size && H[l].deg < H[j].deg) ? l : j;
		if (rr < size && H[rr].deg < H[s].deg) s = rr;
		if (s == j) break;
		{ rcm_node t = H[j]; H[j] = H[s]; H[s] = t; }
		j = s;
	}
	return r;
}

/* Neighbours of i: the union of row i of A (IA/JA) and of A^T (IT/JT) in
 * ascending order, each once (symrcm.c:116-176). Returns their count. */
static int rcm_neighbours(int i, const int *IA, const int *JA, const int *IT, const int *JT, int *out)
{
	int j1 = IA[i], j2 = IT[i], m = 0;
	while (j1 < IA[i+1] || j2 < IT[i+1]) {
		if (j1 == IA[i+1]) out[m++] = JT[j2++];
		else if (j2 == IT[i+1]) out[m++] = JA[j1++];
		else {
			int r1 = JA[j1], r2 = JT[j2];
			if (r1 <= r2) { out[m++] = r1; j1++; if (r1 == r2) j2++; }
			else { out[m++] = r2; j2++; }
		}
	}
	return m;
}

/* find_starting_node, symrcm.c:357-488 */
static int rcm_start(int n, const int *IA, const int *JA, const int *IT, const int *JT,
                     const int *D, int start, rcm_node *Q, int *visit, int *nb)
{
	int qh = 0, qt = 0, max_dist = 0, i;
	rcm_node x = { start, D[start], 0 };
	memset(visit, 0, (size_t)n * sizeof(int));
	Q[qt++] = x;
	visit[start] = 1;
	for (;;) {
		while (qh != qt) {
			rcm_node v = Q[qh++];
			int m, q;
			if (v.dist > x.dist || (v.id != x.id && v.deg > x.deg)) x = v;
			m = rcm_neighbours(v.id, IA, JA, IT, JT, nb);
			for (q = 0; q < m; q++) {
				int r = nb[q];
				if (!visit[r]) {
					rcm_node w = { r, D[r], v.dist + 1 };
					Q[qt++] = w;
					visit[r] = 1;
				}
			}
		}
		if (max_dist < x.dist) {
			max_dist = x.dist;
			for (i = 0; i < n; i++) visit[i] = 0;
			visit[x.id] = 1;
			x.dist = 0;
			qt = qh = 0;
			Q[qt++] = x;
		} else break;
	}
	return x.id;
}

void orc_symrcm(int n, const int *IA, const int *JA, int *perm)
{
	int nnz = IA[n], i, k, max_deg = 0, c = -1, qh = 0, qt = 0, s;
	int *IT = calloc((size_t)n + 1, sizeof(int)), *JT = malloc((size_t)nnz * sizeof(int) + 1);
	int *D = calloc((size_t)n, sizeof(int)), *w = calloc((size_t)n + 1, sizeof(int));
	int *visit, *visit2, *nb;
	rcm_node *S, *Q, *Q2;

	/* transpose, symrcm.c:277-308 */
	for (k = 0; k < nnz; k++) w[JA[k]]++;
	for (i = 0; i < n; i++) { IT[i+1] = IT[i] + w[i]; w[i] = IT[i]; }
	for (i = 0; i < n; i++)
		for (k = IA[i]; k < IA[i+1]; k++) JT[w[JA[k]]++] = i;

	/* calc_degrees, symrcm.c:310-355 */
	for (i = 0; i < n; i++)
		for (k = IA[i]; k < IA[i+1]; k++) {
			int col = JA[k], l, found = 0;
			if (++D[col] > max_deg) max_deg = D[col];
			if (col == i) continue;
			for (l = IA[col]; l < IA[col+1]; l++) {
				if (JA[l] == i) { found = 1; break; }
				if (JA[l] > i) break;
			}
			if (!found && ++D[i] > max_deg) max_deg = D[i];
		}
	if (max_deg == 0) {
		for (i = 0; i < n; i++) perm[i] = i;
		free(IT); free(JT); free(D); free(w);
		return;
	}
	S = malloc((size_t)max_deg * sizeof(rcm_node));
	Q = malloc(((size_t)n + 1) * sizeof(rcm_node));
	Q2 = malloc(((size_t)n + 1) * sizeof(rcm_node));
	visit = calloc((size_t)n, sizeof(int));
	visit2 = calloc((size_t)n, sizeof(int));
	{
		int mx = 1;
		for (i = 0; i < n; i++) {
			int len = IA[i+1] - IA[i] + IT[i+1] - IT[i];
			if (len > mx) mx = len;
		}
		nb = malloc((size_t)mx * sizeof(int));
	}
	do {
		rcm_node v;
		for (i = 0; i < n; i++) if (!visit[i]) break;
		v.id = rcm_start(n, IA, JA, IT, JT, D, i, Q2, visit2, nb);
		v.deg = D[v.id];
		v.dist = 0;
		visit[v.id] = 1;
		Q[qt++] = v;
		while (qh != qt) {
			v = Q[qh++];
			perm[++c] = v.id;
			int m = rcm_neighbours(v.id, IA, JA, IT, JT, nb), q;
			s = 0;
			for (q = 0; q < m; q++) {
				int r = nb[q];
				if (!visit[r]) {
					rcm_node nw = { r, D[r], v.dist + 1 };
					heap_push(S, &s, nw);
					visit[r] = 1;
				}
			}
			while (s > 0) Q[qt++] = heap_pop(S, &s);
		}
	} while (c + 1 < n);
	/* reverse, symrcm.c:232-235 */
	for (i = 0, k = n - 1; i <= n/2 - 1; i++, k--) { int t = perm[i]; perm[i] = perm[k]; perm[k] = t; }
	free(IT); free(JT); free(D); free(w); free(S); free(Q); free(Q2); free(visit); free(visit2); free(nb);
}

/* MATRIX_bandwidth, reordering.c:310-332 */
int orc_bandwidth(int n, const int *IA, const int *JA)
{
	int i, bl = 0, br = 0;
	for (i = 0; i < n; i++) {
		if (abs(i - JA[IA[i]]) > bl) bl = i - JA[IA[i]];
		if (abs(JA[IA[i+1]-1] - i) > br) br = JA[IA[i+1]-1] - i;
	}
	return bl > br ? bl : br;
}

/* Row then column permutation (reordering.c:238-308: new row i = old row
 * perm[i]; columns renumbered and sorted within each row) and the slot /
 * node-id remapping of csr_Initialization.c:144-179. */
typedef struct { int col, old; } col_slot;
static int cmp_slot(const void *a, const void *b)
{
	const col_slot *x = a, *y = b;
	return (x->col > y->col) - (x->col < y->col);
}

int orc_reorder_csr(int neq, int nnz, int *IA, int *JA, const int *perm,
                    int nel, int *sbe, int nnodes, int *node_id)
{
	int *inv = malloc((size_t)neq * sizeof(int)), *nIA = malloc(((size_t)neq + 1) * sizeof(int));
	int *nJA = malloc((size_t)nnz * sizeof(int) + 1), *invslot = malloc((size_t)nnz * sizeof(int) + 1);
	col_slot *row = malloc(((size_t)neq + 1) * sizeof(col_slot));
	int i, k, m;
	for (i = 0; i < neq; i++) inv[perm[i]] = i;
	nIA[0] = 0;
	for (i = 0; i < neq; i++) {
		int o = perm[i];
		m = 0;
		for (k = IA[o]; k < IA[o+1]; k++) { row[m].col = inv[JA[k]]; row[m].old = k; m++; }
		qsort(row, (size_t)m, sizeof(col_slot), cmp_slot);
		for (k = 0; k < m; k++) { nJA[nIA[i] + k] = row[k].col; invslot[row[k].old] = nIA[i] + k; }
		nIA[i+1] = nIA[i] + m;
	}
	memcpy(IA, nIA, ((size_t)neq + 1) * sizeof(int));
	memcpy(JA, nJA, (size_t)nnz * sizeof(int));
	for (k = 0; k < 9*nel; k++) sbe[k] = (sbe[k] < nnz) ? invslot[sbe[k]] : nnz;
	for (k = 0; k < nnodes; k++) if (node_id[k] != -1) node_id[k] = inv[node_id[k]];
	free(inv); free(nIA); free(nJA); free(invslot); free(row);
	return orc_bandwidth(neq, IA, JA);
}

/* ------------------------------------------------------------------------ */
/* Edge structure, ede_Initialization.c:16-170.                             */
static void ede_sort3(const int *l, int *I, int *ord)
{
	if (l[0] < l[1] && l[0] < l[2]) {
		if (l[1] < l[2]) { ord[0] = 0; ord[1] = 1; ord[2] = 2; }
		else             { ord[0] = 0; ord[1] = 2; ord[2] = 1; }
	} else if (l[1] < l[2]) {
		if (l[0] < l[2]) { ord[0] = 1; ord[1] = 0; ord[2] = 2; }
		else             { ord[0] = 1; ord[1] = 2; ord[2] = 0; }
	} else {
		if (l[0] < l[1]) { ord[0] = 2; ord[1] = 0; ord[2] = 1; }
		else             { ord[0] = 2; ord[1] = 1; ord[2] = 0; }
	}
	I[0] = l[ord[0]]; I[1] = l[ord[1]]; I[2] = l[ord[2]];
}

int orc_ede_pattern(int neq, int nel, const int *lm, int *lm2, int *ebe, int *order)
{
	int rows = neq + 1, K, i, total = 0, nedge;
	int *cnt = calloc((size_t)rows, sizeof(int)), *start = malloc(((size_t)rows + 1) * sizeof(int));
	int *buf, *ulen = malloc((size_t)rows * sizeof(int)), *ind = malloc(((size_t)rows + 1) * sizeof(int));
	for (K = 0; K < nel; K++) {
		int I[3], o[3];
		ede_sort3(lm + 3*K, I, o);
		cnt[I[0]] += 2; cnt[I[1]] += 1;
	}
	start[0] = 0;
	for (i = 0; i < rows; i++) start[i+1] = start[i] + cnt[i];
	buf = malloc((size_t)start[rows] * sizeof(int) + 1);
	memset(cnt, 0, (size_t)rows * sizeof(int));
	for (K = 0; K < nel; K++) {
		int I[3], o[3];
		ede_sort3(lm + 3*K, I, o);
		buf[start[I[0]] + cnt[I[0]]++] = I[1];
		buf[start[I[0]] + cnt[I[0]]++] = I[2];
		buf[start[I[1]] + cnt[I[1]]++] = I[2];
	}
	for (i = 0; i < rows; i++) { ulen[i] = sort_unique(buf + start[i], cnt[i]); total += ulen[i]; }
	/* The reference counts the single (neq, neq) dump edge and then drops one
	 * (ede_Initialization.c:103); without such an edge its edge arrays would
	 * overflow, so that case is refused here. */
	if (ulen[neq] != 1) { free(cnt); free(start); free(buf); free(ulen); free(ind); return -1; }
	nedge = total - 1;
	ind[0] = 0;
	for (i = 0; i < rows; i++) ind[i+1] = ind[i] + (i < neq ? ulen[i] : 0);
	if (lm2) {
		for (i = 0; i < neq; i++) {
			int k;
			for (k = 0; k < ulen[i]; k++) { lm2[2*(ind[i]+k)] = i; lm2[2*(ind[i]+k)+1] = buf[start[i]+k]; }
		}
		for (K = 0; K < nel; K++) {
			int I[3], o[3];
			ede_sort3(lm + 3*K, I, o);
			ebe[3*K+0] = ind[I[0]] + find_in_row(buf + start[I[0]], 0, ulen[I[0]], I[1]);
			ebe[3*K+1] = ind[I[0]] + find_in_row(buf + start[I[0]], 0, ulen[I[0]], I[2]);
			ebe[3*K+2] = ind[I[1]] + find_in_row(buf + start[I[1]], 0, ulen[I[1]], I[2]);
			order[3*K] = o[0]; order[3*K+1] = o[1]; order[3*K+2] = o[2];
		}
	}
	free(cnt); free(start); free(buf); free(ulen); free(ind);
	return nedge;
}

/* ------------------------------------------------------------------------ */
/* Shock-capturing length scales: h_shock_2sqrtArea.c:3-8,                  */
/* h_shock_sqrtArea.c:3-61, h_shock_Option1.c:3-19, h_shock_Option2.c:3-19.  */
static double h_shock(const orc_transport *t, int e, double bx, double by, double u1, double u2,
                      double u3, double y23, double y31, double y12, double x32, double x13,
                      double x21, double Area)
{
	double P1, P2, P3;
	switch (t->hshock) {
	case ORC_H_SQRTAREA:
		/* Every branch of h_shock_sqrtArea.c:25-57 assigns the same value. */
		return 2*sqrt(fabs(Area));
	case ORC_H_OPTION1: {
		double a1, a2, ng;
		P1 = fabs(u1*y23*y23 + u2*y31*y23 + u3*y12*y23 + u1*x32*x32 + u2*x13*x32 + u3*x21*x32);
		P2 = fabs(u1*y23*y31 + u2*y31*y31 + u3*y12*y31 + u1*x32*x13 + u2*x13*x13 + u3*x21*x13);
		P3 = fabs(u1*y23*y12 + u2*y31*y12 + u3*y12*y12 + u1*x32*x21 + u2*x13*x21 + u3*x21*x21);
		a1 = y23*u1 + y31*u2 + y12*u3;
		a2 = x32*u1 + x13*u2 + x21*u3;
		ng = sqrt(a1*a1 + a2*a2);
		return (P1+P2+P3 >= 1e-12) ? 4*Area*ng/(P1 + P2 + P3) : 0;
	}
	case ORC_H_OPTION2: {
		double nb;
		P1 = fabs(bx*y23 + by*x32);
		P2 = fabs(bx*y31 + by*x13);
		P3 = fabs(bx*y12 + by*x21);
		nb = sqrt(bx*bx + by*by);
		return (P1+P2+P3 >= 1e-12) ? 4*Area*nb/(P1 + P2 + P3) : 0;
	}
	default:
		return sqrt(fabs(2*Area));
	}
}

/* CAU_ShockCapture.c:3-30 and YZBeta_ShockCapture.c:3-27. */
static double shock_capture(int kind, double kx, double ky, double bx, double by, double g,
                            double ue1, double ue2, double ue3, double ueb, double feb,
                            double y23, double y31, double y12, double x32, double x13,
                            double x21, double invArea, double h)
{
	double BetaGradu, Ru, G0, G1, nG;
	BetaGradu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
	Ru = BetaGradu + g*ueb - feb;
	G0 = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
	G1 = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
	nG = sqrt(G0*G0 + G1*G1);
	if (kind == ORC_YZBETA) {
		double nRu = fabs(Ru), nu = fabs(ueb);
		if (nu >= 1e-12 && nG >= 1e-12)
			return 0.25*h*nRu/nG + 0.125*h*h*nRu/nu;
		return 0;
	} else {
		double third = 1./3., bxp, byp, kp, nbp, Pee;
		if (!(nG > 0)) return 0;
		bxp = BetaGradu*G0/(nG*nG);
		byp = BetaGradu*G1/(nG*nG);
		kp = bxp*bxp*kx + byp*byp*ky;
		nbp = sqrt(bxp*bxp + byp*byp);
		Pee = 0.5*h*nbp*nbp*nbp/kp;
		if (third*Pee < 0.7) return 0.5*h*third*Pee*fabs(Ru)/nG;
		return 0.5*h*0.7*fabs(Ru)/nG;
	}
}

/* ------------------------------------------------------------------------ */
/* Build_K_F_SUPG.c:5-163 with eval_U.c:12-22, F_assembly.c:3-35 and the    */
/* assembly pointers ebe_assembly.c:3-18, ede_assembly.c:3-35,               */
/* csr_assembly.c:3-24.                                                      */
void orc_build_supg(const orc_transport *t, const double *u, double *A, double *F)
{
	const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
	const double kx = t->k, ky = t->k, gamma = t->gamma;
	int E, J;
	double *U = malloc((size_t)t->nnodes * sizeof(double));

	/* setzeros.c:3-19 */
	if (t->scheme == ORC_EBE) memset(A, 0, sizeof(double) * 9 * (size_t)t->nel);
	else if (t->scheme == ORC_EDE) memset(A, 0, sizeof(double) * 4 * ((size_t)t->nedge + 1));
	else memset(A, 0, sizeof(double) * ((size_t)t->nnz + 1));
	for (J = 0; J < t->nnodes; J++)
		U[J] = (t->node_id[J] >= 0) ? u[t->node_id[J]] : t->upresc[J];
	for (J = 0; J < t->neq; J++) F[J] = 0;

	for (E = 0; E < t->nel; E++) {
		int J1 = t->vert[3*E], J2 = t->vert[3*E+1], J3 = t->vert[3*E+2];
		double X0 = t->x[J1], X1 = t->x[J2], X2 = t->x[J3];
		double Y0 = t->y[J1], Y1 = t->y[J2], Y2 = t->y[J3];
		double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
		double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
		double TwoA = x21*y31 - x13*y12, Area = 0.5*TwoA, invArea = 1.0/Area;
		double h = sqrt(fabs(TwoA));
		double bx = t->beta[2*E], by = t->beta[2*E+1];
		double norm = sqrt(bx*bx + by*by), tau = (norm > 0) ? 0.5*h/norm : 0;
		double fe1 = t->fsrc[3*E], fe2 = t->fsrc[3*E+1], fe3 = t->fsrc[3*E+2];
		double feb = third*(fe1+fe2+fe3);
		double ue1 = U[J1], ue2 = U[J2], ue3 = U[J3], ueb = third*(ue1 + ue2 + ue3);
		double D12, D13, D23, C11, C12, C13, R11, R12, Cpg12, Cpg13, Cpg23, Rpg11, Rpg21, Rpg31;
		double hs, Eu, Csc12, Csc13, Csc23, ke[3][3], Fe[3];
		const int jv[3] = { J1, J2, J3 };
		const double Xv[3] = { X0, X1, X2 }, Yv[3] = { Y0, Y1, Y2 };
		int a, b;

		D12 = 0.25*invArea*((kx * y23 * y31) + (ky * x32 * x13));
		D13 = 0.25*invArea*((kx * y23 * y12) + (ky * x32 * x21));
		D23 = 0.25*invArea*((kx * y31 * y12) + (ky * x13 * x21));
		C11 = sixth*(bx*y23 + by*x32);
		C12 = sixth*(bx*y31 + by*x13);
		C13 = sixth*(bx*y12 + by*x21);
		R11 = sixth*(gamma*Area);
		R12 = twelfth*(gamma * Area);
		Cpg12 = 0.25*invArea*tau * (y23*(bx*bx*y31 + bx*by*x13) + x32*(bx*by*y31 + by*by*x13));
		Cpg13 = 0.25*invArea*tau * (y23*(bx*bx*y12 + bx*by*x21) + x32*(bx*by*y12 + by*by*x21));
		Cpg23 = 0.25*invArea*tau * (y31*(bx*bx*y12 + bx*by*x21) + x13*(bx*by*y12 + by*by*x21));
		Rpg11 = sixth*tau*gamma * (bx*y23 + by*x32);
		Rpg21 = sixth*tau*gamma * (bx*y31 + by*x13);
		Rpg31 = sixth*tau*gamma * (bx*y12 + by*x21);

		hs = h_shock(t, E, bx, by, ue1, ue2, ue3, y23, y31, y12, x32, x13, x21, Area);
		Eu = shock_capture(t->shock, kx, ky, bx, by, gamma, ue1, ue2, ue3, ueb, feb,
		                   y23, y31, y12, x32, x13, x21, invArea, hs);
		Csc12 = Eu*0.25*invArea*(y23*y31 + x32*x13);
		Csc13 = Eu*0.25*invArea*(y23*y12 + x32*x21);
		Csc23 = Eu*0.25*invArea*(y31*y12 + x13*x21);

		ke[0][0] = -(D12 + D13) + C11 - (Cpg12 + Cpg13) + R11 + Rpg11 - (Csc12 + Csc13);
		ke[0][1] = D12 + C12 + Cpg12 + R12 + Rpg11 + Csc12;
		ke[0][2] = D13 + C13 + Cpg13 + R12 + Rpg11 + Csc13;
		ke[1][0] = D12 + C11 + Cpg12 + R12 + Rpg21 + Csc12;
		ke[1][1] = -(D12 + D23) + C12 - (Cpg12 + Cpg23) + R11 + Rpg21 - (Csc12 + Csc23);
		ke[1][2] = D23 + C13 + Cpg23 + R12 + Rpg21 + Csc23;
		ke[2][0] = D13 + C11 + Cpg13 + R12 + Rpg31 + Csc13;
		ke[2][1] = D23 + C12 + Cpg23 + R12 + Rpg31 + Csc23;
		ke[2][2] = -(D13 + D23) + C13 - (Cpg13 + Cpg23) + R11 + Rpg31 - (Csc13 + Csc23);

		Fe[0] = Area*twelfth*(2*fe1 +  fe2  +  fe3 ) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32);
		Fe[1] = Area*twelfth*(  fe1 + 2*fe2 +  fe3 ) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13);
		Fe[2] = Area*twelfth*(  fe1 +  fe2  + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21);

		/* F_assembly.c:5-27: load plus Dirichlet lift from Type == 0 nodes.
		 * The boundary-flux block (:30-58) multiplies by the integer 1/6 == 0. */
		for (a = 0; a < 3; a++) {
			int ja = jv[a];
			if (t->node_type[ja] < 1) continue;
			F[t->node_id[ja]] += Fe[a];
			for (b = 0; b < 3; b++)
				if (b != a && t->node_type[jv[b]] == 0)
					F[t->node_id[ja]] -= ke[a][b]*t->upresc[jv[b]];
		}
		(void)Xv; (void)Yv;

		if (t->scheme == ORC_EBE) {
			for (a = 0; a < 9; a++) A[9*E + a] = ke[a/3][a%3];
		} else if (t->scheme == ORC_EDE) {
			const int *o = t->order + 3*E, *s = t->sbe + 3*E;
			int I1 = o[0], I2 = o[1], I3 = o[2];
			double *K1 = A + 4*s[0], *K2 = A + 4*s[1], *K3 = A + 4*s[2], *Kd = A + 4*t->nedge;
			K1[0] += 0.5*ke[I1][I1]; K1[1] += ke[I1][I2]; K1[2] += ke[I2][I1]; K1[3] += 0.5*ke[I2][I2];
			K2[0] += 0.5*ke[I1][I1]; K2[1] += ke[I1][I3]; K2[2] += ke[I3][I1]; K2[3] += 0.5*ke[I3][I3];
			K3[0] += 0.5*ke[I2][I2]; K3[1] += ke[I2][I3]; K3[2] += ke[I3][I2]; K3[3] += 0.5*ke[I3][I3];
			Kd[0] = Kd[1] = Kd[2] = Kd[3] = 0;
		} else {
			const int *s = t->sbe + 9*E;
			for (a = 0; a < 9; a++) A[s[a]] += ke[a/3][a%3];
			A[t->nnz] = 0;
		}
	}
	free(U);
}

/* ------------------------------------------------------------------------ */
/* Matrix-vector products.                                                   */
void orc_csrmv(int neq, const int *IA, const int *JA, const double *AA, const double *P, double *Q)
{
	int i, j;                                  /* csrmv.c:15-20 */
	for (i = 0; i < neq; i++) Q[i] = 0;
	for (i = 0; i < neq; i++)
		for (j = IA[i]; j < IA[i+1]; j++) Q[i] += AA[j]*P[JA[j]];
}

void orc_ebemv(int neq, int nel, const int *lm, const double *A, double *P, double *Q)
{
	int I;                                     /* ebemv.c:15-40 */
	for (I = 0; I < neq; I++) Q[I] = 0;
	P[neq] = 0; Q[neq] = 0;
	for (I = 0; I < nel; I++) {
		int i1 = lm[3*I], i2 = lm[3*I+1], i3 = lm[3*I+2];
		double p1 = P[i1], p2 = P[i2], p3 = P[i3];
		const double *a = A + 9*(size_t)I;
		Q[i1] += a[0]*p1 + a[1]*p2 + a[2]*p3;
		Q[i2] += a[3]*p1 + a[4]*p2 + a[5]*p3;
		Q[i3] += a[6]*p1 + a[7]*p2 + a[8]*p3;
		Q[neq] = 0.0;
	}
}

void orc_edemv(int neq, int nedge, const int *lm2, const double *A, double *P, double *Q)
{
	int I;                                     /* edemv.c:15-36 */
	for (I = 0; I < neq; I++) Q[I] = 0;
	P[neq] = 0; Q[neq] = 0;
	for (I = 0; I < nedge; I++) {
		int i1 = lm2[2*I], i2 = lm2[2*I+1];
		double p1 = P[i1], p2 = P[i2];
		const double *a = A + 4*(size_t)I;
		Q[i1] += a[0]*p1 + a[1]*p2;
		Q[i2] += a[2]*p1 + a[3]*p2;
		Q[neq] = 0.0;
	}
}

/* ------------------------------------------------------------------------ */
/* ILU(0): ILUp_precond_setup.c:66-167 with level of fill 0, so the factor   */
/* pattern is A's (ilup.c:164-302 adds nothing at p = 0).  Row i is built    */
/* IKJ style: copy row i, then for each lower entry (ascending column jrow)  */
/* scale by 1/pivot(jrow) and subtract it times U(jrow, :) on the entries    */
/* present in row i.  Dinv holds the inverted pivots.                        */
int orc_ilu0_factor(int n, const int *IA, const int *JA, const double *AA, double *LU, double *Dinv)
{
	int *jw = malloc((size_t)n * sizeof(int)), i, j, k;
	for (j = 0; j < n; j++) jw[j] = -1;
	for (i = 0; i < n; i++) {
		double d = 0;
		for (j = IA[i]; j < IA[i+1]; j++) {
			jw[JA[j]] = j;
			if (JA[j] == i) d = AA[j]; else LU[j] = AA[j];
		}
		for (j = IA[i]; j < IA[i+1] && JA[j] < i; j++) {
			int jrow = JA[j];
			LU[j] *= Dinv[jrow];
			for (k = IA[jrow]; k < IA[jrow+1]; k++) {
				int col = JA[k], pos;
				if (col <= jrow) continue;          /* U part of row jrow */
				pos = jw[col];
				if (pos == -1) continue;
				if (col == i) d -= LU[j] * LU[k];
				else LU[pos] -= LU[j] * LU[k];
			}
		}
		for (j = IA[i]; j < IA[i+1]; j++) jw[JA[j]] = -1;
		if (d == 0) { free(jw); return 1 + i; }
		Dinv[i] = 1.0 / d;
		for (j = IA[i]; j < IA[i+1]; j++) if (JA[j] == i) LU[j] = d;
	}
	free(jw);
	return 0;
}

/* ILU(p) pattern: LEVEL_OF_FILL_lu (ilup.c:164-302).  Row i: the matrix's
 * entries at level 0, then for each lower entry k taken leftmost first, every
 * entry c of U(k,:) at level lev(i,k) + lev(k,c) + 1 <= p (new, or lowering
 * an existing level).  The filled row is emitted as the reference stores it:
 * lower ascending, the diagonal, upper in discovery order (the backward
 * sweep's order, ILUp_precond.c:38-46).  With that layout orc_ilu0_factor
 * and orc_ilu0_apply are the reference's ILUp / ILUp_precond on the filled
 * pattern.  Returns the filled nnz (fIA/fJA may be NULL to count), or -1. */
int orc_iluk_pattern(int n, const int *IA, const int *JA, int p, int *fIA, int *fJA)
{
	int *lev = malloc((size_t)n * sizeof(int)), *buf = malloc((size_t)n * sizeof(int));
	int *pos = malloc((size_t)n * sizeof(int)), *ucnt = calloc((size_t)n, sizeof(int));
	int **ucol = calloc((size_t)n, sizeof(int *)), **ulev = calloc((size_t)n, sizeof(int *));
	int i, j, nnz = 0;
	for (j = 0; j < n; j++) pos[j] = -1;
	if (fIA) fIA[0] = 0;
	for (i = 0; i < n; i++) {
		int nl = 0, nu = i, piv;
		for (j = IA[i]; j < IA[i+1]; j++) {
			int c = JA[j];
			if (c < i) { buf[nl] = c; lev[nl] = 0; pos[c] = nl++; }
			else if (c > i) { buf[nu] = c; lev[nu] = 0; pos[c] = nu++; }
		}
		for (piv = 0; piv < nl; piv++) {
			int best = piv, k, q;
			for (q = piv + 1; q < nl; q++) if (buf[q] < buf[best]) best = q;
			if (best != piv) {
				int tc = buf[piv], tl = lev[piv];
				buf[piv] = buf[best]; lev[piv] = lev[best];
				buf[best] = tc; lev[best] = tl;
				pos[buf[piv]] = piv; pos[buf[best]] = best;
			}
			k = buf[piv];
			for (q = 0; q < ucnt[k]; q++) {
				int c = ucol[k][q], l = ulev[k][q] + lev[piv] + 1;
				if (l > p) continue;
				if (pos[c] == -1) {
					if (c < i) { buf[nl] = c; lev[nl] = l; pos[c] = nl++; }
					else if (c > i) { buf[nu] = c; lev[nu] = l; pos[c] = nu++; }
				} else if (l < lev[pos[c]]) lev[pos[c]] = l;
			}
		}
		for (j = 0; j < nl; j++) pos[buf[j]] = -1;
		for (j = i; j < nu; j++) pos[buf[j]] = -1;
		ucnt[i] = nu - i;
		if (ucnt[i]) {
			ucol[i] = malloc((size_t)ucnt[i] * sizeof(int));
			ulev[i] = malloc((size_t)ucnt[i] * sizeof(int));
			memcpy(ucol[i], buf + i, (size_t)ucnt[i] * sizeof(int));
			memcpy(ulev[i], lev + i, (size_t)ucnt[i] * sizeof(int));
		}
		if (fJA) {
			memcpy(fJA + nnz, buf, (size_t)nl * sizeof(int));
			fJA[nnz + nl] = i;
			memcpy(fJA + nnz + nl + 1, buf + i, (size_t)ucnt[i] * sizeof(int));
		}
		nnz += nl + 1 + ucnt[i];
		if (fIA) fIA[i + 1] = nnz;
	}
	for (i = 0; i < n; i++) { free(ucol[i]); free(ulev[i]); }
	free(lev); free(buf); free(pos); free(ucnt); free(ucol); free(ulev);
	return nnz;
}

/* A's values on the filled pattern (zero at fill entries). */
void orc_iluk_scatter(int n, const int *IA, const int *JA, const double *AA, const int *fIA, const int *fJA,
                      double *fA)
{
	int i, j, q;
	for (i = 0; i < n; i++)
		for (q = fIA[i]; q < fIA[i+1]; q++) {
			fA[q] = 0.0;
			for (j = IA[i]; j < IA[i+1]; j++) if (JA[j] == fJA[q]) { fA[q] = AA[j]; break; }
		}
}

/* ILUp_precond.c:26-46 */
void orc_ilu0_apply(int n, const int *IA, const int *JA, const double *LU, const double *Dinv,
                    const double *p, double *z)
{
	int i, j;
	for (i = 0; i < n; i++) {
		z[i] = p[i];
		for (j = IA[i]; j < IA[i+1] && JA[j] < i; j++) z[i] -= z[JA[j]] * LU[j];
	}
	for (i = n - 1; i >= 0; i--) {
		for (j = IA[i]; j < IA[i+1]; j++) if (JA[j] > i) z[i] -= z[JA[j]] * LU[j];
		z[i] *= Dinv[i];
	}
}

/* ------------------------------------------------------------------------ */
double orc_ddot(int n, const double *x, const double *y)
{
	long i, m = n - 4;                         /* BLAS_Operations/ddot.c:4-18 */
	double s = 0.0;
	for (i = 0; i < m; i += 5)
		s += x[i]*y[i] + x[i+1]*y[i+1] + x[i+2]*y[i+2] + x[i+3]*y[i+3] + x[i+4]*y[i+4];
	for (; i < n; i++) s += x[i]*y[i];
	return s;
}

/* Operator bundle for the solver; mvf/pcf (with ctx) replace the built-in
 * schemes when set. */
typedef struct {
	int scheme, neq, nel, nedge, prec;       /* prec: 0 none, 1 ILU(p), 2 Diag */
	const int *IA, *JA, *lm, *lm2;
	const int *fIA, *fJA;                    /* ILU(p), p > 0: the filled pattern (NULL: A's) */
	const double *A, *LU, *Dinv, *invDiag;
	orc_apply_fn mvf, pcf;
	const void *ctx;
} orc_op;

static void op_mv(const orc_op *o, double *P, double *Q)
{
	if (o->mvf) o->mvf(o->ctx, P, Q);
	else if (o->scheme == ORC_CSR) orc_csrmv(o->neq, o->IA, o->JA, o->A, P, Q);
	else if (o->scheme == ORC_EBE) orc_ebemv(o->neq, o->nel, o->lm, o->A, P, Q);
	else orc_edemv(o->neq, o->nedge, o->lm2, o->A, P, Q);
}

static void op_prec(const orc_op *o, double *p, double *z)
{
	int i;
	if (o->pcf) o->pcf(o->ctx, p, z);
	else if (o->prec == 1) orc_ilu0_apply(o->neq, o->fIA ? o->fIA : o->IA, o->fJA ? o->fJA : o->JA, o->LU,
	                                      o->Dinv, p, z);
	else if (o->prec == 2) for (i = 0; i < o->neq; i++) z[i] = p[i]*o->invDiag[i];  /* Diag_precond.c:3-14 */
}

/* pgmres.c:4-211: restarted GMRES(kmax), left preconditioned, modified
 * Gram-Schmidt, Givens QR; X starts at 0; stops when the preconditioned
 * residual estimate drops to tol*||B|| (B already preconditioned). */
static int orc_pgmres(const orc_op *o, int kmax, int lmax, double tol, const double *B, double *X)
{
	int n = o->neq, i, j, k, l = 0, cont = 0;
	double **u = malloc(((size_t)kmax + 1) * sizeof(double*));
	double *h = calloc(((size_t)kmax + 1) * ((size_t)kmax + 1), sizeof(double));
	double *e = calloc((size_t)kmax + 1, sizeof(double)), *c = calloc((size_t)kmax, sizeof(double));
	double *s = calloc((size_t)kmax, sizeof(double)), *y = calloc((size_t)kmax, sizeof(double));
	double *v = calloc((size_t)n + 1, sizeof(double));
	double normb, eps, rho;
#define H(a, b) h[(size_t)(a)*((size_t)kmax + 1) + (b)]
	for (i = 0; i <= kmax; i++) u[i] = calloc((size_t)n + 1, sizeof(double));
	for (k = 0; k < n; k++) X[k] = 0;
	normb = sqrt(orc_ddot(n, B, B));
	eps = tol*normb;
	do {
		i = 0;
		for (j = 0; j < kmax; j++) memset(u[j], 0, (size_t)n * sizeof(double));
		memcpy(v, X, (size_t)n * sizeof(double));
		op_mv(o, v, u[0]);
		op_prec(o, u[0], u[0]);
		for (k = 0; k < n; k++) u[0][k] += -1.0*B[k];
		for (k = 0; k < n; k++) u[0][k] = -1.0*u[0][k];
		e[0] = sqrt(orc_ddot(n, u[0], u[0]));
		{ double sc = 1.0/e[0]; for (k = 0; k < n; k++) u[0][k] = sc*u[0][k]; }
		rho = e[0];
		do {
			cont++;
			memcpy(v, u[i], (size_t)n * sizeof(double));
			op_mv(o, v, u[i+1]);
			op_prec(o, u[i+1], u[i+1]);
			for (j = 0; j <= i; j++) {
				double hj = orc_ddot(n, u[j], u[i+1]);
				H(j, i) = hj;
				for (k = 0; k < n; k++) u[i+1][k] += -hj*u[j][k];
			}
			H(i+1, i) = sqrt(orc_ddot(n, u[i+1], u[i+1]));
			{ double sc = 1.0/H(i+1, i); for (k = 0; k < n; k++) u[i+1][k] = sc*u[i+1][k]; }
			for (j = 0; j <= i-1; j++) {
				double h1 =  c[j]*H(j, i) + s[j]*H(j+1, i);
				double h2 = -s[j]*H(j, i) + c[j]*H(j+1, i);
				H(j, i) = h1; H(j+1, i) = h2;
			}
			{
				double r = sqrt(H(i, i)*H(i, i) + H(i+1, i)*H(i+1, i));
				c[i] = H(i, i) / r;
				s[i] = H(i+1, i) / r;
				H(i, i) = r;
				H(i+1, i) = 0.0;
				e[i+1] = -s[i]*e[i];
				e[i] = c[i]*e[i];
				rho = fabs(e[i+1]);
			}
			i++;
		} while (rho > eps && i < kmax);
		i--;
		y[i] = e[i] / H(i, i);
		for (j = i-1; j >= 0; j--) {
			double soma = 0.0;
			for (k = j+1; k <= i; k++) soma = soma + H(j, k)*y[k];
			y[j] = (e[j] - soma)/H(j, j);
		}
		for (j = 0; j <= i; j++)
			for (k = 0; k < n; k++) X[k] = X[k] + u[j][k]*y[j];
		l++;
	} while (rho > eps && l < lmax);
#undef H
	for (i = 0; i <= kmax; i++) free(u[i]);
	free(u); free(h); free(e); free(c); free(s); free(y); free(v);
	return cont;
}

int orc_pgmres_cb(int neq, orc_apply_fn mv, orc_apply_fn prec, const void *ctx, int kmax, int lmax,
                  double tol, const double *B, double *X)
{
	orc_op o;
	memset(&o, 0, sizeof o);
	o.neq = neq; o.mvf = mv; o.pcf = prec; o.ctx = ctx;
	return orc_pgmres(&o, kmax, lmax, tol, B, X);
}

/* The refinement loop of the to-solution variant (see g_refine_to): returns
 * the final true relative residual; *its accumulates the pgmres iterations.
 * refine == 0: only the true residual of the reference's own solution. */
static double refine_solve(const orc_op *o, double *u, const double *Fraw, int kmax, int lmax, double tol,
                           int *its, int *rounds, int refine)
{
	int n = o->neq, k, r;
	double *v = malloc(((size_t)n + 1) * sizeof(double)), *q = malloc(((size_t)n + 1) * sizeof(double));
	double *d = malloc(((size_t)n + 1) * sizeof(double)), nb, rel = 0.0, prev = 0.0, ratio = 1.0, tr = tol;
	nb = sqrt(orc_ddot(n, Fraw, Fraw));
	for (r = 0; ; r++) {
		memcpy(v, u, ((size_t)n + 1) * sizeof(double));
		v[n] = 0.0;
		op_mv(o, v, q);
		for (k = 0; k < n; k++) q[k] = Fraw[k] - q[k];
		q[n] = 0.0;
		rel = nb > 0 ? sqrt(orc_ddot(n, q, q)) / nb : 0.0;
		if (!refine || rel <= g_refine_to || r >= g_refine_max || !(rel == rel)) break;
		/* The loosest pgmres tolerance expected to reach the target: the last
		 * solve reduced the true residual by (rel/prev) at preconditioned
		 * tolerance tr, so the true/preconditioned ratio is about
		 * (rel/prev)/tr; aim at half the target, within [g_refine_tol, 0.5]. */
		ratio = r == 0 ? rel / tol : (rel / prev) / tr;
		if (!(ratio >= 1.0)) ratio = 1.0;
		tr = 0.5 * g_refine_to / rel / ratio;
		if (tr < g_refine_tol) tr = g_refine_tol;
		if (tr > 0.5) tr = 0.5;
		prev = rel;
		op_prec(o, q, q);                       /* the correction system's RHS, M^-1 r */
		*its += orc_pgmres(o, kmax, lmax, tr, q, d);
		for (k = 0; k < n; k++) u[k] += d[k];
	}
	*rounds = r;
	free(v); free(q); free(d);
	return rel;
}

/* Diag_precond_{CSR,EBE,EDE}_setup.c: extract the diagonal, invert, F *= 1/D. */
static void diag_setup(orc_op *o, double *invDiag, double *F)
{
	int n = o->neq, I, E;
	double *D = calloc((size_t)n + 1, sizeof(double));
	if (o->scheme == ORC_CSR) {
		for (I = 0; I < n; I++)
			for (E = o->IA[I]; E < o->IA[I+1]; E++) if (o->JA[E] == I) D[I] = o->A[E];
	} else if (o->scheme == ORC_EBE) {
		for (E = 0; E < o->nel; E++) {
			for (I = 0; I < 3; I++) D[o->lm[3*E+I]] += o->A[9*(size_t)E + 4*I];
			D[n] = 0;
		}
	} else {
		for (E = 0; E < o->nedge; E++) {
			D[o->lm2[2*E]] += o->A[4*(size_t)E];
			D[o->lm2[2*E+1]] += o->A[4*(size_t)E + 3];
			D[n] = 0;
		}
	}
	for (I = 0; I < n; I++) invDiag[I] = 1.0/D[I];
	invDiag[n] = 1.0;
	for (I = 0; I < n; I++) F[I] *= invDiag[I];
	free(D);
	o->invDiag = invDiag;
}

/* ------------------------------------------------------------------------ */
static int classify_element(const double *x, const double *y, const int *v)
{
	int c1 = 0, c2 = 0, c3 = 0, c4 = 0, j;     /* Preprocess.c:108-152 */
	for (j = 0; j < 3; j++) {
		if (x[v[j]] == 0.0) c1++;
		if (y[v[j]] == 0.0) c2++;
		if (x[v[j]] == 1.0) c3++;
		if (y[v[j]] == 1.0) c4++;
	}
	if (c1 == 2) return (c1 == c2) ? 5 : (c1 == c4) ? 8 : 1;
	if (c2 == 2) return (c2 == c3) ? 6 : 2;
	if (c3 == 2) return (c3 == c4) ? 7 : 3;
	if (c4 == 2) return 4;
	return -1;
}

/* Preprocess.c:160-237 + Process.c:283-335 (with precond_setup after every
 * Build, as Process.c:53 intends). */
int orc_transport_run(int nnodes, const double *x, const double *y, const int *ntype,
		int nel, const int *vert, double k, double gamma,
		const double *beta, const double *fsrc, const double *upresc,
		const char *scheme, const char *reord, const char *precond,
		const char *shock, const char *hshock, const char *outflow,
		int kmax, int lmax, double tol, int npicard, double nonlin_tol,
		int *info, int *node_id, int *etype,
		int *IA_out, int *JA_out, int *sbe_out, int *order_out,
		double *Afirst, double *Ffirst, double *Fprec,
		const double *Pin, double *Qmv, double *Zpc,
		double *uhist, int *iters)
{
	orc_transport t;
	orc_op o;
	int *lm = malloc(3 * (size_t)nel * sizeof(int)), neq, I, it = 0;
	size_t nA;
	double *A, *F, *u, *uold, *LU = NULL, *Dinv = NULL, *invDiag = NULL, *Fraw = NULL, *fA = NULL, err = 100.0;
	int *fIA = NULL, *fJA = NULL;
	size_t nLU = 0;

	double t0 = now_s(), t1;
	memset(&t, 0, sizeof t);
	memset(&o, 0, sizeof o);
	memset(g_times, 0, sizeof g_times);
	neq = orc_fill_lm(nnodes, ntype, nel, vert, node_id, lm);
	for (I = 0; I < nel; I++) etype[I] = classify_element(x, y, vert + 3*I);
	t.nnodes = nnodes; t.nel = nel; t.neq = neq;
	t.x = x; t.y = y; t.node_type = ntype; t.node_id = node_id; t.vert = vert; t.etype = etype;
	t.beta = beta; t.fsrc = fsrc; t.upresc = upresc; t.k = k; t.gamma = gamma;
	t.shock = strcasecmp(shock, "YZBeta") == 0 ? ORC_YZBETA : ORC_CAU;
	t.hshock = strcasecmp(hshock, "sqrtArea") == 0 ? ORC_H_SQRTAREA :
		strcasecmp(hshock, "Option1") == 0 ? ORC_H_OPTION1 :
		strcasecmp(hshock, "Option2") == 0 ? ORC_H_OPTION2 : ORC_H_2SQRTAREA;
	t.outflow = strcasecmp(outflow, "YES") == 0;
	info[0] = neq; info[1] = 0; info[2] = 0; info[3] = 0;
	o.neq = neq; o.nel = nel; o.lm = lm;

	if (strcasecmp(scheme, "EBE") == 0) {
		t.scheme = ORC_EBE;
		nA = 9 * (size_t)nel;
	} else if (strcasecmp(scheme, "EDE") == 0) {
		t.scheme = ORC_EDE;
		t.nedge = orc_ede_pattern(neq, nel, lm, NULL, NULL, NULL);
		if (t.nedge < 0) { free(lm); return -1; }
		orc_ede_pattern(neq, nel, lm, JA_out, sbe_out, order_out);
		t.sbe = sbe_out; t.order = order_out;
		info[2] = t.nedge;
		o.lm2 = JA_out; o.nedge = t.nedge;
		nA = 4 * ((size_t)t.nedge + 1);
	} else {
		t.scheme = ORC_CSR;
		t.nnz = orc_csr_pattern(neq, nel, lm, NULL, NULL, NULL);
		orc_csr_pattern(neq, nel, lm, IA_out, JA_out, sbe_out);
		info[3] = orc_bandwidth(neq, IA_out, JA_out);
		if (strcasecmp(reord, "SYMRCM") == 0) {
			int *perm = malloc((size_t)neq * sizeof(int) + 1);
			orc_symrcm(neq, IA_out, JA_out, perm);
			info[3] = orc_reorder_csr(neq, t.nnz, IA_out, JA_out, perm, nel, sbe_out, nnodes, node_id);
			free(perm);
		}
		t.sbe = sbe_out;
		info[1] = t.nnz;
		o.IA = IA_out; o.JA = JA_out;
		nA = (size_t)t.nnz + 1;
	}
	o.scheme = t.scheme;
	o.prec = strcasecmp(precond, "NOT") == 0 ? 0 : strcasecmp(precond, "Diag") == 0 ? 2 : 1;
	if (o.prec == 1 && t.scheme != ORC_CSR) { free(lm); return -2; }
	/* "ILU<p>" (ILUp_precond_setup.c:15): p > 0 factors on the filled pattern */
	if (o.prec == 1 && strncasecmp(precond, "ILU", 3) == 0 && atoi(precond + 3) > 0) {
		int lvl = atoi(precond + 3), fnnz = orc_iluk_pattern(neq, IA_out, JA_out, lvl, NULL, NULL);
		fIA = malloc(((size_t)neq + 1) * sizeof(int));
		fJA = malloc((size_t)fnnz * sizeof(int) + 4);
		fA = malloc((size_t)fnnz * sizeof(double) + 8);
		orc_iluk_pattern(neq, IA_out, JA_out, lvl, fIA, fJA);
		o.fIA = fIA; o.fJA = fJA;
		nLU = (size_t)fnnz + 1;
	}

	A = calloc(nA, sizeof(double));
	F = calloc((size_t)neq + 1, sizeof(double));
	u = calloc((size_t)neq + 1, sizeof(double));
	uold = calloc((size_t)neq + 1, sizeof(double));
	if (o.prec == 1) { LU = calloc(nLU ? nLU : nA, sizeof(double)); Dinv = calloc((size_t)neq + 1, sizeof(double)); }
	if (o.prec == 2) invDiag = calloc((size_t)neq + 1, sizeof(double));
	if (g_refine_to > 0) Fraw = calloc((size_t)neq + 1, sizeof(double));
	o.A = A; o.LU = LU; o.Dinv = Dinv;
	t1 = now_s();
	g_times[0] = t1 - t0;

	double refined_s = 0.0;
	while (it < npicard && (nonlin_tol <= 0 || err > nonlin_tol) &&
	       !(g_refine_to > 0 && g_refine_budget > 0 && refined_s > g_refine_budget)) {
		double tstep = now_s();
		it++;
		memcpy(uold, u, (size_t)neq * sizeof(double));
		t0 = tstep;
		orc_build_supg(&t, u, A, F);
		if (Fraw) memcpy(Fraw, F, ((size_t)neq + 1) * sizeof(double));
		t1 = now_s();
		g_times[1] += t1 - t0;
		if (it == 1) {
			double *tmp = malloc(((size_t)neq + 1) * sizeof(double));
			memcpy(Ffirst, F, ((size_t)neq + 1) * sizeof(double));
			memcpy(Afirst, A, nA * sizeof(double));
			memcpy(tmp, Pin, ((size_t)neq + 1) * sizeof(double));
			op_mv(&o, tmp, Qmv);
			free(tmp);
		}
		t0 = now_s();
		if (o.prec == 1 && o.fIA) {
			orc_iluk_scatter(neq, o.IA, o.JA, A, o.fIA, o.fJA, fA);
			if (orc_ilu0_factor(neq, o.fIA, o.fJA, fA, LU, Dinv)) { it = -3; break; }
			orc_ilu0_apply(neq, o.fIA, o.fJA, LU, Dinv, F, F);
		} else if (o.prec == 1) {
			if (orc_ilu0_factor(neq, o.IA, o.JA, A, LU, Dinv)) { it = -3; break; }
			orc_ilu0_apply(neq, o.IA, o.JA, LU, Dinv, F, F);
		} else if (o.prec == 2) {
			diag_setup(&o, invDiag, F);
		}
		g_times[2] += now_s() - t0;
		if (it == 1) {
			memcpy(Fprec, F, ((size_t)neq + 1) * sizeof(double));
			memcpy(Zpc, Pin, ((size_t)neq + 1) * sizeof(double));
			op_prec(&o, (double *)Pin, Zpc);
		}
		t0 = now_s();
		iters[it-1] = orc_pgmres(&o, kmax, lmax, tol, F, u);
		if (g_refine_to > 0 && it - 1 < ORC_MAX_STEPS) {
			int rounds = 0;
			double rel = refine_solve(&o, u, Fraw, kmax, lmax, tol, &iters[it-1], &rounds,
			                          it - 1 >= g_refine_from);
			g_refine_res[it-1] = rel;
			g_refine_its[it-1] = rounds;
		}
		t1 = now_s();
		if (g_refine_to > 0 && it - 1 >= g_refine_from) refined_s += t1 - tstep;
		g_times[3] += t1 - t0;
		if (it - 1 < ORC_MAX_STEPS) g_step[it-1] = t1 - tstep;
		memcpy(uhist + (size_t)(it-1)*((size_t)neq + 1), u, ((size_t)neq + 1) * sizeof(double));
		err = 0.0;
		for (I = 0; I < neq; I++) {
			double d = fabs(u[I] - uold[I]);
			if (I == 0 || d > err) err = d;
		}
	}
	free(lm); free(A); free(F); free(u); free(uold); free(LU); free(Dinv); free(invDiag); free(Fraw);
	free(fIA); free(fJA); free(fA);
	return it;
}

int orc_csr_gmres(int neq, const int *IA, const int *JA, const double *AA, int use_ilu0,
                  int kmax, int lmax, double tol, double *B, double *X)
{
	orc_op o;
	int it;
	double *LU = NULL, *Dinv = NULL;
	memset(&o, 0, sizeof o);
	o.scheme = ORC_CSR; o.neq = neq; o.IA = IA; o.JA = JA; o.A = AA; o.prec = use_ilu0 ? 1 : 0;
	if (use_ilu0) {
		LU = malloc((size_t)IA[neq] * sizeof(double) + 8);
		Dinv = malloc((size_t)neq * sizeof(double) + 8);
		if (orc_ilu0_factor(neq, IA, JA, AA, LU, Dinv)) { free(LU); free(Dinv); return -1; }
		orc_ilu0_apply(neq, IA, JA, LU, Dinv, B, B);
		o.LU = LU; o.Dinv = Dinv;
	}
	it = orc_pgmres(&o, kmax, lmax, tol, B, X);
	free(LU); free(Dinv);
	return it;
}
