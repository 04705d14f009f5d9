/*
 * Algebraic multigrid preconditioner, double pairwise aggregation ("DPA",
 * 00_CommonFiles/Solvers_and_Preconditioners/CSR/AMG/amg_dpa.c:424-463 with
 * the deck string "AMG 2 NCL beta omega nr", amg_precond.c:26-105): host
 * set-up of the hierarchy and the level schedules of its SOR smoothers; the
 * V-cycle runs on the device (csrc/amg.cu).
 *
 * Set-up per level: a pairwise matching of the level's graph -- the
 * counting-sort greedy matching of amg_dpa.c:30-173 (beta >= 0) or the
 * half-approximate maximum-product matching of bcm_linmatch.c (Preis'
 * algorithm as BootCMatch 0.9 implements it; beta == -1) -- then the
 * Galerkin product P^T A P of amg_dpa.c:175-392 (rows of a pair summed, their
 * columns merged).  The set-up is sequential greedy work (like SYMRCM) and
 * stays on the host; its ordering and tie rules are those of the reference,
 * so the hierarchy is the reference's bit for bit.  Plain C.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_amg.h"

/* ---- host CSR ------------------------------------------------------------ */
typedef struct {
	int n, nnz;
	int *ptr, *col;
	double *val, *diag;
} hmat;

static int hmat_alloc(hmat *A, int n, int nnz)
{
	A->n = n; A->nnz = nnz;
	A->ptr = calloc((size_t)n + 1, sizeof(int));
	A->col = calloc((size_t)(nnz ? nnz : 1), sizeof(int));
	A->val = calloc((size_t)(nnz ? nnz : 1), sizeof(double));
	A->diag = calloc((size_t)(n ? n : 1), sizeof(double));
	return (A->ptr && A->col && A->val && A->diag) ? 0 : FEMGPU_E_NOMEM;
}

static void hmat_free(hmat *A)
{
	free(A->ptr); free(A->col); free(A->val); free(A->diag);
	memset(A, 0, sizeof *A);
}

/* Row lists with the reference's list operations (amg_list.c): nodes in an
 * array, each row a singly linked list with head and tail. */
typedef struct { int elem; double val; int next; } lnode;
typedef struct { lnode *nd; int cnt, cap; int *head, *tail, *len; } rowlists;

static int rl_init(rowlists *L, int rows, int cap)
{
	L->cap = cap > 0 ? cap : 1; L->cnt = 0;
	L->nd = malloc(sizeof(lnode) * (size_t)L->cap);
	L->head = malloc(sizeof(int) * (size_t)(rows ? rows : 1));
	L->tail = malloc(sizeof(int) * (size_t)(rows ? rows : 1));
	L->len = calloc((size_t)(rows ? rows : 1), sizeof(int));
	if (!L->nd || !L->head || !L->tail || !L->len) return FEMGPU_E_NOMEM;
	for (int i = 0; i < rows; i++) L->head[i] = L->tail[i] = -1;
	return 0;
}

static void rl_free(rowlists *L) { free(L->nd); free(L->head); free(L->tail); free(L->len); }

static int rl_new(rowlists *L, int e, double v)
{
	if (L->cnt == L->cap) {
		lnode *p = realloc(L->nd, sizeof(lnode) * (size_t)L->cap * 2);
		if (!p) return -1;
		L->nd = p; L->cap *= 2;
	}
	L->nd[L->cnt].elem = e; L->nd[L->cnt].val = v; L->nd[L->cnt].next = -1;
	return L->cnt++;
}

static int rl_tail(rowlists *L, int r, int e, double v)        /* insert_l_tail */
{
	int t = rl_new(L, e, v);
	if (t < 0) return -1;
	if (L->tail[r] >= 0) { L->nd[L->tail[r]].next = t; L->tail[r] = t; }
	else L->head[r] = L->tail[r] = t;
	L->len[r]++;
	return t;
}

static int rl_head(rowlists *L, int r, int e, double v)        /* insert_l_head */
{
	int t = rl_new(L, e, v);
	if (t < 0) return -1;
	L->nd[t].next = L->head[r];
	L->head[r] = t;
	if (L->tail[r] < 0) L->tail[r] = t;
	L->len[r]++;
	return t;
}

static int rl_sorted(rowlists *L, int r, int e, double v)      /* insert_l_sort: after equal elems */
{
	int t = rl_new(L, e, v), c;
	if (t < 0) return -1;
	if (!L->len[r] || e < L->nd[L->head[r]].elem) {
		L->nd[t].next = L->head[r];
		L->head[r] = t;
		if (L->tail[r] < 0) L->tail[r] = t;
	} else {
		for (c = L->head[r]; L->nd[c].next >= 0 && e >= L->nd[L->nd[c].next].elem; c = L->nd[c].next) {}
		L->nd[t].next = L->nd[c].next;
		L->nd[c].next = t;
		if (L->nd[t].next < 0) L->tail[r] = t;
	}
	L->len[r]++;
	return t;
}

/* ---- transpose and symmetric sums (amg_matrix.c:63-250) -------------------- */
static int transpose(const hmat *A, hmat *T)
{
	int i, j, k = 0;
	rowlists L;
	if (rl_init(&L, A->n, A->nnz) || hmat_alloc(T, A->n, A->nnz)) return FEMGPU_E_NOMEM;
	for (i = 0; i < A->n; i++)
		for (j = A->ptr[i]; j < A->ptr[i + 1]; j++)
			if (rl_tail(&L, A->col[j], i, A->val[j]) < 0) return FEMGPU_E_NOMEM;
	for (i = 0; i < A->n; i++) {
		for (int t = L.head[i]; t >= 0; t = L.nd[t].next, k++) { T->val[k] = L.nd[t].val; T->col[k] = L.nd[t].elem; }
		T->diag[i] = A->diag[i];
		T->ptr[i + 1] = k;
	}
	rl_free(&L);
	return 0;
}

/* |A| + |A^T| merged row by row from the back (sum_abs), or only its strict
 * upper triangle (sum_upper; the matrices here have a symmetric pattern). */
static int abs_sum(const hmat *A, const hmat *T, int upper, hmat *S)
{
	int i, k = 0, nnz = 0;
	rowlists L;
	if (rl_init(&L, A->n, A->nnz + T->nnz)) return FEMGPU_E_NOMEM;
	for (i = 0; i < A->n; i++) {
		int j = A->ptr[i + 1] - 1, jt = T->ptr[i + 1] - 1;
		while (j >= A->ptr[i] || jt >= T->ptr[i]) {
			int ina = j >= A->ptr[i], inb = jt >= T->ptr[i];
			if (upper && !((ina && A->col[j] > i) || (inb && T->col[jt] > i))) break;
			if (ina && inb && A->col[j] == T->col[jt]) {
				if (rl_head(&L, i, A->col[j], fabs(A->val[j]) + fabs(T->val[jt])) < 0) return FEMGPU_E_NOMEM;
				j--; jt--;
			} else if ((ina && (!inb || A->col[j] > T->col[jt])) || !inb) {
				if (rl_head(&L, i, A->col[j], fabs(A->val[j])) < 0) return FEMGPU_E_NOMEM;
				j--;
			} else {
				if (rl_head(&L, i, T->col[jt], fabs(T->val[jt])) < 0) return FEMGPU_E_NOMEM;
				jt--;
			}
			nnz++;
		}
	}
	if (hmat_alloc(S, A->n, nnz)) return FEMGPU_E_NOMEM;
	for (i = 0; i < A->n; i++) {
		for (int t = L.head[i]; t >= 0; t = L.nd[t].next, k++) { S->val[k] = L.nd[t].val; S->col[k] = L.nd[t].elem; }
		S->ptr[i + 1] = k;
	}
	rl_free(&L);
	return 0;
}

/* ---- counting-sort greedy matching (amg_dpa.c:30-173) ---------------------- */
typedef struct { int *prev, *next, *m, *in, *bhead, *btail, *bcnt; int n, min_m; } countsort;

static int cs_init(countsort *c, int n)
{
	c->n = n; c->min_m = 2 * n;
	c->prev = malloc(sizeof(int) * (size_t)n); c->next = malloc(sizeof(int) * (size_t)n);
	c->m = malloc(sizeof(int) * (size_t)n); c->in = calloc((size_t)n, sizeof(int));
	c->bhead = malloc(sizeof(int) * 2 * (size_t)n); c->btail = malloc(sizeof(int) * 2 * (size_t)n);
	c->bcnt = calloc(2 * (size_t)n, sizeof(int));
	if (!c->prev || !c->next || !c->m || !c->in || !c->bhead || !c->btail || !c->bcnt) return FEMGPU_E_NOMEM;
	for (int b = 0; b < 2 * n; b++) c->bhead[b] = c->btail[b] = -1;
	return 0;
}

static void cs_free(countsort *c)
{
	free(c->prev); free(c->next); free(c->m); free(c->in); free(c->bhead); free(c->btail); free(c->bcnt);
}

static void cs_append(countsort *c, int i, int m)
{
	c->m[i] = m;
	c->next[i] = -1;
	c->prev[i] = c->btail[m];
	if (c->btail[m] >= 0) c->next[c->btail[m]] = i; else c->bhead[m] = i;
	c->btail[m] = i;
	c->bcnt[m]++;
}

static void cs_unlink(countsort *c, int i)
{
	int m = c->m[i];
	if (c->prev[i] >= 0) c->next[c->prev[i]] = c->next[i]; else c->bhead[m] = c->next[i];
	if (c->next[i] >= 0) c->prev[c->next[i]] = c->prev[i]; else c->btail[m] = c->prev[i];
	c->bcnt[m]--;
}

static void cs_insert(countsort *c, int i, int m)
{
	cs_append(c, i, m);
	c->in[i] = 1;
	if (m < c->min_m) c->min_m = m;
}

static void cs_remove(countsort *c, int i)
{
	int m = c->m[i];
	cs_unlink(c, i);
	c->in[i] = 0;
	if (c->bcnt[c->min_m] == 0)
		for (c->min_m = m + 1; c->min_m < 2 * c->n && c->bcnt[c->min_m] == 0; c->min_m++) {}
}

static void cs_move(countsort *c, int i, int new_m)
{
	int m = c->m[i];
	cs_unlink(c, i);
	cs_append(c, i, new_m);
	if (new_m < c->min_m) c->min_m = new_m;
	else if (c->bcnt[c->min_m] == 0)
		for (c->min_m = m + 1; c->min_m < 2 * c->n && c->bcnt[c->min_m] == 0; c->min_m++) {}
}

static int match_greedy(const hmat *A0, double beta, int *rmatch)
{
	hmat T, A;
	countsort c;
	int i, j, n = A0->n, nc = 0, rc;
	int *sptr, *scol, ns = 0;
	double *mx;
	if ((rc = transpose(A0, &T)) || (rc = abs_sum(A0, &T, 0, &A))) return rc;
	hmat_free(&T);
	mx = calloc((size_t)n, sizeof(double));
	sptr = calloc((size_t)n + 1, sizeof(int));
	scol = malloc(sizeof(int) * (size_t)(A.nnz ? A.nnz : 1));
	if (!mx || !sptr || !scol || cs_init(&c, n)) return FEMGPU_E_NOMEM;
	for (i = 0; i < n; i++)
		for (j = A.ptr[i]; j < A.ptr[i + 1]; j++) if (fabs(A.val[j]) > mx[i]) mx[i] = fabs(A.val[j]);
	for (i = 0; i < n; i++) {                           /* strong neighbours S_i */
		for (j = A.ptr[i]; j < A.ptr[i + 1]; j++)
			if (i != A.col[j] && A.val[j] > beta * mx[i]) scol[ns++] = A.col[j];
		sptr[i + 1] = ns;
	}
	for (i = 0; i < n; i++) cs_insert(&c, i, (sptr[i + 1] - sptr[i]) + n);
	while (c.min_m < 2 * n) {
		int max_j, exist = 0, in_s = 0;
		i = c.bhead[c.min_m];
		nc++;
		max_j = A.ptr[i];
		for (j = A.ptr[i]; j < A.ptr[i + 1]; j++)
			if (i != A.col[j] && c.in[A.col[j]]) {
				if (A.val[j] >= A.val[max_j] || !exist) max_j = j;
				exist = 1;
			}
		j = A.col[max_j];
		for (int s = sptr[i]; s < sptr[i + 1]; s++) if (scol[s] == j) { in_s = 1; break; }
		if (in_s && exist) {
			rmatch[i] = j; rmatch[j] = i;
			cs_remove(&c, i);
			cs_remove(&c, j);
			for (int s = sptr[i]; s < sptr[i + 1]; s++) if (c.in[scol[s]]) cs_move(&c, scol[s], c.m[scol[s]] - 1);
			for (int s = sptr[j]; s < sptr[j + 1]; s++) if (c.in[scol[s]]) cs_move(&c, scol[s], c.m[scol[s]] - 1);
		} else {
			rmatch[i] = -1;
			cs_remove(&c, i);
			for (int s = sptr[i]; s < sptr[i + 1]; s++) if (c.in[scol[s]]) cs_move(&c, scol[s], c.m[scol[s]] - 1);
		}
	}
	rmatch[n] = n - nc;
	free(mx); free(sptr); free(scol); cs_free(&c); hmat_free(&A);
	return 0;
}

/* ---- half-approximate maximum-product matching (bcm_linmatch.c) ------------ */
typedef struct { const hmat *W; int *rmatch; int pairs; } hmatch;

static double w_at(const hmat *W, int r, int c)
{
	for (int k = W->ptr[r]; k < W->ptr[r + 1]; k++) if (W->col[k] == c) return W->val[k];
	return -HUGE_VAL;   /* not reached: every pair looked up is an entry of W's strict upper triangle */
}

static void list_drop(int *lst, int *len, int v)     /* remove the first v, keep order */
{
	int k = -1, i;
	for (i = 0; i < *len && k == -1; i++) if (lst[i] == v) k = i;
	if (k >= 0) { (*len)--; for (i = k; i < *len; i++) lst[i] = lst[i + 1]; }
}

static int try_match(hmatch *H, int row, int col, int *jrow, int ljrow, int *jcol, int ljcol)
{
	const hmat *W = H->W;
	int *rm = H->rmatch;
	double cw;
	list_drop(jrow, &ljrow, col);
	list_drop(jcol, &ljcol, row);
	cw = w_at(W, row, col);
	while (rm[row] == -1 && rm[col] == -1 && (ljrow != 0 || ljcol != 0)) {
		if (rm[row] == -1 && ljrow != 0) {
			int t = jrow[0], i;
			double nw = w_at(W, row, t);
			ljrow--;
			for (i = 0; i < ljrow; i++) jrow[i] = jrow[i + 1];
			if (nw > cw && rm[t] == -1) {
				int nz = W->ptr[t + 1] - W->ptr[t];
				int *tl = malloc(sizeof(int) * (size_t)(nz ? nz : 1));
				if (!tl) return FEMGPU_E_NOMEM;
				memcpy(tl, W->col + W->ptr[t], sizeof(int) * (size_t)nz);
				int rc = try_match(H, row, t, jrow, ljrow, tl, nz);
				free(tl);
				if (rc) return rc;
			}
		}
		if (rm[col] == -1 && ljcol != 0) {
			int t = jcol[0], i;
			double nw = w_at(W, col, t);
			ljcol--;
			for (i = 0; i < ljcol; i++) jcol[i] = jcol[i + 1];
			if (nw > cw && rm[t] == -1) {
				int nz = W->ptr[t + 1] - W->ptr[t];
				int *tl = malloc(sizeof(int) * (size_t)(nz ? nz : 1));
				if (!tl) return FEMGPU_E_NOMEM;
				memcpy(tl, W->col + W->ptr[t], sizeof(int) * (size_t)nz);
				int rc = try_match(H, col, t, jcol, ljcol, tl, nz);
				free(tl);
				if (rc) return rc;
			}
		}
	}
	if (rm[row] == -1 && rm[col] == -1) { rm[row] = col; rm[col] = row; H->pairs++; }
	return 0;
}

static int match_hmatch(const hmat *A0, int *rmatch)
{
	hmat T, B, W;
	hmatch H;
	int i, j, rc, n = A0->n;
	int *jrow, *jjrow;
	double mn;
	if ((rc = transpose(A0, &T)) || (rc = abs_sum(A0, &T, 1, &B))) return rc;
	hmat_free(&T);
	if (hmat_alloc(&W, B.n, B.nnz)) return FEMGPU_E_NOMEM;
	memcpy(W.ptr, B.ptr, sizeof(int) * ((size_t)B.n + 1));
	memcpy(W.col, B.col, sizeof(int) * (size_t)B.nnz);
	mn = B.nnz ? fabs(B.val[0]) : 0.0;
	for (i = 1; i < B.nnz; i++) if (mn > fabs(B.val[i])) mn = fabs(B.val[i]);
	for (i = 0; i < B.nnz; i++) W.val[i] = log(fabs(B.val[i]) / (0.999 * mn));
	for (i = 0; i < n; i++) rmatch[i] = -1;
	jrow = malloc(sizeof(int) * (size_t)(n ? n : 1));
	jjrow = malloc(sizeof(int) * (size_t)(n ? n : 1));
	if (!jrow || !jjrow) return FEMGPU_E_NOMEM;
	H.W = &W; H.rmatch = rmatch; H.pairs = 0;
	for (i = 0; i < n; i++) {
		int nz = B.ptr[i + 1] - B.ptr[i];
		for (j = 0; j < nz; j++) jrow[j] = B.col[B.ptr[i] + j];
		for (j = 0; j < nz; j++) {
			int cno = B.col[B.ptr[i] + j], nzc = B.ptr[cno + 1] - B.ptr[cno];
			for (int k = 0; k < nzc; k++) jjrow[k] = B.col[B.ptr[cno] + k];
			if (rmatch[i] == -1 && rmatch[cno] == -1 && (rc = try_match(&H, i, cno, jrow, nz, jjrow, nzc)))
				return rc;
		}
	}
	rmatch[n] = H.pairs;
	free(jrow); free(jjrow); hmat_free(&B); hmat_free(&W);
	return 0;
}

/* ---- Galerkin product with the pairwise prolongator (amg_dpa.c:175-392) ---- */
static int galerkin(const hmat *A, const int *rmatch, hmat *C)
{
	int n = A->n, nc = n - rmatch[n], line = 0, i, nnz = 0, k = 0;
	rowlists L;
	int *pair = malloc(sizeof(int) * (size_t)(n ? n : 1)), *pair_aux = malloc(sizeof(int) * (size_t)(n ? n : 1));
	int *pair_ind = calloc((size_t)(n ? n : 1), sizeof(int));
	if (!pair || !pair_aux || !pair_ind || rl_init(&L, nc, A->nnz)) return FEMGPU_E_NOMEM;
	for (i = 0; i < n; i++) pair_aux[i] = -1;
#define PUT(COL, VAL) do {                                                                      \
	int c_ = (COL);                                                                            \
	if (pair_aux[c_] == i) {                                                                   \
		L.nd[pair[c_]].val += (VAL);                                                           \
	} else {                                                                                   \
		if (rmatch[c_] == -1) { if (rl_tail(&L, line, c_, (VAL)) < 0) return FEMGPU_E_NOMEM; } \
		else if (c_ > rmatch[c_]) { if (rl_sorted(&L, line, rmatch[c_], (VAL)) < 0) return FEMGPU_E_NOMEM; } \
		else {                                                                                 \
			int t_ = rl_tail(&L, line, c_, (VAL));                                             \
			if (t_ < 0) return FEMGPU_E_NOMEM;                                                 \
			pair[rmatch[c_]] = t_;                                                             \
			pair_aux[rmatch[c_]] = i;                                                          \
		}                                                                                      \
		nnz++;                                                                                 \
	} } while (0)
	for (i = 0; i < n; i++) {
		if (rmatch[i] == -1) {
			for (int a = A->ptr[i]; a < A->ptr[i + 1]; a++) PUT(A->col[a], A->val[a]);
			pair_ind[i] = line++;
		} else if (i < rmatch[i]) {
			int a = A->ptr[i], ae = A->ptr[i + 1], b = A->ptr[rmatch[i]], be = A->ptr[rmatch[i] + 1];
			while (a < ae || b < be) {
				if (b == be) { PUT(A->col[a], A->val[a]); a++; }
				else if (a == ae || A->col[a] > A->col[b]) { PUT(A->col[b], A->val[b]); b++; }
				else if (A->col[a] < A->col[b]) { PUT(A->col[a], A->val[a]); a++; }
				else { PUT(A->col[a], A->val[a] + A->val[b]); a++; b++; }
			}
			pair_ind[i] = pair_ind[rmatch[i]] = line++;
		}
	}
#undef PUT
	if (hmat_alloc(C, nc, nnz)) return FEMGPU_E_NOMEM;
	for (i = 0; i < nc; i++) {
		for (int t = L.head[i]; t >= 0; t = L.nd[t].next, k++) {
			C->val[k] = L.nd[t].val;
			C->col[k] = pair_ind[L.nd[t].elem];
			if (pair_ind[L.nd[t].elem] == i) C->diag[i] = L.nd[t].val;
		}
		C->ptr[i + 1] = k;
	}
	rl_free(&L); free(pair); free(pair_aux); free(pair_ind);
	return 0;
}

/* ---- level schedules of the SOR sweeps -------------------------------------- */
/* Rows in the order a level-by-level sweep processes them; lev [nlev+1].  In
 * the forward sweep (SOR_relax) every coupled pair (i, j), i < j, in either
 * row's pattern orders i before j: j reads the new u[i], i the old u[j].  The
 * reverse sweep (SOR_relax_rev) orders j before i. */
static int sor_levels(const hmat *A, int reverse, int **rows_out, int **lev_out, int *nlev_out)
{
	int n = A->n, i, nlev = 0;
	int *lv = calloc((size_t)(n ? n : 1), sizeof(int)), *cnt, *rows, *fill;
	if (!lv) return FEMGPU_E_NOMEM;
	for (int s = 0; s < n; s++) {
		int r = reverse ? n - 1 - s : s;
		for (int k = A->ptr[r]; k < A->ptr[r + 1]; k++) {     /* earlier rows of r's own pattern */
			int c = A->col[k];
			if ((reverse ? c > r : c < r) && lv[c] + 1 > lv[r]) lv[r] = lv[c] + 1;
		}
		for (int k = A->ptr[r]; k < A->ptr[r + 1]; k++) {     /* later rows r appears in */
			int c = A->col[k];
			if ((reverse ? c < r : c > r) && lv[r] + 1 > lv[c]) lv[c] = lv[r] + 1;
		}
		if (lv[r] + 1 > nlev) nlev = lv[r] + 1;
	}
	cnt = calloc((size_t)nlev + 1, sizeof(int));
	rows = malloc(sizeof(int) * (size_t)(n ? n : 1));
	fill = malloc(sizeof(int) * (size_t)nlev + 1);
	if (!cnt || !rows || !fill) return FEMGPU_E_NOMEM;
	for (i = 0; i < n; i++) cnt[lv[i] + 1]++;
	for (i = 0; i < nlev; i++) cnt[i + 1] += cnt[i];
	memcpy(fill, cnt, sizeof(int) * (size_t)nlev);
	for (int s = 0; s < n; s++) { int r = reverse ? n - 1 - s : s; rows[fill[lv[r]]++] = r; }
	free(lv); free(fill);
	*rows_out = rows; *lev_out = cnt; *nlev_out = nlev;
	return 0;
}

/* Runs of levels: a level wider than AMG_WIDE rows is its own grid launch,
 * the levels between wide ones go to one thread block. */
#define AMG_WIDE 8192
static int segments(const int *lev, int nlev, fg_amg_seg **out, int *nout)
{
	int ns = 0;
	fg_amg_seg *s = malloc(sizeof(fg_amg_seg) * (size_t)(nlev ? nlev : 1));
	if (!s) return FEMGPU_E_NOMEM;
	for (int l = 0; l < nlev;) {
		if (lev[l + 1] - lev[l] > AMG_WIDE) { s[ns].l0 = l; s[ns].l1 = l + 1; s[ns].wide = 1; ns++; l++; continue; }
		s[ns].l0 = l;
		while (l < nlev && lev[l + 1] - lev[l] <= AMG_WIDE) l++;
		s[ns].l1 = l; s[ns].wide = 0; ns++;
	}
	*out = s; *nout = ns;
	return 0;
}

/* ---- host utilities (no GPU) ---------------------------------------------- */
static int wrap(int n, const int *IA, const int *JA, const double *AA, hmat *A)
{
	if (n <= 0 || !IA || !JA || !AA || IA[0] != 0) return FEMGPU_E_ARG;
	for (int i = 0; i < n; i++) {
		if (IA[i + 1] < IA[i]) return FEMGPU_E_ARG;
		for (int k = IA[i]; k < IA[i + 1]; k++) if (JA[k] < 0 || JA[k] >= n) return FEMGPU_E_ARG;
	}
	if (hmat_alloc(A, n, IA[n])) return FEMGPU_E_NOMEM;
	memcpy(A->ptr, IA, sizeof(int) * ((size_t)n + 1));
	memcpy(A->col, JA, sizeof(int) * (size_t)IA[n]);
	memcpy(A->val, AA, sizeof(double) * (size_t)IA[n]);
	for (int i = 0; i < n; i++)
		for (int k = IA[i]; k < IA[i + 1]; k++) if (JA[k] == i) A->diag[i] = AA[k];
	return 0;
}

int femgpu_dpa_match(int n, const int *IA, const int *JA, const double *AA, double beta, int *rmatch)
{
	hmat A = { 0 };
	int rc;
	if (!rmatch || (beta != -1.0 && !(beta >= 0.0))) return FEMGPU_E_ARG;
	if ((rc = wrap(n, IA, JA, AA, &A))) return rc;
	rc = beta == -1.0 ? match_hmatch(&A, rmatch) : match_greedy(&A, beta, rmatch);
	hmat_free(&A);
	return rc;
}

int femgpu_dpa_galerkin(int n, const int *IA, const int *JA, const double *AA, const int *rmatch, int *nc_nnz,
                        int *IC, int *JC, double *AC)
{
	hmat A = { 0 }, C = { 0 };
	int rc;
	if (!rmatch || !nc_nnz) return FEMGPU_E_ARG;
	for (int i = 0; i < n; i++)
		if (rmatch[i] < -1 || rmatch[i] >= n || (rmatch[i] >= 0 && rmatch[rmatch[i]] != i)) return FEMGPU_E_ARG;
	if ((rc = wrap(n, IA, JA, AA, &A))) return rc;
	rc = galerkin(&A, rmatch, &C);
	if (!rc) {
		nc_nnz[0] = C.n; nc_nnz[1] = C.nnz;
		if (IC) memcpy(IC, C.ptr, sizeof(int) * ((size_t)C.n + 1));
		if (JC) memcpy(JC, C.col, sizeof(int) * (size_t)C.nnz);
		if (AC) memcpy(AC, C.val, sizeof(double) * (size_t)C.nnz);
	}
	hmat_free(&A);
	hmat_free(&C);
	return rc;
}

/* ---- context ------------------------------------------------------------------ */
#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)
#define UP(dst, src, bytes) do { DM(dst, bytes); CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g->stream)); } while (0)

static void free_levels(femgpu_amg *g)
{
	for (int l = 0; l < g->nlevels; l++) {
		fg_amg_level *L = &g->lv[l];
		void *p[] = { L->ptr, L->col, L->val, L->diag, L->fw_rows, L->fw_lev, L->bw_rows, L->bw_lev,
		              L->quad, L->agg2, l ? L->f : NULL, l ? L->u : NULL };
		for (int i = 0; i < (int)(sizeof p / sizeof p[0]); i++) if (p[i]) cudaFree(p[i]);
		free(L->h_ptr); free(L->h_col); free(L->h_val); free(L->h_match);
		free(L->h_fw_lev); free(L->h_bw_lev); free(L->fw_seg); free(L->bw_seg);
	}
	free(g->lv);
	g->lv = NULL;
	g->nlevels = 0;
	if (g->qcopy) { cudaFree(g->qcopy); g->qcopy = NULL; }
}

int femgpu_amg_create(femgpu_amg **out, int ncl, double beta, double omega, int nr)
{
	femgpu_amg *g;
	if (!out || ncl < 1 || nr < 1 || !(omega > 0.0) || (beta != -1.0 && !(beta >= 0.0))) return FEMGPU_E_ARG;
	g = calloc(1, sizeof *g);
	if (!g) return FEMGPU_E_NOMEM;
	g->ncl = ncl; g->beta = beta; g->omega = omega; g->nr = nr;
	if (cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
		free(g);
		return FEMGPU_E_CUDA;
	}
	g->stream = g->own_stream;
	*out = g;
	return 0;
}

void femgpu_amg_destroy(femgpu_amg *g)
{
	if (!g) return;
	cudaStreamSynchronize(g->stream);
	free_levels(g);
	if (g->own_stream) cudaStreamDestroy(g->own_stream);
	free(g);
}

int femgpu_amg_set_stream(femgpu_amg *g, void *stream)
{
	if (!g) return FEMGPU_E_ARG;
	CK(cudaStreamSynchronize(g->stream));
	g->stream = stream ? (cudaStream_t)stream : g->own_stream;
	return 0;
}

/* Device copy of a smoothed level: CSR, diagonal, SOR schedules; f and u
 * except on level 0 (the caller's vectors). */
static int upload_level(femgpu_amg *g, int l, fg_amg_level *D, const hmat *A)
{
	int *rows, *lev, nlev, rc;
	UP(D->ptr, A->ptr, sizeof(int) * ((size_t)A->n + 1));
	UP(D->col, A->col, sizeof(int) * (size_t)(A->nnz ? A->nnz : 1));
	UP(D->val, A->val, sizeof(double) * (size_t)(A->nnz ? A->nnz : 1));
	UP(D->diag, A->diag, sizeof(double) * (size_t)A->n);
	if (l) { DM(D->f, sizeof(double) * (size_t)A->n); DM(D->u, sizeof(double) * (size_t)A->n); }
	if ((rc = sor_levels(A, 0, &rows, &lev, &nlev))) return rc;
	D->h_fw_lev = lev; D->fw_nlev = nlev;
	rc = segments(lev, nlev, &D->fw_seg, &D->fw_nseg);
	if (!rc) rc = fgh_dmalloc((void **)&D->fw_rows, sizeof(int) * (size_t)A->n);
	if (!rc) rc = fgh_dmalloc((void **)&D->fw_lev, sizeof(int) * ((size_t)nlev + 1));
	if (!rc && (cudaMemcpy(D->fw_rows, rows, sizeof(int) * (size_t)A->n, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(D->fw_lev, lev, sizeof(int) * ((size_t)nlev + 1), cudaMemcpyHostToDevice) != cudaSuccess))
		rc = FEMGPU_E_CUDA;
	free(rows);
	if (rc) return rc;
	if ((rc = sor_levels(A, 1, &rows, &lev, &nlev))) return rc;
	D->h_bw_lev = lev; D->bw_nlev = nlev;
	rc = segments(lev, nlev, &D->bw_seg, &D->bw_nseg);
	if (!rc) rc = fgh_dmalloc((void **)&D->bw_rows, sizeof(int) * (size_t)A->n);
	if (!rc) rc = fgh_dmalloc((void **)&D->bw_lev, sizeof(int) * ((size_t)nlev + 1));
	if (!rc && (cudaMemcpy(D->bw_rows, rows, sizeof(int) * (size_t)A->n, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(D->bw_lev, lev, sizeof(int) * ((size_t)nlev + 1), cudaMemcpyHostToDevice) != cudaSuccess))
		rc = FEMGPU_E_CUDA;
	free(rows);
	return rc;
}

/* Restriction and prolongation between smoothed levels l and l+2: the <= 4
 * level-l rows of each level-(l+2) row in the order dpa_fine2coarse sums
 * them, and the composite aggregate of each level-l row. */
static int upload_maps(fg_amg_level *D, const int *m0, int n0, const int *m1, int n1)
{
	int *agg0 = malloc(sizeof(int) * (size_t)n0), *agg1 = malloc(sizeof(int) * (size_t)n1);
	int *f1 = malloc(sizeof(int) * (size_t)n1), *f2 = malloc(sizeof(int) * (size_t)n1);
	int nc1 = n0 - m0[n0], nc2 = n1 - m1[n1], j, rc = 0;
	int4 *quad = malloc(sizeof(int4) * (size_t)(nc2 ? nc2 : 1));
	if (!agg0 || !agg1 || !f1 || !f2 || !quad) rc = FEMGPU_E_NOMEM;
	if (!rc) {
		for (int i = 0, k = 0; i < n0; i++) {          /* level l -> l+1, first/second members */
			if (m0[i] == -1) { agg0[i] = k; f1[k] = i; f2[k] = -1; k++; }
			else if (i < m0[i]) { agg0[i] = agg0[m0[i]] = k; f1[k] = i; f2[k] = m0[i]; k++; }
		}
		for (int i = 0, k = 0; i < n1; i++) {          /* level l+1 -> l+2 */
			int a = -1, b = -1;
			if (m1[i] == -1) a = i;
			else if (i < m1[i]) { a = i; b = m1[i]; }
			else continue;
			agg1[a] = k;
			if (b >= 0) agg1[b] = k;
			quad[k].x = f1[a]; quad[k].y = f2[a];
			quad[k].z = b >= 0 ? f1[b] : -1; quad[k].w = b >= 0 ? f2[b] : -1;
			k++;
		}
		for (j = 0; j < n0; j++) agg0[j] = agg1[agg0[j]];
		(void)nc1;
		D->nc2 = nc2;
		if (fgh_dmalloc((void **)&D->quad, sizeof(int4) * (size_t)(nc2 ? nc2 : 1)) ||
		    fgh_dmalloc((void **)&D->agg2, sizeof(int) * (size_t)n0) ||
		    cudaMemcpy(D->quad, quad, sizeof(int4) * (size_t)nc2, cudaMemcpyHostToDevice) != cudaSuccess ||
		    cudaMemcpy(D->agg2, agg0, sizeof(int) * (size_t)n0, cudaMemcpyHostToDevice) != cudaSuccess)
			rc = FEMGPU_E_CUDA;
	}
	free(agg0); free(agg1); free(f1); free(f2); free(quad);
	return rc;
}

/* dpa_setup (amg_dpa.c:424-463) on a host CSR matrix, then the device copy. */
int femgpu_amg_setup(femgpu_amg *g, int n, const int *IA, const int *JA, const double *AA)
{
	int L, l, rc = 0;
	hmat *H;
	if (!g || n <= 0 || !IA || !JA || !AA || IA[0] != 0 || IA[n] < 0) return FEMGPU_E_ARG;
	for (int i = 0; i < n; i++) {
		if (IA[i + 1] < IA[i]) return FEMGPU_E_ARG;
		for (int k = IA[i]; k < IA[i + 1]; k++) if (JA[k] < 0 || JA[k] >= n) return FEMGPU_E_ARG;
	}
	L = 2 * g->ncl + 1;
	CK(cudaStreamSynchronize(g->stream));
	free_levels(g);
	H = calloc((size_t)L, sizeof(hmat));
	g->lv = calloc((size_t)L, sizeof(fg_amg_level));
	if (!H || !g->lv) { free(H); return FEMGPU_E_NOMEM; }
	g->nlevels = L;
	rc = hmat_alloc(&H[0], n, IA[n]);
	if (!rc) {
		memcpy(H[0].ptr, IA, sizeof(int) * ((size_t)n + 1));
		memcpy(H[0].col, JA, sizeof(int) * (size_t)IA[n]);
		memcpy(H[0].val, AA, sizeof(double) * (size_t)IA[n]);
		for (int i = 0; i < n; i++)                    /* amg_precond.c:80-83 */
			for (int k = IA[i]; k < IA[i + 1]; k++) if (JA[k] == i) H[0].diag[i] = AA[k];
	}
	for (l = 0; l < L - 1 && !rc; l++) {
		int *rm = malloc(sizeof(int) * ((size_t)H[l].n + 1));
		if (!rm) { rc = FEMGPU_E_NOMEM; break; }
		g->lv[l].h_match = rm;
		rc = g->beta == -1.0 ? match_hmatch(&H[l], rm) : match_greedy(&H[l], g->beta, rm);
		if (!rc) rc = galerkin(&H[l], rm, &H[l + 1]);
	}
	for (l = 0; l < L && !rc; l++) {
		fg_amg_level *D = &g->lv[l];
		D->n = H[l].n; D->nnz = H[l].nnz;
		if (!(l & 1)) rc = upload_level(g, l, D, &H[l]);
		if (!rc && !(l & 1) && l < L - 1)
			rc = upload_maps(D, g->lv[l].h_match, H[l].n, g->lv[l + 1].h_match, H[l + 1].n);
		D->h_ptr = H[l].ptr; D->h_col = H[l].col; D->h_val = H[l].val;     /* kept for inspection */
		H[l].ptr = NULL; H[l].col = NULL; H[l].val = NULL;
	}
	if (!rc) rc = fgh_dmalloc((void **)&g->qcopy, sizeof(double) * (size_t)n);
	if (!rc && cudaStreamSynchronize(g->stream) != cudaSuccess) rc = FEMGPU_E_CUDA;
	for (l = 0; l < L; l++) { free(H[l].ptr); free(H[l].col); free(H[l].val); free(H[l].diag); }
	free(H);
	if (rc) free_levels(g);
	return rc;
}

int femgpu_amg_levels(const femgpu_amg *g) { return g ? g->nlevels : FEMGPU_E_ARG; }

int femgpu_amg_level(const femgpu_amg *g, int l, int *n_nnz, int *IA, int *JA, double *AA, int *rmatch)
{
	const fg_amg_level *D;
	if (!g || l < 0 || l >= g->nlevels || !n_nnz) return FEMGPU_E_ARG;
	D = &g->lv[l];
	n_nnz[0] = D->n; n_nnz[1] = D->nnz;
	if (IA) memcpy(IA, D->h_ptr, sizeof(int) * ((size_t)D->n + 1));
	if (JA) memcpy(JA, D->h_col, sizeof(int) * (size_t)D->nnz);
	if (AA) memcpy(AA, D->h_val, sizeof(double) * (size_t)D->nnz);
	if (rmatch && D->h_match) memcpy(rmatch, D->h_match, sizeof(int) * ((size_t)D->n + 1));
	return 0;
}

int femgpu_amg_apply_dev(femgpu_amg *g, const double *q, double *z)
{
	if (!g || !q || !z) return FEMGPU_E_ARG;
	if (!g->nlevels) { fgh_set_error("AMG apply before setup"); return FEMGPU_E_NOT_BUILT; }
	KR(fg_amg_vcycle(g, q, z, NULL));
	return 0;
}

int femgpu_amg_apply(femgpu_amg *g, const double *q_host, double *z_host)
{
	double *q = NULL, *z = NULL;
	int rc, n;
	if (!g || !q_host || !z_host || !g->nlevels) return FEMGPU_E_ARG;
	n = g->lv[0].n;
	if ((rc = fgh_dmalloc((void **)&q, sizeof(double) * (size_t)n)) ||
	    (rc = fgh_dmalloc((void **)&z, sizeof(double) * (size_t)n)))
		return rc;
	CK(cudaMemcpyAsync(q, q_host, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, g->stream));
	rc = femgpu_amg_apply_dev(g, q, z);
	if (!rc) CK(cudaMemcpyAsync(z_host, z, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g->stream));
	CK(cudaStreamSynchronize(g->stream));
	cudaFree(q);
	cudaFree(z);
	return rc;
}
