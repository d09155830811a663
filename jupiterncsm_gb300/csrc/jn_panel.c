/*
 * jn_panel.c — host side of the panel engine: panels, warp tasks, the
 * persistent-CTA schedule and the coefficient compaction (see jn_problem.h).
 *
 * The semantics are those of the reference kernels
 * (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:
 * n list :20-77, p list :79-132, n x p lists :134-210, off-diagonal
 * transposes :212-462); the order in which contributions are added does not
 * matter because the device sums them as exact 64-bit integers.
 */
#define _GNU_SOURCE        /* qsort_r */
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jn_problem.h"

#define ERR(...) do { snprintf(err, errlen, __VA_ARGS__); goto fail; } while (0)

void jn_panels_free(jn_plan_t *p)
{
	free(p->panels); free(p->ptasks); free(p->pcta); free(p->pflush_ptr); free(p->pflush); free(p->pmeta); free(p->pblocks);
	free(p->pperm);
	p->panels = NULL; p->ptasks = NULL; p->pcta = NULL; p->pflush_ptr = NULL; p->pflush = NULL; p->pmeta = NULL;
	p->pblocks = NULL; p->pperm = NULL;
	p->npanels = 0; p->nptasks = 0; p->pgrid = 0; p->npflush = 0; p->n_pmeta = 0; p->n_coef = 0; p->psmem_words = 0;
}

/* lanes per row: a narrow panel puts floor(32 / ncols) rows side by side */
static int lanes_per_row(int ncols) { return ncols < 32 ? ncols : 32; }

/* Column chunks of a panel: 32-column chunks, then the rest.  A chunk of w
 * columns runs floor(32 / w) rows side by side in a warp; when that leaves
 * more than an eighth of the lanes idle, the largest power of two below w is
 * split off as its own chunk (its rows fill the warp exactly) and the rest
 * is chunked the same way.  Chunk k starts at column i0[k] and is cw[k]
 * wide; returns the number of chunks after the 32-column ones (at most 6),
 * whose count is ncols / 32. */
static int tail_chunks(int ncols, int *i0, int *cw)
{
	int n = 0, at = ncols - ncols % 32, w = ncols % 32;
	while (w > 0) {
		if (8 * (w * (32 / w)) >= 7 * 32) { i0[n] = at; cw[n++] = w; break; }
		int p = 1;
		while (2 * p < w) p *= 2;
		i0[n] = at; cw[n++] = p;
		at += p;
		w -= p;
	}
	return n;
}

/* The order of a list's entries in every panel that uses the list.  A warp
 * adds the contributions of up to 32 consecutive rows at once (narrow
 * panels put several rows side by side), and each 32-column chunk of a wide
 * panel is one set of entries.  Lanes whose contributions land on the same
 * shared-memory word serialise, and in by-out order equal destinations sit
 * next to each other.  So the entries are dealt out greedily: the
 * destination with the most entries left among those not used in the last
 * LIST_GAP - 1 positions (a repeat only when none is left), and within it the
 * first entry whose source was not used in that window either (else the one
 * used longest ago).  On the 4He Nmax 6 two- plus three-body workload this
 * halves the shared-memory wavefronts of the product's atomics.  The sums
 * are exact integers, so the order never changes a result bit.
 *
 * m: the list's packed entries (source | destination << 16) in by-out
 * order; writes perm[k] = the by-out index of the entry at position k.
 * last_src: 65 536 positions in the running count *clock, which advances
 * past each list so that no state carries over. */
#define LIST_GAP 32
typedef struct { int64_t *last_src; int64_t clock; int32_t *run0, *left, *heap, *queue; int64_t *release; } list_order_t;

static int heap_before(const int32_t *left, int32_t a, int32_t b) { return left[a] != left[b] ? left[a] > left[b] : a < b; }
static void heap_push(int32_t *h, int *nh, const int32_t *left, int32_t r)
{
	int k = (*nh)++;
	h[k] = r;
	while (k > 0 && heap_before(left, h[k], h[(k - 1) / 2])) { int32_t t = h[k]; h[k] = h[(k - 1) / 2]; h[(k - 1) / 2] = t; k = (k - 1) / 2; }
}
static int32_t heap_pop(int32_t *h, int *nh, const int32_t *left)
{
	const int32_t top = h[0];
	h[0] = h[--(*nh)];
	for (int k = 0;;) {
		int c = 2 * k + 1;
		if (c >= *nh) break;
		if (c + 1 < *nh && heap_before(left, h[c + 1], h[c])) c++;
		if (!heap_before(left, h[c], h[k])) break;
		int32_t t = h[k]; h[k] = h[c]; h[c] = t; k = c;
	}
	return top;
}

static void list_order(const uint32_t *m, int64_t n, uint32_t *perm, list_order_t *w)
{
	/* runs of equal destination; a run's entries not yet placed are kept in perm-sized scratch: run r owns
	   [run0[r], run0[r] + left[r]) of `rest`, which starts as the by-out indices */
	int32_t nr = 0;
	for (int64_t e = 0; e < n; e++)
		if (e == 0 || (m[e] >> 16) != (m[e - 1] >> 16)) w->run0[nr++] = (int32_t)e;
	for (int32_t r = 0; r < nr; r++) w->left[r] = (int32_t)((r + 1 < nr ? w->run0[r + 1] : n) - w->run0[r]);
	int32_t *rest = w->heap + nr;   /* n slots after the heap's nr */
	for (int64_t e = 0; e < n; e++) rest[e] = (int32_t)e;
	int nh = 0, q0 = 0, q1 = 0;
	for (int32_t r = 0; r < nr; r++) heap_push(w->heap, &nh, w->left, r);
	const int64_t base = w->clock;
	for (int64_t k = 0; k < n; k++) {
		const int64_t now = base + k;
		while (q0 < q1 && w->release[q0] <= now) heap_push(w->heap, &nh, w->left, w->queue[q0++]);
		const int32_t r = nh ? heap_pop(w->heap, &nh, w->left) : w->queue[q0++];
		int32_t *s = rest + w->run0[r];
		int best = 0;
		for (int a = 0; a < w->left[r]; a++) {
			const int64_t t = w->last_src[m[s[a]] & 0xffffu];
			if (now - t >= LIST_GAP) { best = a; break; }
			if (t < w->last_src[m[s[best]] & 0xffffu]) best = a;
		}
		const int32_t e = s[best];
		memmove(s + best, s + best + 1, (size_t)(w->left[r] - best - 1) * sizeof(int32_t));
		w->left[r]--;
		perm[k] = (uint32_t)e;
		w->last_src[m[e] & 0xffffu] = now;
		if (w->left[r] > 0) { w->queue[q1] = r; w->release[q1++] = now + LIST_GAP; }
	}
	w->clock = base + n + LIST_GAP;
}

static double task_cost(const jn_plan_t *p, const uint32_t *T)
{
	const int R = 32 / (int)(T[3] >> 24);
	const int diag = (p->panels[T[0]].kind & JN_PANEL_DIAG) != 0;
	return (double)((T[2] - T[1] + R - 1) / R) * (diag ? 1.0 : 2.0) + 4.0;
}

/* qsort_r comparators: the plan comes with the call, so concurrent panel
 * builds share no state */
static int cmp_task_cost(const void *a, const void *b, void *plan)
{
	const jn_plan_t *p = (const jn_plan_t *)plan;
	const double ca = task_cost(p, a), cb = task_cost(p, b);
	if (ca != cb) return ca > cb ? -1 : 1;
	return memcmp(a, b, 4 * sizeof(uint32_t));
}

/* panels sorted by (output block, input block) so that a CTA's run of tasks touches few blocks */
static int cmp_panel(const void *a, const void *b, void *plan)
{
	const jn_plan_t *p = (const jn_plan_t *)plan;
	const jn_instr_t *x = &p->instr[*(const int *)a], *y = &p->instr[*(const int *)b];
	if (x->bout != y->bout) return x->bout < y->bout ? -1 : 1;
	if (x->bin != y->bin) return x->bin < y->bin ? -1 : 1;
	return *(const int *)a - *(const int *)b;
}

int jn_panels_build(jn_plan_t *p, int grid, int iter, char *err, size_t errlen)
{
	int *order = NULL;
	jn_panels_free(p);
	if (p->dim > JN_PANEL_MAX_DIM) ERR("dimension %lld is above the panel engine's %d", (long long)p->dim, JN_PANEL_MAX_DIM);
	if (grid < 1) ERR("panel grid of %d CTAs", grid);
	if (iter < 1 || iter > 4096) ERR("panel tasks of %d rows per lane", iter);
	/* accumulator layout: block rows padded to an odd length, so that a warp
	   walking a column (stride Nn) hits 32 different shared-memory banks */
	p->pblocks = malloc((p->nblocks ? p->nblocks : 1) * 4 * sizeof(uint32_t));
	if (!p->pblocks) ERR("out of host memory");
	p->psmem_words = 0;
	for (int b = 0; b < p->nblocks; b++) {
		const jn_block_t *B = &p->blocks[b];
		p->pblocks[4 * b] = (uint32_t)B->offset;
		p->pblocks[4 * b + 1] = (uint32_t)p->psmem_words;
		p->pblocks[4 * b + 2] = (uint32_t)B->Np;
		p->pblocks[4 * b + 3] = (uint32_t)B->Nn;
		p->psmem_words += B->Np * (B->Nn | 1);
	}
	/* packed list entries, by-out order: source | destination << 16 */
	p->n_pmeta = 0;
	for (int l = 0; l < p->nlists; l++) {
		p->lists[l].pmeta = p->n_pmeta;
		p->n_pmeta += p->lists[l].len;
	}
	if (p->n_pmeta > 0xffffffffll) ERR("index lists too long for the panel engine");
	p->pmeta = malloc((p->n_pmeta ? p->n_pmeta : 1) * sizeof(uint32_t));
	p->pperm = malloc((p->n_pmeta ? p->n_pmeta : 1) * sizeof(uint32_t));
	if (!p->pmeta || !p->pperm) ERR("out of host memory");
	{
		int64_t lmax = 1;
		for (int l = 0; l < p->nlists; l++) lmax = p->lists[l].len > lmax ? p->lists[l].len : lmax;
		list_order_t w = {0};
		uint32_t *bym = malloc((size_t)lmax * sizeof(uint32_t));
		w.last_src = malloc(65536 * sizeof(int64_t));
		w.run0 = malloc((size_t)lmax * sizeof(int32_t));
		w.left = malloc((size_t)lmax * sizeof(int32_t));
		w.heap = malloc((size_t)(2 * lmax) * sizeof(int32_t));
		w.queue = malloc((size_t)lmax * sizeof(int32_t));
		w.release = malloc((size_t)lmax * sizeof(int64_t));
		const int ok = bym && w.last_src && w.run0 && w.left && w.heap && w.queue && w.release;
		if (ok) {
			for (int s = 0; s < 65536; s++) w.last_src[s] = -(int64_t)LIST_GAP;
			w.clock = 0;
			for (int l = 0; l < p->nlists; l++) {
				const jn_list_t *L = &p->lists[l];
				for (int64_t e = 0; e < L->len; e++) bym[e] = p->ent[2 * (L->ent_out + e)];
				list_order(bym, L->len, p->pperm + L->pmeta, &w);
				for (int64_t k = 0; k < L->len; k++) p->pmeta[L->pmeta + k] = bym[p->pperm[L->pmeta + k]];
			}
		}
		free(bym); free(w.last_src); free(w.run0); free(w.left); free(w.heap); free(w.queue); free(w.release);
		if (!ok) ERR("out of host memory");
	}
	/* panels */
	order = malloc((p->ninstr ? p->ninstr : 1) * sizeof(int));
	for (int i = 0; i < p->ninstr; i++) order[i] = i;
	qsort_r(order, p->ninstr, sizeof(int), cmp_panel, p);
	p->panels = calloc(p->ninstr ? p->ninstr : 1, sizeof(jn_panel_t));
	if (!order || !p->panels) ERR("out of host memory");
	int64_t coef = 0, ntask = 0;
	for (int q = 0; q < p->ninstr; q++) {
		const jn_instr_t *x = &p->instr[order[q]];
		const jn_block_t *bi = &p->blocks[x->bin], *bo = &p->blocks[x->bout];
		jn_panel_t *P = &p->panels[q];
		P->c_off = coef;
		P->instr = order[q];
		P->out_off = (int32_t)bo->offset;
		P->in_off = (int32_t)bi->offset;
		P->Nn_out = (int32_t)bo->Nn;
		P->Nn_in = (int32_t)bi->Nn;
		P->Np_out = (int32_t)bo->Np;
		P->Np_in = (int32_t)bi->Np;
		P->out_blk = x->bout;
		P->in_blk = x->bin;
		P->kind = x->kind | (x->bin == x->bout ? JN_PANEL_DIAG : 0);
		const jn_list_t *Ln = x->ln >= 0 ? &p->lists[x->ln] : NULL, *Lp = x->lp >= 0 ? &p->lists[x->lp] : NULL;
		if (x->kind == JN_KIND_NP) {
			const int rows_n = Ln->len > Lp->len;
			P->nrows = (int32_t)(rows_n ? Ln->len : Lp->len);
			P->ncols = (int32_t)(rows_n ? Lp->len : Ln->len);
			if (rows_n) P->kind |= JN_PANEL_ROWS_N;
			coef += (int64_t)P->nrows * P->ncols;
		} else if (x->kind == JN_KIND_N) {
			P->nrows = (int32_t)bo->Np;
			P->ncols = (int32_t)Ln->len;
			coef += P->ncols;
		} else {
			P->nrows = (int32_t)Lp->len;
			P->ncols = (int32_t)bo->Nn;
			coef += P->nrows;
		}
		P->row_meta = Lp ? (uint32_t)Lp->pmeta : 0;
		P->col_meta = Ln ? (uint32_t)Ln->pmeta : 0;
		if (P->kind & JN_PANEL_ROWS_N) {
			P->row_meta = (uint32_t)Ln->pmeta;
			P->col_meta = (uint32_t)Lp->pmeta;
		}
		if (x->kind == JN_KIND_N && P->nrows > 65535) ERR("instruction %d: %d spectator rows", order[q], P->nrows);
		if (P->nrows > 0 && P->ncols > 0) {
			int ci[8], cwv[8];
			const int nc = tail_chunks(P->ncols, ci, cwv);
			ntask += (int64_t)(P->ncols / 32) * ((P->nrows + iter - 1) / iter);
			for (int k = 0; k < nc; k++) {
				const int64_t rows_per_task = (int64_t)(32 / cwv[k]) * iter;
				ntask += (P->nrows + rows_per_task - 1) / rows_per_task;
			}
		}
	}
	p->npanels = p->ninstr;
	p->n_coef = coef;
	p->nptasks = ntask;
	p->ptasks = malloc((ntask ? ntask : 1) * 4 * sizeof(uint32_t));
	if (!p->ptasks) ERR("out of host memory");
	int64_t t = 0;
	for (int q = 0; q < p->npanels; q++) {
		const jn_panel_t *P = &p->panels[q];
		if (P->nrows <= 0 || P->ncols <= 0) continue;
		int ci[8], cwv[8];
		const int nt = tail_chunks(P->ncols, ci, cwv), nfull = P->ncols / 32;
		for (int k = 0; k < nfull + nt; k++) {
			const int cw = k < nfull ? 32 : cwv[k - nfull], R = 32 / cw, i0 = k < nfull ? 32 * k : ci[k - nfull];
			const int64_t rows_per_task = (int64_t)R * iter;
			for (int64_t j0 = 0; j0 < P->nrows; j0 += rows_per_task) {
				const int64_t j1 = j0 + rows_per_task < P->nrows ? j0 + rows_per_task : P->nrows;
				uint32_t *T = p->ptasks + 4 * t;
				T[0] = (uint32_t)q;
				T[1] = (uint32_t)j0;
				T[2] = (uint32_t)j1;
				T[3] = (uint32_t)i0 | ((uint32_t)cw << 24);
				t++;
			}
		}
	}
	p->pgrid = grid;
	if (jn_panels_partition(p, grid, &p->pcta, &p->pflush_ptr, &p->pflush, &p->npflush, &p->pcta_words))
		ERR("out of host memory");
	/* within each CTA's run, heaviest tasks first: the warps that finish last
	   then finish with small tasks (the order never changes a result bit) */
	for (int b = 0; b < grid; b++) {
		qsort_r(p->ptasks + 4 * (size_t)p->pcta[b], p->pcta[b + 1] - p->pcta[b], 4 * sizeof(uint32_t), cmp_task_cost, p);
	}
	/* every device index stays inside its buffer: checked once here */
	for (int q = 0; q < p->npanels; q++) {
		const jn_panel_t *P = &p->panels[q];
		const jn_instr_t *x = &p->instr[P->instr];
		const jn_block_t *bi = &p->blocks[x->bin], *bo = &p->blocks[x->bout];
		if ((x->kind != JN_KIND_N && (int64_t)P->row_meta + P->nrows > p->n_pmeta) ||
		    (x->kind != JN_KIND_P && (int64_t)P->col_meta + P->ncols > p->n_pmeta))
			ERR("panel %d: list entries out of range", q);
		if (x->kind == JN_KIND_NP && (int64_t)P->nrows * P->ncols != (int64_t)p->lists[x->ln].len * p->lists[x->lp].len)
			ERR("panel %d: shape", q);
		if (x->kind == JN_KIND_N && (bi->Np != bo->Np)) ERR("panel %d: spectator rows differ", q);
		if (x->kind == JN_KIND_P && (bi->Nn != bo->Nn)) ERR("panel %d: spectator columns differ", q);
	}
	free(order);
	return 0;
fail:
	free(order);
	jn_panels_free(p);
	return 1;
}

int jn_panels_partition(const jn_plan_t *p, int grid, uint32_t **cta_out, uint32_t **flush_ptr_out,
			uint32_t **flush_out, int64_t *nflush_out, int64_t *words_out)
{
	int64_t words_max = 0;
	const int64_t ntask = p->nptasks;
	uint32_t *cta = malloc((size_t)(grid + 1) * sizeof(uint32_t));
	uint32_t *fptr = malloc((size_t)(grid + 1) * sizeof(uint32_t));
	double *cost = malloc((ntask ? ntask : 1) * sizeof(double));
	unsigned char *touched = calloc(p->nblocks ? p->nblocks : 1, 1);
	size_t fcap = 1024;
	int64_t nf = 0;
	uint32_t *flush = malloc(fcap * sizeof(uint32_t));
	if (grid < 1 || !cta || !fptr || !cost || !touched || !flush) goto fail;
	double total = 0;
	for (int64_t k = 0; k < ntask; k++) {
		cost[k] = task_cost(p, p->ptasks + 4 * k);
		total += cost[k];
	}
	/* persistent CTAs: contiguous runs of tasks of equal cost */
	{
		double acc = 0;
		int64_t k = 0;
		cta[0] = 0;
		for (int b = 1; b <= grid; b++) {
			const double target = total * b / grid;
			while (k < ntask && acc + 0.5 * cost[k] < target) acc += cost[k++];
			cta[b] = (uint32_t)(b == grid ? ntask : k);
		}
	}
	/* the blocks each CTA touches (forward into the output block, transpose
	   into the input block), each at its place in the CTA's own accumulator:
	   rows padded to Nn | 1, blocks one after another */
	for (int b = 0; b < grid; b++) {
		fptr[b] = (uint32_t)nf;
		memset(touched, 0, p->nblocks);
		for (uint32_t k = cta[b]; k < cta[b + 1]; k++) {
			const jn_instr_t *x = &p->instr[p->panels[p->ptasks[4 * k]].instr];
			touched[x->bout] = 1;
			if (x->bin != x->bout) touched[x->bin] = 1;
		}
		int64_t words = 0;
		for (int i = 0; i < p->nblocks; i++) {
			if (!touched[i] || p->blocks[i].Np <= 0 || p->blocks[i].Nn <= 0) continue;
			if ((size_t)(2 * nf + 2) > fcap) {
				fcap *= 2;
				uint32_t *g = realloc(flush, fcap * sizeof(uint32_t));
				if (!g) goto fail;
				flush = g;
			}
			flush[2 * nf] = (uint32_t)i;
			flush[2 * nf + 1] = (uint32_t)words;
			nf++;
			words += p->blocks[i].Np * (p->blocks[i].Nn | 1);
		}
		if (words > words_max) words_max = words;
	}
	fptr[grid] = (uint32_t)nf;
	free(cost); free(touched);
	*cta_out = cta; *flush_ptr_out = fptr; *flush_out = flush; *nflush_out = nf;
	if (words_out) *words_out = words_max;
	return 0;
fail:
	free(cta); free(fptr); free(cost); free(touched); free(flush);
	return 1;
}

void jn_panels_coefficients(const jn_plan_t *p, const double *me, double *c64, float *c32)
{
	for (int q = 0; q < p->npanels; q++) {
		const jn_panel_t *P = &p->panels[q];
		const jn_instr_t *x = &p->instr[P->instr];
		const jn_me_t *M = &p->mes[x->me];
		const double *m = me + M->offset;
		const uint32_t *ent = p->ent;
		if (x->kind == JN_KIND_NP) {
			const jn_list_t *Ln = &p->lists[x->ln], *Lp = &p->lists[x->lp];
			const int rows_n = (P->kind & JN_PANEL_ROWS_N) != 0;
			for (int32_t j = 0; j < P->nrows; j++)
				for (int32_t i = 0; i < P->ncols; i++) {
					const int32_t ep = rows_n ? i : j, en = rows_n ? j : i;
					const uint32_t mp = ent[2 * (Lp->ent_out + p->pperm[Lp->pmeta + ep]) + 1];
					const uint32_t mn = ent[2 * (Ln->ent_out + p->pperm[Ln->pmeta + en]) + 1];
					double v = m[(mn & 0x7fffffffu) + (int64_t)M->nd_n * (mp & 0x7fffffffu)];
					if ((mp ^ mn) & 0x80000000u) v = -v;
					const int64_t at = P->c_off + (int64_t)j * P->ncols + i;
					if (c64) c64[at] = v;
					if (c32) c32[at] = (float)v;
				}
		} else {
			const jn_list_t *L = &p->lists[x->kind == JN_KIND_N ? x->ln : x->lp];
			for (int64_t e = 0; e < L->len; e++) {
				const uint32_t mi = ent[2 * (L->ent_out + p->pperm[L->pmeta + e]) + 1];
				double v = m[mi & 0x7fffffffu];
				/* single-species terms skip |M| < 1e-12 (matrix_vector_multiplication.c:52-53) */
				if (fabs(v) < 1e-12) v = 0.0;
				if (mi & 0x80000000u) v = -v;
				if (c64) c64[P->c_off + e] = v;
				if (c32) c32[P->c_off + e] = (float)v;
			}
		}
	}
}

int jn_panels_coefficients_int(const jn_plan_t *p, const double *me, int32_t *ci, int *Sc, int *k)
{
	double *c = malloc((p->n_coef ? p->n_coef : 1) * sizeof(double));
	if (!c) return 1;
	jn_panels_coefficients(p, me, c, NULL);
	double cmax = 0.0;
	for (int64_t e = 0; e < p->n_coef; e++) cmax = fmax(cmax, fabs(c[e]));
	int ec = 0, eb = 0;
	if (cmax > 0.0) frexp(cmax, &ec);               /* cmax < 2^ec */
	*Sc = cmax > 0.0 ? 30 - ec : 0;
	if (p->abs_bound > 0.0) frexp(p->abs_bound, &eb); /* abs_bound < 2^eb */
	/* |c_int x_int| <= 2^60: the shift 30 rounds every product to a 32-bit
	   integer (|v| <= 2^30), whose 64-bit addition mostly touches only the low
	   word (the high word takes a carry about |v| / 2^32 of the time); element sums stay below
	   2^62 as long as sum |c_int x_int| < abs_bound 2^Sc 2^30 stays below
	   2^(61 + k), which a larger shift guarantees where needed */
	*k = 30;
	if (p->abs_bound > 0.0 && eb + *Sc - 31 > *k) *k = eb + *Sc - 31;
	for (int64_t e = 0; e < p->n_coef; e++) ci[e] = (int32_t)llrint(ldexp(c[e], *Sc));
	free(c);
	return 0;
}

void jn_panels_gather_index(const jn_plan_t *p, uint32_t *gather)
{
	const uint32_t *ent = p->ent;
	for (int q = 0; q < p->npanels; q++) {
		const jn_panel_t *P = &p->panels[q];
		const jn_instr_t *x = &p->instr[P->instr];
		const jn_me_t *M = &p->mes[x->me];
		if (x->kind == JN_KIND_NP) {
			const jn_list_t *Ln = &p->lists[x->ln], *Lp = &p->lists[x->lp];
			const int rows_n = (P->kind & JN_PANEL_ROWS_N) != 0;
			for (int32_t j = 0; j < P->nrows; j++)
				for (int32_t i = 0; i < P->ncols; i++) {
					const int32_t ep = rows_n ? i : j, en = rows_n ? j : i;
					const uint32_t mp = ent[2 * (Lp->ent_out + p->pperm[Lp->pmeta + ep]) + 1];
					const uint32_t mn = ent[2 * (Ln->ent_out + p->pperm[Ln->pmeta + en]) + 1];
					const uint64_t at = (uint64_t)M->offset + (mn & 0x7fffffffu) + M->nd_n * (mp & 0x7fffffffu);
					gather[P->c_off + (int64_t)j * P->ncols + i] = (uint32_t)at | ((mp ^ mn) & 0x80000000u);
				}
		} else {
			const jn_list_t *L = &p->lists[x->kind == JN_KIND_N ? x->ln : x->lp];
			for (int64_t e = 0; e < L->len; e++) {
				const uint32_t mi = ent[2 * (L->ent_out + p->pperm[L->pmeta + e]) + 1];
				gather[P->c_off + e] = (uint32_t)(M->offset + (mi & 0x7fffffffu)) | (mi & 0x80000000u) | 0x40000000u;
			}
		}
	}
}
