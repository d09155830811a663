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
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jn_problem.h"

#define ERR(...) do { snprintf(err, errlen, __VA_ARGS__); goto fail; } while (0)

void jn_panels_free(jn_plan_t *p)
{
	free(p->panels); free(p->ptasks); free(p->pcta); free(p->pflush_ptr); free(p->pflush); free(p->pmeta);
	p->panels = NULL; p->ptasks = NULL; p->pcta = NULL; p->pflush_ptr = NULL; p->pflush = NULL; p->pmeta = NULL;
	p->npanels = 0; p->nptasks = 0; p->pgrid = 0; p->npflush = 0; p->n_pmeta = 0; p->n_coef = 0;
}

static int lanes_log2(int ncols)
{
	int lg = 0;
	while ((1 << lg) < ncols && lg < 5) lg++;
	return lg;
}

/* panels sorted by (output block, input block) so that a CTA's run of tasks touches few blocks */
static const jn_plan_t *g_sort_plan;
static int cmp_panel(const void *a, const void *b)
{
	const jn_instr_t *x = &g_sort_plan->instr[*(const int *)a], *y = &g_sort_plan->instr[*(const int *)b];
	if (x->bout != y->bout) return x->bout < y->bout ? -1 : 1;
	if (x->bin != y->bin) return x->bin < y->bin ? -1 : 1;
	return *(const int *)a - *(const int *)b;
}

int jn_panels_build(jn_plan_t *p, int grid, char *err, size_t errlen)
{
	int *order = NULL;
	double *cost = NULL;
	unsigned char *touched = NULL;
	jn_panels_free(p);
	if (p->dim > JN_PANEL_MAX_DIM) ERR("dimension %lld is above the panel engine's %d", (long long)p->dim, JN_PANEL_MAX_DIM);
	if (grid < 1) ERR("panel grid of %d CTAs", grid);
	/* packed list entries, by-out order: source | destination << 16 */
	p->n_pmeta = 0;
	for (int l = 0; l < p->nlists; l++) {
		p->lists[l].pmeta = p->n_pmeta;
		p->n_pmeta += p->lists[l].len;
	}
	if (p->n_pmeta > 0xffffffffll) ERR("index lists too long for the panel engine");
	p->pmeta = malloc((p->n_pmeta ? p->n_pmeta : 1) * sizeof(uint32_t));
	if (!p->pmeta) ERR("out of host memory");
	for (int l = 0; l < p->nlists; l++) {
		const jn_list_t *L = &p->lists[l];
		for (int64_t e = 0; e < L->len; e++) p->pmeta[L->pmeta + e] = p->ent[2 * (L->ent_out + e)];
	}
	/* panels */
	order = malloc((p->ninstr ? p->ninstr : 1) * sizeof(int));
	for (int i = 0; i < p->ninstr; i++) order[i] = i;
	g_sort_plan = p;
	qsort(order, p->ninstr, sizeof(int), cmp_panel);
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
		P->kind = x->kind | (x->bin == x->bout ? JN_PANEL_DIAG : 0);
		const jn_list_t *Ln = x->ln >= 0 ? &p->lists[x->ln] : NULL, *Lp = x->lp >= 0 ? &p->lists[x->lp] : NULL;
		if (x->kind == JN_KIND_NP) {
			P->nrows = (int32_t)Lp->len;
			P->ncols = (int32_t)Ln->len;
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
		if (P->nrows > 0 && P->ncols > 0) {
			const int lg = lanes_log2(P->ncols), R = 32 >> lg;
			const int64_t rows_per_task = (int64_t)R * JN_PANEL_ITER;
			ntask += ((P->ncols + 31) / 32) * ((P->nrows + rows_per_task - 1) / rows_per_task);
		}
	}
	p->npanels = p->ninstr;
	p->n_coef = coef;
	p->nptasks = ntask;
	p->ptasks = malloc((ntask ? ntask : 1) * 4 * sizeof(uint32_t));
	cost = malloc((ntask ? ntask : 1) * sizeof(double));
	if (!p->ptasks || !cost) ERR("out of host memory");
	int64_t t = 0;
	for (int q = 0; q < p->npanels; q++) {
		const jn_panel_t *P = &p->panels[q];
		if (P->nrows <= 0 || P->ncols <= 0) continue;
		const int lg = lanes_log2(P->ncols), R = 32 >> lg;
		const int64_t rows_per_task = (int64_t)R * JN_PANEL_ITER;
		const int diag = (P->kind & JN_PANEL_DIAG) != 0;
		for (int i0 = 0; i0 < P->ncols; i0 += 32)
			for (int64_t j0 = 0; j0 < P->nrows; j0 += rows_per_task) {
				const int64_t j1 = j0 + rows_per_task < P->nrows ? j0 + rows_per_task : P->nrows;
				uint32_t *T = p->ptasks + 4 * t;
				T[0] = (uint32_t)q;
				T[1] = (uint32_t)j0;
				T[2] = (uint32_t)j1;
				T[3] = (uint32_t)i0 | ((uint32_t)lg << 24);
				/* warp time: one pass per R rows, the transpose doubles the work, plus set-up */
				cost[t] = (double)((j1 - j0 + R - 1) / R) * (diag ? 1.0 : 1.7) + 6.0;
				t++;
			}
	}
	/* persistent CTAs: contiguous runs of tasks of equal cost */
	p->pgrid = grid;
	p->pcta = malloc((size_t)(grid + 1) * sizeof(uint32_t));
	if (!p->pcta) ERR("out of host memory");
	double total = 0;
	for (int64_t k = 0; k < ntask; k++) total += cost[k];
	{
		double acc = 0;
		int64_t k = 0;
		p->pcta[0] = 0;
		for (int b = 1; b <= grid; b++) {
			const double target = total * b / grid;
			while (k < ntask && acc + 0.5 * cost[k] < target) acc += cost[k++];
			p->pcta[b] = (uint32_t)(b == grid ? ntask : k);
		}
	}
	/* the blocks each CTA touches: forward into the output block, transpose into the input block */
	touched = calloc(p->nblocks ? p->nblocks : 1, 1);
	p->pflush_ptr = malloc((size_t)(grid + 1) * sizeof(uint32_t));
	size_t fcap = 1024;
	p->pflush = malloc(fcap * 2 * sizeof(uint32_t));
	if (!touched || !p->pflush_ptr || !p->pflush) ERR("out of host memory");
	p->npflush = 0;
	for (int b = 0; b < grid; b++) {
		p->pflush_ptr[b] = (uint32_t)p->npflush;
		memset(touched, 0, p->nblocks);
		for (uint32_t k = p->pcta[b]; k < p->pcta[b + 1]; k++) {
			const jn_instr_t *x = &p->instr[p->panels[p->ptasks[4 * k]].instr];
			touched[x->bout] = 1;
			if (x->bin != x->bout) touched[x->bin] = 1;
		}
		/* blocks are laid out in index order: merge neighbours into ranges */
		for (int i = 0; i < p->nblocks; i++) {
			if (!touched[i]) continue;
			const uint32_t off = (uint32_t)p->blocks[i].offset, len = (uint32_t)(p->blocks[i].Np * p->blocks[i].Nn);
			if (!len) continue;
			if (p->npflush > p->pflush_ptr[b] && p->pflush[2 * (p->npflush - 1)] + p->pflush[2 * (p->npflush - 1) + 1] == off) {
				p->pflush[2 * (p->npflush - 1) + 1] += len;
				continue;
			}
			if ((size_t)p->npflush == fcap) {
				fcap *= 2;
				p->pflush = realloc(p->pflush, fcap * 2 * sizeof(uint32_t));
				if (!p->pflush) ERR("out of host memory");
			}
			p->pflush[2 * p->npflush] = off;
			p->pflush[2 * p->npflush + 1] = len;
			p->npflush++;
		}
	}
	p->pflush_ptr[grid] = (uint32_t)p->npflush;
	/* every device index stays inside its buffer: checked once here */
	for (int q = 0; q < p->npanels; q++) {
		const jn_panel_t *P = &p->panels[q];
		const jn_instr_t *x = &p->instr[P->instr];
		const jn_block_t *bi = &p->blocks[x->bin], *bo = &p->blocks[x->bout];
		if ((x->kind != JN_KIND_N && (int64_t)P->row_meta + P->nrows > p->n_pmeta) ||
		    (x->kind != JN_KIND_P && (int64_t)P->col_meta + P->ncols > p->n_pmeta))
			ERR("panel %d: list entries out of range", q);
		if (x->kind == JN_KIND_N && (bi->Np != bo->Np)) ERR("panel %d: spectator rows differ", q);
		if (x->kind == JN_KIND_P && (bi->Nn != bo->Nn)) ERR("panel %d: spectator columns differ", q);
	}
	free(order); free(cost); free(touched);
	return 0;
fail:
	free(order); free(cost); free(touched);
	jn_panels_free(p);
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
			for (int32_t j = 0; j < P->nrows; j++) {
				const uint32_t mp = ent[2 * (Lp->ent_out + j) + 1];
				const double *mrow = m + (int64_t)M->nd_n * (mp & 0x7fffffffu);
				const int64_t base = P->c_off + (int64_t)j * P->ncols;
				for (int32_t i = 0; i < P->ncols; i++) {
					const uint32_t mn = ent[2 * (Ln->ent_out + i) + 1];
					double v = mrow[mn & 0x7fffffffu];
					if ((mp ^ mn) & 0x80000000u) v = -v;
					if (c64) c64[base + i] = v;
					if (c32) c32[base + i] = (float)v;
				}
			}
		} else {
			const jn_list_t *L = &p->lists[x->kind == JN_KIND_N ? x->ln : x->lp];
			for (int64_t e = 0; e < L->len; e++) {
				const uint32_t mi = ent[2 * (L->ent_out + e) + 1];
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
