/*
 * plan_emulator.c — test helper: executes the device plan built by
 * jn_problem.c on the CPU, statement for statement like jn_units_kernel and
 * jn_reduce_kernel in jn_matvec.cu, so that the plan (CSR views, terms,
 * tiles, chunks) can be checked against the oracle without a GPU.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../../jupiterncsm_gb300/csrc/jn_problem.h"

static double term_element(const jn_plan_t *P, const jn_term_t *t, const double *x, int p, int n)
{
	const double *xs = x + t->src_off, *me = P->me + t->me_off;
	const uint32_t *rp = P->rowptr, *ent = P->ent;
	double acc = 0.0;
	if (t->kind == JN_KIND_P) {
		for (uint32_t j = rp[t->p_ptr + p]; j < rp[t->p_ptr + p + 1]; j++) {
			uint32_t src = ent[2 * j], mi = ent[2 * j + 1];
			double m = me[mi & 0x7fffffffu];
			if (fabs(m) < 1e-12) continue;
			if (mi & 0x80000000u) m = -m;
			acc = fma(m, xs[(size_t)src * t->Nn_src + n], acc);
		}
	} else if (t->kind == JN_KIND_N) {
		for (uint32_t j = rp[t->n_ptr + n]; j < rp[t->n_ptr + n + 1]; j++) {
			uint32_t src = ent[2 * j], mi = ent[2 * j + 1];
			double m = me[mi & 0x7fffffffu];
			if (fabs(m) < 1e-12) continue;
			if (mi & 0x80000000u) m = -m;
			acc = fma(m, xs[(size_t)p * t->Nn_src + src], acc);
		}
	} else {
		uint32_t j0 = rp[t->n_ptr + n], j1 = rp[t->n_ptr + n + 1];
		if (j0 == j1) return 0.0;
		for (uint32_t i = rp[t->p_ptr + p]; i < rp[t->p_ptr + p + 1]; i++) {
			uint32_t ps = ent[2 * i], mip = ent[2 * i + 1];
			const double *mrow = me + (size_t)t->nd * (mip & 0x7fffffffu);
			const double *xrow = xs + (size_t)ps * t->Nn_src;
			for (uint32_t j = j0; j < j1; j++) {
				uint32_t ns = ent[2 * j], min = ent[2 * j + 1];
				double m = mrow[min & 0x7fffffffu];
				if ((mip ^ min) & 0x80000000u) m = -m;
				acc = fma(m, xrow[ns], acc);
			}
		}
	}
	return acc;
}

void *emu_open(const char *comb, const char *order, const char *lists, const char *mes, int Z, int N, int units,
	       char *err, int errlen)
{
	jn_plan_t *p = calloc(1, sizeof *p);
	if (jn_plan_build(p, comb, order, lists, mes, Z, N, units, err, (size_t)errlen)) { free(p); return NULL; }
	return p;
}

long emu_dimension(void *h) { return (long)((jn_plan_t *)h)->dim; }
int emu_units(void *h) { return ((jn_plan_t *)h)->nunits; }
int emu_tiles(void *h) { return ((jn_plan_t *)h)->ntiles; }

/* y (+)= H x following the kernel's warp mapping (one lane per piece
 * element, terms of a unit in order) and the chunk-ordered reduction */
void emu_matvec(void *h, const double *x, double *y, int accumulate)
{
	const jn_plan_t *P = h;
	double *partial = calloc(P->n_partial ? P->n_partial : 1, sizeof(double));
	for (int b = 0; b < P->nunits; b++) {
		const jn_unit_t *u = &P->units[b];
		const jn_tile_t *tile = &P->tiles[u->tile];
		const int E = tile->nrows * tile->ncols;
		for (int lane = 0; lane < E; lane++) {
			int p = tile->row0 + lane / tile->ncols, n = tile->col0 + lane % tile->ncols;
			double acc = 0.0;
			for (int64_t q = u->t0; q < u->t1; q++) acc += term_element(P, &P->terms[P->unit_terms[q]], x, p, n);
			partial[tile->partial + (int64_t)u->chunk * E + lane] = acc;
		}
	}
	for (int ti = 0; ti < P->ntiles; ti++) {
		const jn_tile_t *t = &P->tiles[ti];
		const int E = t->nrows * t->ncols;
		for (int e = 0; e < E; e++) {
			double s = 0.0;
			for (int c = 0; c < t->nchunks; c++) s += partial[t->partial + (int64_t)c * E + e];
			int64_t at = t->dst_off + (int64_t)(t->row0 + e / t->ncols) * t->Nn + t->col0 + e % t->ncols;
			y[at] = accumulate ? y[at] + s : s;
		}
	}
	free(partial);
}

void emu_close(void *h) { jn_plan_free(h); free(h); }
