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
			uint32_t src = t->transpose ? ent[2 * j] >> 16 : ent[2 * j] & 0xffffu, mi = ent[2 * j + 1];
			double m = me[mi & 0x7fffffffu];
			if (fabs(m) < 1e-12) continue;
			if (mi & 0x80000000u) m = -m;
			acc = fma(m, xs[(size_t)src * t->Nn_src + n], acc);
		}
	} else if (t->kind == JN_KIND_N) {
		for (uint32_t j = rp[t->n_ptr + n]; j < rp[t->n_ptr + n + 1]; j++) {
			uint32_t src = t->transpose ? ent[2 * j] >> 16 : ent[2 * j] & 0xffffu, mi = ent[2 * j + 1];
			double m = me[mi & 0x7fffffffu];
			if (fabs(m) < 1e-12) continue;
			if (mi & 0x80000000u) m = -m;
			acc = fma(m, xs[(size_t)p * t->Nn_src + src], acc);
		}
	} else {
		uint32_t j0 = rp[t->n_ptr + n], j1 = rp[t->n_ptr + n + 1];
		if (j0 == j1) return 0.0;
		for (uint32_t i = rp[t->p_ptr + p]; i < rp[t->p_ptr + p + 1]; i++) {
			uint32_t ps = t->transpose ? ent[2 * i] >> 16 : ent[2 * i] & 0xffffu, mip = ent[2 * i + 1];
			const double *mrow = me + (size_t)t->nd * (mip & 0x7fffffffu);
			const double *xrow = xs + (size_t)ps * t->Nn_src;
			for (uint32_t j = j0; j < j1; j++) {
				uint32_t ns = t->transpose ? ent[2 * j] >> 16 : ent[2 * j] & 0xffffu, min = ent[2 * j + 1];
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

/* ------------------------------------------------------------------ */
/* block-tile plan: CPU model of jn_prep_kernel, jn_tile_kernel and
 * jn_finalize_kernel, lane for lane, with every index checked.  The
 * fixed-point sums are exact, so the model reproduces the GPU result bit for
 * bit when it forms the same runs and rounds the same way. */
#include <stdio.h>

static int emu_fail;
#define CHECK(c) do { if (!(c)) { if (!emu_fail) fprintf(stderr, "plan emulator: %s failed at %s:%d\n", #c, __FILE__, __LINE__); emu_fail = 1; return; } } while (0)

static int fixed_exponent(float xmax, double bound)
{
	double yb = bound * (double)xmax;
	if (!(yb > 0.0)) return 0;
	uint64_t bits;
	memcpy(&bits, &yb, 8);
	int e = (int)((bits >> 52) & 0x7ff) - 1022;
	int S = 62 - e;
	return S < -60 ? -60 : (S > 100 ? 100 : S);
}

static int pow2_at_least(int v) { int b = 1; while (b < v) b <<= 1; return b; }

static int tiny64(double m) { uint64_t b; memcpy(&b, &m, 8); return (b & 0x7fffffffffffffffull) < 0x3D719799812DEA11ull; }

static void tile_model(const jn_plan_t *P, const jn_btile_t *tl, const double *x64, const float *x32, const double *me64,
		       const float *me32, int f32, int S, int64_t *gacc)
{
	const int Nn = tl->Nn, E = tl->nrows * Nn;
	int64_t *sacc = calloc(E ? E : 1, sizeof(int64_t));
	const uint32_t *ent = P->ent;
	double scale = ldexp(1.0, S);
	float scalef = (float)scale;
	for (int64_t pc = tl->pc0; pc < tl->pc1; pc++) {
		const jn_piece_t *pcs = &P->pieces[pc];
		CHECK(pcs->term >= 0 && pcs->term < P->nterms);
		const jn_term_t *t = &P->terms[pcs->term];
		const int tr = t->transpose != 0, Ns = t->Nn_src;
		for (int lane = 0; lane < 32; lane++) {
			if (t->kind != JN_KIND_N) {
				const int ncol = t->kind == JN_KIND_NP ? (int)(t->n_e1 - t->n_e0) : t->Nn_dst;
				const int b = ncol >= 32 ? 32 : pow2_at_least(ncol), a = 32 / b;
				const int gi = lane / b, gj = lane % b;
				const uint32_t na = pcs->a1 - pcs->a0, per = (na + a - 1) / a;
				const uint32_t e0 = pcs->a0 + gi * per, e1 = (pcs->a1 < e0 + per) ? pcs->a1 : e0 + per;
				for (int cj = gj; cj < ncol; cj += b) {
					int scol, dcol;
					uint32_t kn = 0, sn = 0;
					if (t->kind == JN_KIND_NP) {
						CHECK(t->n_e0 + cj < (uint64_t)P->n_ent);
						uint32_t qx = ent[2 * (t->n_e0 + cj)], qy = ent[2 * (t->n_e0 + cj) + 1];
						int nin = qx & 0xffff, nout = qx >> 16;
						scol = tr ? nout : nin; dcol = tr ? nin : nout;
						kn = qy & 0x7fffffffu; sn = qy;
					} else { scol = dcol = cj; }
					CHECK(dcol >= 0 && dcol < Nn);
					double run = 0; float runf = 0; int cur = -1;
					for (uint32_t ep = e0; ep < e1; ep++) {
						CHECK(ep < (uint64_t)P->n_ent);
						uint32_t qx = ent[2 * ep], qy = ent[2 * ep + 1];
						int pin = qx & 0xffff, pout = qx >> 16;
						int srow = tr ? pout : pin, drow = tr ? pin : pout;
						if (drow != cur) {
							if (cur >= 0) sacc[(cur - tl->row0) * Nn + dcol] += f32 ? llrintf(runf * scalef) : llrint(run * scale);
							run = 0; runf = 0; cur = drow;
							CHECK(cur >= tl->row0 && cur < tl->row0 + tl->nrows);
						}
						uint32_t kp = qy & 0x7fffffffu;
						size_t mi = t->kind == JN_KIND_NP ? (size_t)kn + (size_t)t->nd * kp : (size_t)kp;
						CHECK(t->me_off + (int64_t)mi < P->n_me);
						size_t xi = (size_t)t->src_off + (size_t)srow * Ns + scol;
						CHECK((int64_t)xi < P->dim);
						int neg = ((qy ^ sn) & 0x80000000u) != 0;
						if (f32) {
							float m = me32[t->me_off + mi];
							if (neg) m = -m;
							runf = fmaf(m, x32[xi], runf);
						} else {
							double m = me64[t->me_off + mi];
							if (t->kind == JN_KIND_P && tiny64(m)) continue;
							if (neg) m = -m;
							run = fma(m, x64[xi], run);
						}
					}
					if (cur >= 0) sacc[(cur - tl->row0) * Nn + dcol] += f32 ? llrintf(runf * scalef) : llrint(run * scale);
				}
			} else {
				const int ncol = (int)(t->n_e1 - t->n_e0);
				const int b = ncol >= 32 ? 32 : pow2_at_least(ncol), a = 32 / b;
				const int gi = lane / b, gj = lane % b;
				for (int cj = gj; cj < ncol; cj += b) {
					uint32_t qx = ent[2 * (t->n_e0 + cj)], qy = ent[2 * (t->n_e0 + cj) + 1];
					int nin = qx & 0xffff, nout = qx >> 16;
					int scol = tr ? nout : nin, dcol = tr ? nin : nout;
					CHECK(dcol < Nn);
					int neg = (qy & 0x80000000u) != 0;
					for (uint32_t r = pcs->a0 + gi; r < pcs->a1; r += a) {
						CHECK((int)r >= tl->row0 && (int)r < tl->row0 + tl->nrows);
						size_t xi = (size_t)t->src_off + (size_t)r * Ns + scol;
						CHECK((int64_t)xi < P->dim);
						if (f32) {
							float m = me32[t->me_off + (qy & 0x7fffffffu)];
							if (neg) m = -m;
							sacc[(r - tl->row0) * Nn + dcol] += llrintf(m * x32[xi] * scalef);
						} else {
							double m = me64[t->me_off + (qy & 0x7fffffffu)];
							if (tiny64(m)) continue;
							if (neg) m = -m;
							sacc[(r - tl->row0) * Nn + dcol] += llrint(m * x64[xi] * scale);
						}
					}
				}
			}
		}
	}
	for (int i = 0; i < E; i++) gacc[tl->dst_off + (int64_t)tl->row0 * Nn + i] += sacc[i];
	free(sacc);
}

/* returns 0 on success, 1 when an index check failed */
int emu_matvec3(void *h, const double *x, double *y, int accumulate, int f32)
{
	const jn_plan_t *P = h;
	emu_fail = 0;
	float xmax = 0;
	float *x32 = malloc((P->dim ? P->dim : 1) * sizeof(float));
	float *me32 = NULL;
	for (int64_t i = 0; i < P->dim; i++) {
		x32[i] = (float)x[i];
		float v = (float)fabs(x[i]) * 1.0000002f;
		if (v > xmax) xmax = v;
	}
	if (f32) {
		me32 = malloc((P->n_me ? P->n_me : 1) * sizeof(float));
		for (int b = 0; b < P->nmes; b++)
			for (int64_t e = 0; e < P->mes[b].len; e++) {
				double v = P->me[P->mes[b].offset + e];
				me32[P->mes[b].offset + e] = (P->mes[b].single && fabs(v) < 1e-12) ? 0.0f : (float)v;
			}
	}
	int S = fixed_exponent(xmax, P->abs_bound);
	int64_t *gacc = calloc(P->dim ? P->dim : 1, sizeof(int64_t));
	for (int t = 0; t < P->nbtiles && !emu_fail; t++) tile_model(P, &P->btiles[t], x, x32, P->me, me32, f32, S, gacc);
	double unit = ldexp(1.0, -S);
	for (int64_t i = 0; i < P->dim; i++) y[i] = accumulate ? y[i] + (double)gacc[i] * unit : (double)gacc[i] * unit;
	free(gacc); free(x32); free(me32);
	return emu_fail;
}
