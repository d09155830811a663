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
			uint32_t src = ent[2 * j] & 0xffffu, mi = ent[2 * j + 1];
			double m = me[mi & 0x7fffffffu];
			if (fabs(m) < 1e-12) continue;
			if (mi & 0x80000000u) m = -m;
			acc = fma(m, xs[(size_t)src * t->Nn_src + n], acc);
		}
	} else if (t->kind == JN_KIND_N) {
		for (uint32_t j = rp[t->n_ptr + n]; j < rp[t->n_ptr + n + 1]; j++) {
			uint32_t src = ent[2 * j] & 0xffffu, mi = ent[2 * j + 1];
			double m = me[mi & 0x7fffffffu];
			if (fabs(m) < 1e-12) continue;
			if (mi & 0x80000000u) m = -m;
			acc = fma(m, xs[(size_t)p * t->Nn_src + src], acc);
		}
	} else {
		uint32_t j0 = rp[t->n_ptr + n], j1 = rp[t->n_ptr + n + 1];
		if (j0 == j1) return 0.0;
		for (uint32_t i = rp[t->p_ptr + p]; i < rp[t->p_ptr + p + 1]; i++) {
			uint32_t ps = ent[2 * i] & 0xffffu, mip = ent[2 * i + 1];
			const double *mrow = me + (size_t)t->nd * (mip & 0x7fffffffu);
			const double *xrow = xs + (size_t)ps * t->Nn_src;
			for (uint32_t j = j0; j < j1; j++) {
				uint32_t ns = ent[2 * j] & 0xffffu, min = ent[2 * j + 1];
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
	if (jn_plan_build_units(p, units, err, (size_t)errlen)) { jn_plan_free(p); free(p); return NULL; }
	return p;
}

long emu_dimension(void *h) { return (long)((jn_plan_t *)h)->dim; }
int emu_btiles_off(void *h) { return ((jn_plan_t *)h)->btiles_off; }
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


static int tiny64(double m) { uint64_t b; memcpy(&b, &m, 8); return (b & 0x7fffffffffffffffull) < 0x3D719799812DEA11ull; }

static void tile_model(const jn_plan_t *P, const jn_btile_t *tl, const double *x64, const float *x32, const double *me64,
		       const float *me32, int f32, int S, int64_t *gacc)
{
	const int Nn = tl->Nn, stride = tl->stride, E = tl->nrows * Nn;
	CHECK(stride >= Nn && (stride & 1));
	CHECK(tl->nrows * stride <= P->max_tile_elems);
	int64_t *sacc = calloc(E ? E : 1, sizeof(int64_t));
	const uint32_t *ent = P->ent, *W = P->walks;
	double scale = ldexp(1.0, S);
	float scalef = (float)scale;
	for (int64_t it = tl->pc0; it < tl->pc1; it++) {
	CHECK(it < P->nitems);
	const uint32_t first = P->items[2 * it], w = P->items[2 * it + 1] & 0xff, nsub = P->items[2 * it + 1] >> 8;
	CHECK((w == 8 || w == 16 || w == 32) && nsub >= 1 && nsub * w <= 32 && first + nsub <= (uint64_t)P->npieces);
	for (uint32_t sub = 0; sub < nsub; sub++) {
		const jn_piece_t *task = &P->pieces[first + sub];
		const int term = (int)JN_TASK_TERM(task->head), kind = (int)JN_TASK_KIND(task->head);
		const int count = (int)JN_TASK_COUNT(task->head);
		CHECK(term < P->nterms && count >= 1 && (uint32_t)count <= w && kind <= JN_TASK_N_B);
		CHECK(kind == (int)JN_TASK_KIND(P->pieces[first].head));
		const jn_term_t *t = &P->terms[term];
		const jn_tterm_t *tt = &P->tterms[term];
		CHECK(tt->me_off == t->me_off && tt->src_off == t->src_off && tt->nd == t->nd && tt->Nn_src == t->Nn_src &&
		      tt->transpose == t->transpose);
		const int Ns = t->Nn_src, nd = t->nd;
		for (int lane = 0; lane < count; lane++) {
			const uint32_t lb = task->lane_base + lane;
			for (uint32_t q = 0; q < task->loop_len; q++) {
				const uint32_t lq = task->loop_base + q;
				double run = 0;
				float runf = 0;
				int drow, dcol;
				uint32_t p0 = 0, p1 = 0, n0 = 0, n1 = 0;
				int ccol = -1, rrow = -1;
#define WALK(i, a, b, idx) do { CHECK((int64_t)(i) < P->nwalks); a = W[2 * (i)]; b = a + (W[2 * (i) + 1] & 0xffff); idx = (int)(W[2 * (i) + 1] >> 16); } while (0)
				if (kind == JN_TASK_NP_A) { CHECK(lb >= t->nw0 && lb < t->nw1 && lq >= t->pw0 && lq < t->pw1); WALK(lb, n0, n1, dcol); WALK(lq, p0, p1, drow); }
				else if (kind == JN_TASK_NP_B) { CHECK(lb >= t->pw0 && lb < t->pw1 && lq >= t->nw0 && lq < t->nw1); WALK(lb, p0, p1, drow); WALK(lq, n0, n1, dcol); }
				else if (kind == JN_TASK_P_A) { CHECK(lq >= t->pw0 && lq < t->pw1); WALK(lq, p0, p1, drow); ccol = (int)lb; dcol = ccol; }
				else if (kind == JN_TASK_P_B) { CHECK(lb >= t->pw0 && lb < t->pw1); WALK(lb, p0, p1, drow); ccol = (int)lq; dcol = ccol; }
				else if (kind == JN_TASK_N_A) { CHECK(lb >= t->nw0 && lb < t->nw1); WALK(lb, n0, n1, dcol); rrow = (int)lq; drow = rrow; }
				else { CHECK(lq >= t->nw0 && lq < t->nw1); WALK(lq, n0, n1, dcol); rrow = (int)lb; drow = rrow; }
#undef WALK
				CHECK(drow >= tl->row0 && drow < tl->row0 + tl->nrows && dcol >= 0 && dcol < Nn);
#define VISIT(MI, XI, NEG, SKIP_TINY)                                                       \
				do {                                                                \
					CHECK(t->me_off + (int64_t)(MI) < P->n_me);                  \
					CHECK((int64_t)(XI) >= 0 && (int64_t)(XI) < P->dim);         \
					if (f32) { float m_ = me32[t->me_off + (MI)]; if (NEG) m_ = -m_; runf = fmaf(m_, x32[XI], runf); } \
					else { double m_ = me64[t->me_off + (MI)]; if ((SKIP_TINY) && tiny64(m_)) break; if (NEG) m_ = -m_; run = fma(m_, x64[XI], run); } \
				} while (0)
				if (kind == JN_TASK_NP_A) {
					for (uint32_t j = n0; j < n1; j++) {
						uint32_t qx = ent[2 * j], qy = ent[2 * j + 1];
						int scol = (int)(qx & 0xffff);
						int ndst = (int)(qx >> 16);
						CHECK(ndst == dcol);
						for (uint32_t i = p0; i < p1; i++) {
							uint32_t px = ent[2 * i], py = ent[2 * i + 1];
							int srow = (int)(px & 0xffff);
							int pdst = (int)(px >> 16);
							CHECK(pdst == drow);
							size_t mi = (qy & 0x7fffffffu) + (size_t)nd * (py & 0x7fffffffu);
							VISIT(mi, t->src_off + srow * Ns + scol, ((py ^ qy) & 0x80000000u) != 0, 0);
						}
					}
				} else if (kind == JN_TASK_NP_B) {
					for (uint32_t i = p0; i < p1; i++) {
						uint32_t px = ent[2 * i], py = ent[2 * i + 1];
						int srow = (int)(px & 0xffff);
						for (uint32_t j = n0; j < n1; j++) {
							uint32_t qx = ent[2 * j], qy = ent[2 * j + 1];
							int scol = (int)(qx & 0xffff);
							size_t mi = (qy & 0x7fffffffu) + (size_t)nd * (py & 0x7fffffffu);
							VISIT(mi, t->src_off + srow * Ns + scol, ((py ^ qy) & 0x80000000u) != 0, 0);
						}
					}
				} else if (kind == JN_TASK_P_A || kind == JN_TASK_P_B) {
					CHECK(ccol >= 0 && ccol < Nn);
					for (uint32_t i = p0; i < p1; i++) {
						uint32_t px = ent[2 * i], py = ent[2 * i + 1];
						int srow = (int)(px & 0xffff);
						VISIT(py & 0x7fffffffu, t->src_off + srow * Ns + ccol, (py & 0x80000000u) != 0, 1);
					}
				} else {
					for (uint32_t j = n0; j < n1; j++) {
						uint32_t qx = ent[2 * j], qy = ent[2 * j + 1];
						int scol = (int)(qx & 0xffff);
						VISIT(qy & 0x7fffffffu, t->src_off + rrow * Ns + scol, (qy & 0x80000000u) != 0, 1);
					}
				}
#undef VISIT
				sacc[(drow - tl->row0) * Nn + dcol] += f32 ? llrintf(runf * scalef) : llrint(run * scale);
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

/* task statistics of the block-tile plan: tasks, tiles, lane slots, walk steps */
void emu_task_stats(void *h, double *out)
{
	const jn_plan_t *P = h;
	double lanes = 0, steps = 0, visits = 0, kinds[4] = { 0, 0, 0, 0 };
	for (int64_t k = 0; k < P->npieces; k++) {
		const jn_piece_t *t = &P->pieces[k];
		double c = JN_TASK_COUNT(t->head);
		lanes += c;
		steps += t->loop_len;
		visits += c * t->loop_len;
		kinds[JN_TASK_KIND(t->head) >> 1] += 1;
	}
	out[0] = (double)P->npieces; out[1] = P->nbtiles; out[2] = lanes; out[3] = steps; out[4] = visits;
	out[5] = kinds[0]; out[6] = kinds[1]; out[7] = kinds[2]; out[8] = kinds[3];
}

/* ------------------------------------------------------------------ */
/* panel engine: CPU model of jn_panel_kernel, lane for lane, with every
 * index checked.  FP64: every contribution (c x) 2^S is rounded once to an
 * integer and added.  32-bit: coefficients and x are 32-bit fixed-point
 * integers, and every exact 64-bit product is rounded once by the shift k.  The fixed-point sums are exact, so the model reproduces the GPU
 * bit for bit. */
static void panel_lane_model(const jn_plan_t *P, const jn_panel_t *pn, uint32_t j0, uint32_t j1, int R, int r, int i,
			     const double *x64, const int32_t *xi, const double *c64, const int32_t *ci, int f32, int S,
			     int k, int64_t *acc)
{
	const int kind = pn->kind & 7, diag = (pn->kind & JN_PANEL_DIAG) != 0;
	const int rows_n = kind == JN_KIND_NP && (pn->kind & JN_PANEL_ROWS_N);
	const int MRo = rows_n ? 1 : pn->Nn_out, MCo = rows_n ? pn->Nn_out : 1;
	const int MRi = rows_n ? 1 : pn->Nn_in, MCi = rows_n ? pn->Nn_in : 1;
	const double scale = ldexp(1.0, S);
	const int64_t bias = k > 0 ? (int64_t)1 << (k - 1) : 0;
	/* a CTA's shared-memory accumulator holds each block it touches with rows padded to Nn | 1 */
	CHECK(pn->out_blk >= 0 && pn->in_blk >= 0 && pn->out_blk < P->nblocks && pn->in_blk < P->nblocks);
	int sc, dc;
	if (kind == JN_KIND_P) {
		sc = dc = i;
	} else {
		CHECK((int64_t)pn->col_meta + i < P->n_pmeta);
		const uint32_t m = P->pmeta[pn->col_meta + i];
		sc = (int)(m & 0xffffu);
		dc = (int)(m >> 16);
	}
	for (uint32_t j = j0 + r; j < j1; j += R) {
		int sr, dr;
		int64_t cidx;
		if (kind == JN_KIND_N) {
			sr = dr = (int)j;
			cidx = pn->c_off + i;
		} else {
			CHECK((int64_t)pn->row_meta + j < P->n_pmeta);
			const uint32_t m = P->pmeta[pn->row_meta + j];
			sr = (int)(m & 0xffffu);
			dr = (int)(m >> 16);
			cidx = kind == JN_KIND_NP ? pn->c_off + (int64_t)j * pn->ncols + i : pn->c_off + j;
		}
		CHECK(cidx >= 0 && cidx < P->n_coef);
		/* the element stays inside its blocks */
		CHECK(rows_n ? (sr < pn->Nn_in && dr < pn->Nn_out) : (sc < pn->Nn_in && dc < pn->Nn_out));
		const int64_t at_i = pn->in_off + (int64_t)sr * MRi + (int64_t)sc * MCi;
		const int64_t at_o = pn->out_off + (int64_t)dr * MRo + (int64_t)dc * MCo;
		CHECK(at_i >= 0 && at_i < P->dim && at_o >= 0 && at_o < P->dim);
		/* the padded shared-memory positions stay inside their blocks */
		const int64_t so = (int64_t)(rows_n ? dc : dr) * (pn->Nn_out | 1) + (rows_n ? dr : dc);
		const int64_t si = (int64_t)(rows_n ? sc : sr) * (pn->Nn_in | 1) + (rows_n ? sr : sc);
		CHECK(so >= 0 && so < (int64_t)pn->Np_out * (pn->Nn_out | 1) && si >= 0 && si < (int64_t)pn->Np_in * (pn->Nn_in | 1));
		if (f32) {
			/* 32-bit fixed point: exact 64-bit product, rounded by the shift k */
			const int64_t cv = ci[cidx];
			acc[at_o] += (cv * xi[at_i] + bias) >> k;
			if (!diag) acc[at_i] += (cv * xi[at_o] + bias) >> k;
		} else {
			const double cv = c64[cidx];
			double t = cv * x64[at_i];
			acc[at_o] += (int64_t)llrint(t * scale);
			if (!diag) {
				t = cv * x64[at_o];
				acc[at_i] += (int64_t)llrint(t * scale);
			}
		}
	}
}

int emu_matvec4(void *h, const double *x, double *y, int accumulate, int f32)
{
	jn_plan_t *P = h;
	char err[512];
	emu_fail = 0;
	if (!P->panels && jn_panels_build(P, 152 * 2, JN_PANEL_ITER, err, sizeof err)) {
		fprintf(stderr, "plan emulator: %s\n", err);
		return 1;
	}
	float xmax = 0;
	for (int64_t i = 0; i < P->dim; i++) {
		float v = (float)fabs(x[i]) * 1.0000002f;
		if (v > xmax) xmax = v;
	}
	const int S = fixed_exponent(xmax, P->abs_bound);
	/* 32-bit path: x as 32-bit fixed point, |x| 2^Sx < 2^30 for the FP32 bound xmax */
	uint32_t xb;
	memcpy(&xb, &xmax, 4);
	int Sx = 0;
	if (xb & 0x7fffffffu) {
		Sx = 30 - ((int)((xb >> 23) & 0xff) - 126);
		Sx = Sx < -900 ? -900 : (Sx > 900 ? 900 : Sx);
	}
	int32_t *xi = malloc((P->dim ? P->dim : 1) * sizeof(int32_t));
	for (int64_t i = 0; i < P->dim; i++) xi[i] = (int32_t)llrint(x[i] * ldexp(1.0, Sx));
	double *c64 = f32 ? NULL : malloc((P->n_coef ? P->n_coef : 1) * sizeof(double));
	int32_t *ci = f32 ? malloc((P->n_coef ? P->n_coef : 1) * sizeof(int32_t)) : NULL;
	int Sc = 0, k = 0;
	if (f32) jn_panels_coefficients_int(P, P->me, ci, &Sc, &k);
	else jn_panels_coefficients(P, P->me, c64, NULL);
	int64_t *acc = calloc(P->dim ? P->dim : 1, sizeof(int64_t));
	/* every task once, every CTA's task range covering all of them */
	if (P->pcta[0] != 0 || P->pcta[P->pgrid] != (uint32_t)P->nptasks) { emu_fail = 1; fprintf(stderr, "plan emulator: CTA ranges\n"); }
	/* each CTA's accumulator: its blocks one after another within pcta_words, and
	   every block a task of the CTA writes among them */
	{
		int64_t *at = malloc((P->nblocks ? P->nblocks : 1) * sizeof(int64_t));
		for (int b = 0; b < P->pgrid && !emu_fail; b++) {
			for (int q = 0; q < P->nblocks; q++) at[q] = -1;
			int64_t next = 0;
			for (uint32_t f = P->pflush_ptr[b]; f < P->pflush_ptr[b + 1] && !emu_fail; f++) {
				const uint32_t blk = P->pflush[2 * f], off = P->pflush[2 * f + 1];
				if (blk >= (uint32_t)P->nblocks || off != next || at[blk] >= 0) { emu_fail = 1; break; }
				at[blk] = off;
				next += P->blocks[blk].Np * (P->blocks[blk].Nn | 1);
			}
			if (next > P->pcta_words) emu_fail = 1;
			for (uint32_t t = P->pcta[b]; t < P->pcta[b + 1] && !emu_fail; t++) {
				const jn_panel_t *pn = &P->panels[P->ptasks[4 * t]];
				if (at[pn->out_blk] < 0 || (!(pn->kind & JN_PANEL_DIAG) && at[pn->in_blk] < 0)) emu_fail = 1;
			}
			if (emu_fail) fprintf(stderr, "plan emulator: accumulator layout of CTA %d\n", b);
		}
		free(at);
	}
	for (int64_t t = 0; t < P->nptasks && !emu_fail; t++) {
		const uint32_t *T = P->ptasks + 4 * t;
		if (T[0] >= (uint32_t)P->npanels) { emu_fail = 1; break; }
		const jn_panel_t *pn = &P->panels[T[0]];
		const int cw = (int)(T[3] >> 24);
		if (cw < 1 || cw > 32 || T[1] >= T[2] || T[2] > (uint32_t)pn->nrows) { emu_fail = 1; break; }
		const int R = 32 / cw;
		for (int lane = 0; lane < 32 && !emu_fail; lane++) {
			const int r = lane / cw, i = (int)(T[3] & 0xffffffu) + (lane - r * cw);
			if (r >= R || i >= pn->ncols) continue;
			panel_lane_model(P, pn, T[1], T[2], R, r, i, x, xi, c64, ci, f32, S, k, acc);
		}
	}
	const double unit = f32 ? ldexp(1.0, k - Sc - Sx) : ldexp(1.0, -S);
	for (int64_t i = 0; i < P->dim; i++) y[i] = accumulate ? y[i] + (double)acc[i] * unit : (double)acc[i] * unit;
	free(acc); free(xi); free(c64); free(ci);
	return emu_fail;
}

/* Shared-memory wavefronts of the panel kernel's atomics, warp instruction by
 * warp instruction, under the plan's schedule: lanes whose words share a
 * bank (32 banks of 4 bytes) serialise, the same word included.  out:
 * {forward instructions, forward wavefronts, transpose instructions,
 * transpose wavefronts}.  by_out != 0 counts them with every list in by-out
 * order instead of the plan's panel order.  Returns 1 if pperm is not a
 * permutation of some list or pmeta disagrees with it. */
int emu_panel_wavefronts(void *h, int by_out, double *out)
{
	jn_plan_t *P = h;
	char err[512];
	if (!P->panels && jn_panels_build(P, 152 * 3, JN_PANEL_ITER, err, sizeof err)) return 1;
	uint32_t *meta = malloc((P->n_pmeta ? P->n_pmeta : 1) * sizeof(uint32_t));
	unsigned char *seen = calloc(P->n_pmeta ? P->n_pmeta : 1, 1);
	int bad = 0;
	for (int l = 0; l < P->nlists; l++) {
		const jn_list_t *L = &P->lists[l];
		for (int64_t k = 0; k < L->len; k++) {
			const uint32_t e = P->pperm[L->pmeta + k];
			if (e >= (uint32_t)L->len || seen[L->pmeta + e]) { bad = 1; break; }
			seen[L->pmeta + e] = 1;
			if (P->pmeta[L->pmeta + k] != P->ent[2 * (L->ent_out + e)]) bad = 1;
			meta[L->pmeta + k] = by_out ? P->ent[2 * (L->ent_out + k)] : P->pmeta[L->pmeta + k];
		}
	}
	int64_t *at = malloc((P->nblocks ? P->nblocks : 1) * sizeof(int64_t));
	for (int q = 0; q < 4; q++) out[q] = 0;
	for (int b = 0; b < P->pgrid && !bad; b++) {
		for (uint32_t f = P->pflush_ptr[b]; f < P->pflush_ptr[b + 1]; f++) at[P->pflush[2 * f]] = P->pflush[2 * f + 1];
		for (uint32_t t = P->pcta[b]; t < P->pcta[b + 1]; t++) {
			const uint32_t *T = P->ptasks + 4 * t;
			const jn_panel_t *pn = &P->panels[T[0]];
			const int cw = (int)(T[3] >> 24), R = 32 / cw, i0 = (int)(T[3] & 0xffffffu);
			const int kind = pn->kind & 7, diag = (pn->kind & JN_PANEL_DIAG) != 0;
			const int rows_n = kind == JN_KIND_NP && (pn->kind & JN_PANEL_ROWS_N);
			const int64_t so = at[pn->out_blk], si = at[pn->in_blk];
			const int Po = pn->Nn_out | 1, Pi = pn->Nn_in | 1;
			for (uint32_t g = 0; T[1] + g * R < T[2]; g++) {
				int cnt[2][32] = {{0}};
				for (int lane = 0; lane < 32; lane++) {
					const int r = lane / cw, i = i0 + lane - r * cw;
					const uint32_t j = T[1] + g * R + r;
					if (r >= R || i >= pn->ncols || j >= T[2]) continue;
					int sc, dc, sr, dr;
					if (kind == JN_KIND_P) sc = dc = i;
					else { const uint32_t m = meta[pn->col_meta + i]; sc = m & 0xffff; dc = m >> 16; }
					if (kind == JN_KIND_N) sr = dr = (int)j;
					else { const uint32_t m = meta[pn->row_meta + j]; sr = m & 0xffff; dr = m >> 16; }
					cnt[0][(rows_n ? so + (int64_t)dc * Po + dr : so + (int64_t)dr * Po + dc) & 31]++;
					cnt[1][(rows_n ? si + (int64_t)sc * Pi + sr : si + (int64_t)sr * Pi + sc) & 31]++;
				}
				for (int k = 0; k < 2 - diag; k++) {
					int mx = 0;
					for (int q = 0; q < 32; q++) mx = cnt[k][q] > mx ? cnt[k][q] : mx;
					out[2 * k] += 1;
					out[2 * k + 1] += mx;
				}
			}
		}
	}
	free(meta); free(seen); free(at);
	return bad;
}

/* ------------------------------------------------------------------ */
/* walk engine: CPU model of jn_walk_kernel (jn_walk.cu), task by task,
 * lane by lane, with every index checked.  mode 32: FP32 coefficients and
 * x, fused multiply-adds in entry order, the row sum rounded once to the
 * fixed-point unit; mode 64: the same in FP64; mode 1: the exact integer
 * path (52-bit fixed-point coefficients, each block at its own exponent,
 * and x, split into 28 + 24 bits,
 * three 32 x 32 -> 64-bit products per multiply-add, the row sum rounded
 * once to the nearest output unit).  Returns 1 when an index leaves its buffer. */
static int walk_x_exponent52(float xmax)
{
	uint32_t b;
	memcpy(&b, &xmax, 4);
	if (!(b & 0x7fffffffu)) return 0;
	return 52 - ((int)((b >> 23) & 0xff) - 126);
}

int emu_walk_build(void *h)
{
	char err[512];
	jn_plan_t *P = h;
	if (P->wtasks) return 0;
	if (jn_walk_build(P, err, sizeof err)) { fprintf(stderr, "walk plan: %s\n", err); return 1; }
	return 0;
}

/* {tasks, pieces, groups, multiply-adds with padding, row words, lane slots x rows, walk elements,
 * multiply-adds of the product} */
void emu_walk_stats(void *h, double *out)
{
	jn_plan_t *P = h;
	memset(out, 0, 8 * sizeof(double));
	if (emu_walk_build(h)) return;
	out[7] = P->visits;
	out[0] = (double)P->nwtasks; out[1] = (double)P->nwpieces; out[2] = (double)P->n_wgroups; out[3] = P->wvisits;
	out[4] = (double)P->n_wrows; out[5] = P->wlane_slots; out[6] = (double)P->n_wme;
}

/* Lane-set sharing: out[0] lane words stored, out[1] lane words of the
 * distinct sets the tasks reference (equal when no set is orphaned and none
 * overlaps another), out[2] sets referenced by pieces of more than one
 * matrix-element block (shared across instructions). */
typedef struct { uint32_t lanes; int32_t block; int lw; } lane_ref_t;

static int cmp_lane_ref(const void *a, const void *b)
{
	const lane_ref_t *x = a, *y = b;
	if (x->lanes != y->lanes) return x->lanes < y->lanes ? -1 : 1;
	return x->block < y->block ? -1 : x->block > y->block;
}

void emu_walk_lane_sharing(void *h, double *out)
{
	jn_plan_t *P = h;
	memset(out, 0, 3 * sizeof(double));
	if (emu_walk_build(h) || P->nwtasks == 0) return;
	lane_ref_t *r = malloc((size_t)P->nwtasks * sizeof *r);
	for (int64_t t = 0; t < P->nwtasks; t++) {
		const jn_wtask_t *T = &P->wtasks[t];
		r[t].lanes = T->lanes;
		r[t].block = P->wgblock[P->wpieces[T->piece].group0];
		r[t].lw = JN_WALK_LANE_WORDS((int)(T->meta >> 8));
	}
	qsort(r, (size_t)P->nwtasks, sizeof *r, cmp_lane_ref);
	double words = 0, shared = 0;
	int64_t end = 0;           /* first lane word after the sets seen so far */
	for (int64_t t = 0; t < P->nwtasks;) {
		int64_t u = t + 1;
		int multi = 0;
		while (u < P->nwtasks && r[u].lanes == r[t].lanes) {
			if (r[u].block != r[t].block) multi = 1;
			if (r[u].lw != r[t].lw) { words = -1e300; }      /* one set read with two widths */
			u++;
		}
		if (r[t].lanes < end) words = -1e300;                   /* overlapping sets */
		end = r[t].lanes + 32 * (int64_t)r[t].lw;
		words += 32.0 * r[t].lw;
		shared += multi;
		t = u;
	}
	out[0] = (double)P->n_wlanes;
	out[1] = words;
	out[2] = shared;
	free(r);
}

int emu_matvec5(void *h, const double *x, double *y, int accumulate, int mode)
{
	jn_plan_t *P = h;
	if (emu_walk_build(h)) return 1;
	const int64_t D = P->dim, nm = P->n_wme;
	float xmax = 0;
	for (int64_t i = 0; i < D; i++) {
		float v = (float)fabs(x[i]) * 1.0000002f;
		if (v > xmax) xmax = v;
	}
	float *x32 = malloc((D ? D : 1) * sizeof(float)), *a32 = malloc((nm ? nm : 1) * sizeof(float));
	int32_t *xh = malloc((D ? D : 1) * sizeof(int32_t)), *xl = malloc((D ? D : 1) * sizeof(int32_t));
	double *a64 = malloc((nm ? nm : 1) * sizeof(double));
	int32_t *ah = malloc((nm ? nm : 1) * sizeof(int32_t)), *al = malloc((nm ? nm : 1) * sizeof(int32_t));
	int64_t *gacc = calloc(D ? D : 1, sizeof(int64_t));
	const int Sx = walk_x_exponent52(xmax);
	for (int64_t i = 0; i < D; i++) {
		x32[i] = (float)x[i];
		int64_t v = llrint(ldexp(x[i], Sx));
		xh[i] = (int32_t)(v >> 24);
		xl[i] = (int32_t)(v & 0xffffff);
	}
	/* the transposed view that proton walks read: xT[i] = x[perm[i]] in every type */
	double *xT = malloc((D ? D : 1) * sizeof(double));
	float *x32T = malloc((D ? D : 1) * sizeof(float));
	int32_t *xhT = malloc((D ? D : 1) * sizeof(int32_t)), *xlT = malloc((D ? D : 1) * sizeof(int32_t));
	for (int64_t i = 0; i < D; i++) {
		const int64_t q = P->wxt ? P->wxperm[i] : i;
		xT[i] = x[q]; x32T[i] = x32[q]; xhT[i] = xh[q]; xlT[i] = xl[q];
	}
	jn_walk_elements(P, P->me, a64);
	int32_t *split = malloc((nm ? nm : 1) * 2 * sizeof(int32_t));
	uint8_t *gshift = malloc(P->n_wgroups ? P->n_wgroups : 1);
	int Sc = 0;
	jn_walk_int_elements(P, P->me, split, gshift, &Sc);
	for (int64_t e = 0; e < nm; e++) {
		a32[e] = (float)a64[e];
		ah[e] = split[2 * e];
		al[e] = split[2 * e + 1];
	}
	free(split);
	int S = fixed_exponent(xmax, P->abs_bound), sh = 0;
	if (mode == 1) {
		if (Sc + Sx - S < 49) S = Sc + Sx - 49;
		sh = Sc + Sx - S - 48;
		if (sh > 63) sh = 63;
	}
	const float scalef = (float)ldexp(1.0, S);
	const double scale = ldexp(1.0, S);
	int bad = 0;
	int64_t *slot = calloc(JN_WALK_RS * 32, sizeof(int64_t));
	for (int64_t t = 0; t < P->nwtasks && !bad; t++) {
		const jn_wtask_t *T = &P->wtasks[t];
		if (T->piece >= P->nwpieces) { bad = 1; break; }
		const jn_wpiece_t *pc = &P->wpieces[T->piece];
		const int U = (int)((T->meta >> 8) & 0xff), nw = (int)(T->meta & 0xff), LW = JN_WALK_LANE_WORDS(U);
		const int rs = (int)(pc->meta & 0xff), wp = (int)((pc->meta >> 8) & 1), ng = (int)(pc->meta >> 9);
		if ((U != 8 && U != 4 && U != 2) || (int64_t)T->lanes + 32 * LW > P->n_wlanes ||
		    (int64_t)T->walk0 + nw > P->n_wwalks || nw < 1 || nw > 32 || rs < 1 || rs > JN_WALK_RS ||
		    (int64_t)pc->rdst0 + rs > P->n_wrdst || (int64_t)pc->group0 + ng > P->n_wgroups) { bad = 1; break; }
		memset(slot, 0, JN_WALK_RS * 32 * sizeof(int64_t));
		for (int lane = 0; lane < 32 && !bad; lane++) {
			const uint32_t head = P->wlanes[T->lanes + lane], ws = head & 0xffffu, mul = head >> 16;
			if (ws >= (uint32_t)nw) { bad = 1; break; }
			uint32_t src[8], ko[8];
			for (int k = 0; k < U / 2; k++) {
				const uint32_t w = P->wlanes[T->lanes + (1 + k) * 32 + lane];
				src[2 * k] = w & 0xffffu;
				src[2 * k + 1] = w >> 16;
			}
			for (int u = 0; u < U; u++) ko[u] = P->wlanes[T->lanes + (1 + U / 2 + u) * 32 + lane];
			int64_t j = pc->row0;
			for (int g = 0; g < ng && !bad; g++) {
				const int64_t gb = P->wgroups[pc->group0 + g];
				int shg = sh + gshift[pc->group0 + g];
				if (shg > 62) shg = 62;
				int64_t ai[8];
				for (int u = 0; u < U; u++) {
					ai[u] = gb + (ko[u] & 0x3fffffffu);
					if (ai[u] >= nm) { bad = 1; break; }
				}
				for (;;) {
					if (bad || j >= P->n_wrows) { bad = 1; break; }
					const uint32_t row = P->wrows[j++];
					const uint32_t sr = row & 0xffffu, rslot = (row >> 16) & 31u;
					if (rslot >= (uint32_t)rs) { bad = 1; break; }
					int64_t v = 0;
					int64_t A = 0, B = 0;
					float accf = 0.0f;
					double accd = 0.0;
					/* proton walks read the transposed view */
					const double *X64 = wp ? xT : x;
					const float *X32 = wp ? x32T : x32;
					const int32_t *XH = wp ? xhT : xh, *XL = wp ? xlT : xl;
					for (int u = 0; u < U; u++) {
						const int64_t xi = pc->src_off + (int64_t)sr * pc->src_stride + src[u];
						if (xi < 0 || xi >= D) { bad = 1; break; }
						const int m = (int)((mul >> (2 * u)) & 3u), pad = m == 0, neg = m == 3;
						if (mode == 1) {
							int32_t ch = pad ? 0 : ah[ai[u]], cl = pad ? 0 : al[ai[u]];
							if (neg) { ch = -ch; cl = -cl; }
							A += (int64_t)ch * XH[xi];
							B += (int64_t)ch * XL[xi] + (int64_t)cl * XH[xi];
						} else if (mode == 32) {
							float c = pad ? 0.0f : a32[ai[u]];
							if (neg) c = -c;
							accf = fmaf(c, X32[xi], accf);
						} else {
							double c = pad ? 0.0 : a64[ai[u]];
							if (neg) c = -c;
							accd = fma(c, X64[xi], accd);
						}
					}
					if (mode == 1) {
						const int64_t q = A + (B >> 24);
						v = shg ? (q + ((int64_t)1 << (shg - 1))) >> shg : q + ((B >> 23) & 1);
						if (row >> 31) v = -v;
					} else if (mode == 32) {
						v = llrintf(accf * ((row >> 31) ? -scalef : scalef));
					} else {
						v = llrint(accd * ((row >> 31) ? -scale : scale));
					}
					slot[rslot * 32 + ws] = (int64_t)((uint64_t)slot[rslot * 32 + ws] + (uint64_t)v);
					if (row & JN_WALK_GROUP_END) break;
				}
			}
		}
		for (int r = 0; r < rs && !bad; r++)
			for (int w = 0; w < nw; w++) {
				const uint32_t dr = P->wrdst[pc->rdst0 + r], dw = P->wwalks[T->walk0 + w];
				const int64_t yi = pc->dst_off + (wp ? (int64_t)dw * pc->Nn_dst + dr : (int64_t)dr * pc->Nn_dst + dw);
				if (yi < 0 || yi >= D) { bad = 1; break; }
				gacc[yi] = (int64_t)((uint64_t)gacc[yi] + (uint64_t)slot[r * 32 + w]);
			}
	}
	const double unit = ldexp(1.0, -S);
	for (int64_t i = 0; i < D; i++) y[i] = accumulate ? y[i] + (double)gacc[i] * unit : (double)gacc[i] * unit;
	free(slot); free(x32); free(a32); free(xh); free(xl); free(a64); free(ah); free(al); free(gacc); free(gshift);
	free(xT); free(x32T); free(xhT); free(xlT);
	return bad;
}

/* shape of the walk plan by chunk width U = 8, 4, 2: {tasks, rows x tasks,
 * groups x tasks, padded multiply-adds} for each, then slot flushes x tasks */
void emu_walk_shape(void *h, double *out)
{
	jn_plan_t *P = h;
	memset(out, 0, 13 * sizeof(double));
	if (emu_walk_build(h)) return;
	for (int64_t t = 0; t < P->nwtasks; t++) {
		const jn_wtask_t *T = &P->wtasks[t];
		const jn_wpiece_t *pc = &P->wpieces[T->piece];
		const int U = (int)((T->meta >> 8) & 0xff), k = U == 8 ? 0 : (U == 4 ? 1 : 2);
		const int ng = (int)(pc->meta >> 9), rs = (int)(pc->meta & 0xff), nw = (int)(T->meta & 0xff);
		int64_t nrows = 0, j = pc->row0;
		for (int g = 0; g < ng; g++)
			for (;;) { nrows++; if (P->wrows[j++] & JN_WALK_GROUP_END) break; }
		out[4 * k] += 1;
		out[4 * k + 1] += (double)nrows;
		out[4 * k + 2] += ng;
		out[4 * k + 3] += (double)nrows * 32 * U;
		out[12] += (double)rs * nw;
	}
}

/* Structural checks of the walk plan, every index the walk kernel reads
 * against its array: returns the number of violations (0 for a sound plan).
 * Per task: U in {2, 4, 8}, its piece, lane record, walk table, rows,
 * destination rows and groups inside their arrays; per lane: a walk slot
 * below the task's walks and multipliers +1 (01) or -1 (11) for its entries
 * and 0 for padding, padding only after them, an element offset inside the
 * walk element array from every group base; per row: a slot row below the
 * piece's; each group ends with a group-end row; JN_WALK_ROW_SPARE zero
 * words after the last row (the kernel reads two words ahead). */
int64_t emu_walk_validate(void *h)
{
	jn_plan_t *P = h;
	if (emu_walk_build(h)) return -1;
	int64_t bad = 0;
	for (int k = 0; k < JN_WALK_ROW_SPARE; k++) bad += P->wrows[P->n_wrows + k] != 0u;
	for (int64_t t = 0; t < P->nwtasks; t++) {
		const jn_wtask_t *T = &P->wtasks[t];
		if (T->piece >= P->nwpieces) { bad++; continue; }
		const jn_wpiece_t *pc = &P->wpieces[T->piece];
		const int U = (int)((T->meta >> 8) & 0xff), nw = (int)(T->meta & 0xff), LW = JN_WALK_LANE_WORDS(U);
		const int rs = (int)(pc->meta & 0xff), ng = (int)(pc->meta >> 9);
		if ((U != 8 && U != 4 && U != 2) || nw < 1 || nw > 32 || rs < 1 || rs > JN_WALK_RS || ng < 1 ||
		    (int64_t)T->lanes + 32 * LW > P->n_wlanes || (int64_t)T->walk0 + nw > P->n_wwalks ||
		    (int64_t)pc->rdst0 + rs > P->n_wrdst || (int64_t)pc->group0 + ng > P->n_wgroups || pc->row0 < 0) {
			bad++;
			continue;
		}
		for (int lane = 0; lane < 32; lane++) {
			const uint32_t head = P->wlanes[T->lanes + lane], ws = head & 0xffffu, mul = head >> 16;
			if (ws >= (uint32_t)nw) bad++;
			int seen_pad = 0;
			for (int u = 0; u < U; u++) {
				const uint32_t m = (mul >> (2 * u)) & 3u, ko = P->wlanes[T->lanes + (1 + U / 2 + u) * 32 + lane];
				if (m == 2) bad++;                              /* not a multiplier */
				if (m == 0) seen_pad = 1;
				else if (seen_pad) bad++;                       /* an entry after padding */
				if (m != (ko >> 30)) bad++;                     /* the head and the entry word disagree */
				for (int g = 0; g < ng; g++)
					if ((int64_t)P->wgroups[pc->group0 + g] + (ko & 0x3fffffffu) >= P->n_wme) bad++;
			}
			if (mul >> (2 * U)) bad++;                              /* bits beyond the lane's entries */
		}
		int64_t j = pc->row0;
		for (int g = 0; g < ng; g++) {
			for (;;) {
				if (j >= P->n_wrows) { bad++; break; }
				const uint32_t row = P->wrows[j++];
				if ((int)((row >> 16) & 31u) >= rs) bad++;
				if (row & JN_WALK_GROUP_END) break;
			}
		}
		if (j + 1 > P->n_wrows + JN_WALK_ROW_SPARE) bad++;        /* the kernel's read-ahead stays inside */
	}
	return bad;
}

/* Plants one defect in the CPU model's walk plan (test infrastructure: the
 * validator's own test): 0 a nonzero spare row word, 1 the invalid
 * multiplier code 2 in a lane head, 2 a row slot beyond its piece's.
 * Returns 0, or -1 when the plan has nothing to corrupt. */
int emu_walk_corrupt(void *h, int kind)
{
	jn_plan_t *P = h;
	if (emu_walk_build(h) || P->nwtasks < 1) return -1;
	const jn_wtask_t *T = &P->wtasks[0];
	const jn_wpiece_t *pc = &P->wpieces[T->piece];
	if (kind == 0) P->wrows[P->n_wrows] = 1u;
	else if (kind == 1) P->wlanes[T->lanes] = (P->wlanes[T->lanes] & 0xffffu) | (2u << 16);
	else P->wrows[pc->row0] = (P->wrows[pc->row0] & ~(31u << 16)) | (31u << 16);
	return 0;
}

/* FNV-1a digest of every host plan array a product reads (engines 2, 3
 * and 5, the walk element arrays and the bounds): equal digests, equal plans */
static uint64_t fnv(uint64_t x, const void *v, size_t n)
{
	const unsigned char *c = v;
	for (size_t i = 0; i < n; i++) { x ^= c[i]; x *= 1099511628211ull; }
	return x;
}

uint64_t emu_plan_digest(void *h)
{
	jn_plan_t *P = h;
	uint64_t x = 1469598103934665603ull;
	x = fnv(x, P->rowptr, (size_t)P->n_rowptr * 4);
	x = fnv(x, P->ent, (size_t)P->n_ent * 8);
	x = fnv(x, P->me, (size_t)P->n_me * 8);
	x = fnv(x, &P->me_referenced, sizeof P->me_referenced);
	x = fnv(x, P->tiles, (size_t)P->ntiles * sizeof(jn_tile_t));
	x = fnv(x, P->units, (size_t)P->nunits * sizeof(jn_unit_t));
	x = fnv(x, P->unit_terms, (size_t)P->n_unit_terms * 4);
	x = fnv(x, P->btiles, (size_t)P->nbtiles * sizeof(jn_btile_t));
	x = fnv(x, P->pieces, (size_t)P->npieces * sizeof(jn_piece_t));
	x = fnv(x, P->items, (size_t)P->nitems * 8);
	x = fnv(x, &P->abs_bound, sizeof P->abs_bound);
	if (emu_walk_build(h)) return 0;
	x = fnv(x, P->wtasks, (size_t)P->nwtasks * sizeof(jn_wtask_t));
	x = fnv(x, P->wpieces, (size_t)P->nwpieces * sizeof(jn_wpiece_t));
	x = fnv(x, P->wlanes, (size_t)P->n_wlanes * 4);
	x = fnv(x, P->wwalks, (size_t)P->n_wwalks * 4);
	x = fnv(x, P->wrows, (size_t)P->n_wrows * 4);
	x = fnv(x, P->wrdst, (size_t)P->n_wrdst * 4);
	x = fnv(x, P->wgroups, (size_t)P->n_wgroups * 4);
	x = fnv(x, P->wgblock, (size_t)P->n_wgroups * 4);
	const int64_t nm = P->n_wme;
	double *a = malloc((nm ? nm : 1) * sizeof(double));
	int32_t *split = malloc((nm ? nm : 1) * 2 * sizeof(int32_t));
	uint8_t *gs = malloc(P->n_wgroups ? P->n_wgroups : 1);
	int sc = 0;
	if (!a || !split || !gs) { free(a); free(split); free(gs); return 0; }
	jn_walk_elements(P, P->me, a);
	jn_walk_int_elements(P, P->me, split, gs, &sc);
	x = fnv(x, a, (size_t)nm * 8);
	x = fnv(x, split, (size_t)nm * 8);
	x = fnv(x, gs, (size_t)P->n_wgroups);
	x = fnv(x, &sc, sizeof sc);
	free(a); free(split); free(gs);
	return x;
}
