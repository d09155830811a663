/*
 * jn_walk.c — host side of the walk engine (engine 5): directed
 * instructions, row groups, pieces, lane chunks and the walk element array
 * (the layout is described in jn_problem.h).
 *
 * Semantics are the reference Minerva kernels'
 * (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:
 * n list :20-77, p list :79-132, n x p lists :134-210, off-diagonal
 * transposes :212-462, |M| < 1e-12 skip of single-species terms :52-53).
 * The n x p contribution of a proton entry (p_i -> p_o, k_p) and a neutron
 * entry (n_i -> n_o, k_n) is s_p s_n M[k_n + Nd k_p] x[n_i + Nn_i p_i] into
 * y[n_o + Nn_o p_o]; here one of the two lists is walked by destination and
 * the other supplies the rows, and the same contributions are summed in
 * another order (each row sum is rounded once, at a place this plan fixes,
 * and the rounded sums are added as integers, so the order never changes a
 * result between runs).
 */
#define _GNU_SOURCE        /* qsort_r */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>
#include <unistd.h>

#include "jn_problem.h"

#define ERR(...) do { snprintf(err, errlen, __VA_ARGS__); goto fail; } while (0)
#define MASK31 0x7fffffffu

void jn_walk_free(jn_plan_t *p)
{
	free(p->wtasks); free(p->wpieces); free(p->wlanes); free(p->wwalks); free(p->wrows); free(p->wrdst);
	free(p->wgroups); free(p->wgblock); free(p->wtpos); free(p->wxperm);
	p->wtasks = NULL; p->wpieces = NULL; p->wlanes = NULL; p->wwalks = NULL; p->wrows = NULL; p->wrdst = NULL;
	p->wgroups = NULL; p->wgblock = NULL; p->wtpos = NULL; p->wxperm = NULL;
	p->wxt = 0;
	p->nwtasks = p->nwpieces = p->n_wlanes = p->n_wwalks = p->n_wrows = p->n_wrdst = p->n_wgroups = p->n_wme = 0;
	p->wvisits = p->wlane_slots = 0.0;
}

/* ------------------------------------------------------------------ */
/* element arrays on the host, built by all cores: work items are chunks  */
/* of one block (its elements, or the k_p rows of its transposed copy),   */
/* each independent of the others, so the result does not depend on the  */
/* number of threads                                                       */
/* ------------------------------------------------------------------ */
#define WALK_CHUNK (1 << 20)

typedef struct { int b, kind; int64_t e0, e1; } witem_t;     /* kind 0: elements [e0, e1); 1: transposed rows [e0, e1) */

/* the work items of every block: its elements and, where proton walks read it, its transposed copy */
static witem_t *walk_items(const jn_plan_t *p, int64_t *count)
{
	int64_t n = 0, cap = 1024;
	witem_t *it = (witem_t *)malloc((size_t)cap * sizeof(witem_t));
	for (int b = 0; b < p->nmes && it; b++) {
		const jn_me_t *M = &p->mes[b];
		for (int kind = 0; kind < 2; kind++) {
			if (kind && !(p->wtpos && p->wtpos[b] >= 0)) continue;
			const int64_t len = kind ? (int64_t)M->nd_p : M->len;
			const int64_t per = kind ? (M->nd_n ? (WALK_CHUNK + (int64_t)M->nd_n - 1) / (int64_t)M->nd_n : len) : WALK_CHUNK;
			for (int64_t e0 = 0; e0 < len; e0 += per) {
				if (n == cap) {
					cap *= 2;
					witem_t *g = (witem_t *)realloc(it, (size_t)cap * sizeof(witem_t));
					if (!g) { free(it); it = NULL; break; }
					it = g;
				}
				it[n++] = (witem_t){ b, kind, e0, e0 + per < len ? e0 + per : len };
			}
			if (!it) break;
		}
	}
	*count = n;
	return it;
}

typedef struct { const jn_plan_t *p; const witem_t *it; const double *me; double *out; } elem_job_t;

static void elem_item(int64_t i, void *v)
{
	const elem_job_t *j = (const elem_job_t *)v;
	const jn_plan_t *p = j->p;
	const witem_t *w = &j->it[i];
	const jn_me_t *M = &p->mes[w->b];
	if (w->kind == 0) {
		for (int64_t e = w->e0; e < w->e1; e++) {
			const double v = j->me[M->offset + e];
			/* single-species terms skip |M| < 1e-12 (matrix_vector_multiplication.c:52-53) */
			j->out[M->offset + e] = (M->single && fabs(v) < 1e-12) ? 0.0 : v;
		}
	} else {
		/* [k_p][k_n] copy of an n x p block stored [k_n + Nd_n k_p] */
		const int64_t nn = (int64_t)M->nd_n, npp = (int64_t)M->nd_p;
		double *t = j->out + p->wtpos[w->b];
		for (int64_t kp = w->e0; kp < w->e1; kp++)
			for (int64_t kn = 0; kn < nn; kn++) t[kp + npp * kn] = j->me[M->offset + kn + nn * kp];
	}
}

void jn_walk_elements(const jn_plan_t *p, const double *me, double *out)
{
	int64_t n = 0;
	witem_t *it = walk_items(p, &n);
	if (!it) {              /* out of memory for the item list: one block after another */
		for (int b = 0; b < p->nmes; b++) {
			witem_t one[2] = { { b, 0, 0, p->mes[b].len }, { b, 1, 0, (int64_t)p->mes[b].nd_p } };
			elem_job_t j = { p, one, me, out };
			elem_item(0, &j);
			if (p->wtpos && p->wtpos[b] >= 0) elem_item(1, &j);
		}
		return;
	}
	elem_job_t j = { p, it, me, out };
	jn_par_for(n, elem_item, &j);
	free(it);
}

typedef struct { const jn_plan_t *p; const witem_t *it; const double *me; double *imax; const int *sc; int32_t *split; } int_job_t;

/* a block's own element e as the walk element array holds it: single-species
   blocks store |M| < 1e-12 as 0 (matrix_vector_multiplication.c:52-53) */
static inline double own_element(const jn_me_t *M, const double *me, int64_t e)
{
	const double v = me[M->offset + e];
	return (M->single && fabs(v) < 1e-12) ? 0.0 : v;
}

/* max |a| over a chunk of a block's own elements */
static void int_max_item(int64_t i, void *v)
{
	const int_job_t *j = (const int_job_t *)v;
	const witem_t *w = &j->it[i];
	double m = 0.0;
	if (w->kind == 0) {
		const jn_me_t *M = &j->p->mes[w->b];
		for (int64_t e = w->e0; e < w->e1; e++) {
			const double x = fabs(own_element(M, j->me, e));
			if (x > m) m = x;           /* skips NaN as fmax does */
		}
	}
	j->imax[i] = m;
}

/* a 2^s: a product with the normal double 2^s is exact (|a 2^s| < 2^52
 * here) or rounds as ldexp does, so it gives ldexp's bits without its call */
static inline double scaled(double a, int s, double f)
{
	return f != 0.0 ? a * f : ldexp(a, s);
}

/* the 52-bit fixed-point split of a chunk (its elements, or its transposed rows) */
static void int_split_item(int64_t i, void *v)
{
	const int_job_t *j = (const int_job_t *)v;
	const jn_plan_t *p = j->p;
	const witem_t *w = &j->it[i];
	const jn_me_t *M = &p->mes[w->b];
	const int s = j->sc[w->b];
	const double f = s >= -1022 && s <= 1023 ? ldexp(1.0, s) : 0.0;    /* 0: ldexp per element */
	int64_t o, e0, e1;
	if (w->kind == 0) {
		o = M->offset;
		e0 = w->e0;
		e1 = w->e1;
	} else {            /* transposed rows [e0, e1) hold elements kp + Nd_p kn, copied from kn + Nd_n kp */
		o = p->wtpos[w->b];
		const int64_t npp = (int64_t)M->nd_p, nn = (int64_t)M->nd_n;
		for (int64_t kn = 0; kn < nn; kn++)
			for (int64_t kp = w->e0; kp < w->e1; kp++) {
				const int64_t q = o + kp + npp * kn, v = llrint(scaled(j->me[M->offset + kn + nn * kp], s, f));
				j->split[2 * q] = (int32_t)(v >> 24);
				j->split[2 * q + 1] = (int32_t)(v & 0xffffff);
			}
		return;
	}
	for (int64_t e = e0; e < e1; e++) {
		const int64_t v = llrint(scaled(own_element(M, j->me, e), s, f));
		j->split[2 * (o + e)] = (int32_t)(v >> 24);
		j->split[2 * (o + e) + 1] = (int32_t)(v & 0xffffff);
	}
}

void jn_walk_int_elements(const jn_plan_t *p, const double *me, int32_t *split, uint8_t *gshift, int *sc_min)
{
	int *sc = malloc((size_t)(p->nmes ? p->nmes : 1) * sizeof(int));
	double *bmax = calloc((size_t)(p->nmes ? p->nmes : 1), sizeof(double));
	int64_t n = 0;
	witem_t *it = walk_items(p, &n);
	double *imax = malloc((size_t)(n ? n : 1) * sizeof(double));
	int_job_t j = { p, it, me, imax, sc, split };
	if (it && imax) {
		jn_par_for(n, int_max_item, &j);
		for (int64_t i = 0; i < n; i++) bmax[it[i].b] = fmax(bmax[it[i].b], imax[i]);
	} else {
		for (int b = 0; b < p->nmes; b++)
			for (int64_t e = 0; e < p->mes[b].len; e++) bmax[b] = fmax(bmax[b], fabs(own_element(&p->mes[b], me, e)));
	}
	/* each block keeps 52 bits against its own max|M|: |v| 2^sc < 2^52 */
	int lo = 1 << 30;
	for (int b = 0; b < p->nmes; b++) {
		int eb = 0;
		if (bmax[b] > 0.0) frexp(bmax[b], &eb);     /* m < 2^eb */
		sc[b] = bmax[b] > 0.0 ? 52 - eb : (1 << 30);
		if (sc[b] < lo) lo = sc[b];
	}
	if (lo == (1 << 30)) lo = 0;
	for (int b = 0; b < p->nmes; b++)
		if (sc[b] == (1 << 30)) sc[b] = lo;     /* an all-zero block */
	if (it && imax) {
		jn_par_for(n, int_split_item, &j);
	} else {
		for (int b = 0; b < p->nmes; b++) {
			witem_t one[2] = { { b, 0, 0, p->mes[b].len }, { b, 1, 0, (int64_t)p->mes[b].nd_p } };
			int_job_t jb = { p, one, me, NULL, sc, split };
			int_split_item(0, &jb);
			if (p->wtpos && p->wtpos[b] >= 0) int_split_item(1, &jb);
		}
	}
	for (int64_t g = 0; g < p->n_wgroups; g++) {
		const int d = sc[p->wgblock[g]] - lo;
		gshift[g] = (uint8_t)(d > 255 ? 255 : d);
	}
	*sc_min = lo;
	free(sc); free(bmax); free(it); free(imax);
}

/* growable arrays */
typedef struct { void *a; int64_t n, cap; size_t sz; } vec_t;
static int vec_reserve(vec_t *v, int64_t add)
{
	if (v->n + add <= v->cap) return 0;
	int64_t c = v->cap ? v->cap : 1024;
	while (c < v->n + add) c *= 2;
	void *b = realloc(v->a, (size_t)c * v->sz);
	if (!b) return 1;
	v->a = b;
	v->cap = c;
	return 0;
}

typedef struct { uint32_t src, dst, k, sign; } row_t;

static int cmp_row(const void *a, const void *b)
{
	const row_t *x = a, *y = b;
	if (x->k != y->k) return x->k < y->k ? -1 : 1;
	if (x->dst != y->dst) return x->dst < y->dst ? -1 : 1;
	if (x->src != y->src) return x->src < y->src ? -1 : 1;
	return (int)x->sign - (int)y->sign;
}

static int cmp_instr_block(const void *a, const void *b, void *plan)
{
	const jn_plan_t *P = (const jn_plan_t *)plan;
	const jn_instr_t *x = &P->instr[*(const int *)a], *y = &P->instr[*(const int *)b];
	if (x->me != y->me) return x->me < y->me ? -1 : 1;
	if (x->bout != y->bout) return x->bout < y->bout ? -1 : 1;
	if (x->bin != y->bin) return x->bin < y->bin ? -1 : 1;
	return *(const int *)a - *(const int *)b;
}

/* lane chunks of width U over the walks [w0, w0 + nw) */
static int64_t chunks_for(const uint32_t *walks, int64_t w0, int64_t nw, int U)
{
	int64_t n = 0;
	for (int64_t w = 0; w < nw; w++) n += ((walks[2 * (w0 + w) + 1] & 0xffffu) + U - 1) / U;
	return n;
}

/* The lane records of one walk view.  They depend on the list, its view and
 * the chunk width only, so every directed instruction that walks the same
 * view shares them.  Views take their place in the lane array and the walk
 * table in the order of their first use; their records are built by all
 * host cores. */
typedef struct {
	const jn_list_t *W;
	int dir, U;
	int64_t w0, nw;         /* the view's walks in jn_plan_t.walks */
	int64_t nchunk, nsets;
	int64_t lanes0;         /* first lane word */
	uint32_t *wtab;         /* walk table of the view's sets (view-local) */
	int64_t nwtab;
	int64_t walks0;         /* first entry in the plan's walk table */
	uint32_t *set_walk0;    /* per set: first wtab entry (view-local), walk count */
	int status;             /* 1: out of host memory */
} wview_t;

/* One directed instruction (forward, or the transpose of an off-diagonal
 * one): its rows cut into pieces, with row, slot and group arrays local to
 * it until they are joined in instruction order. */
typedef struct {
	int q, dir, view;
	uint32_t *rows, *rdst, *groups;
	int32_t *gblock;
	int64_t nrows, nrdst, ngroups;
	jn_wpiece_t *pieces;    /* row0, rdst0, group0 local */
	int64_t *prows;         /* rows of each piece */
	int64_t npieces;
	int status;             /* 1 memory, 2 row index, 3 walk destination, 4 walk entry, 5 row groups */
} wdir_t;

typedef struct {
	jn_plan_t *p;
	wview_t *views;
	wdir_t *dirs;
	uint32_t *lanes;
} wjob_t;

/* the walk list, the row list and element-row addressing of instruction q */
typedef struct {
	const jn_list_t *W, *RL;
	int wp;
	int64_t base, stride;   /* element row of k_row: base + stride k_row */
	int64_t wlen, rlen;     /* walk-side and row-side k ranges */
} wsides_t;

static wsides_t walk_sides(const jn_plan_t *p, int q)
{
	const jn_instr_t *x = &p->instr[q];
	const jn_me_t *M = &p->mes[x->me];
	wsides_t w = { NULL, NULL, 0, M->offset, 0, M->len, 1 };
	if (x->kind == JN_KIND_NP) {
		const jn_list_t *Ln = &p->lists[x->ln], *Lp = &p->lists[x->lp];
		w.wp = Lp->len > Ln->len;
		w.W = w.wp ? Lp : Ln;
		w.RL = w.wp ? Ln : Lp;
		w.base = w.wp ? p->wtpos[x->me] : M->offset;
		w.stride = w.wp ? (int64_t)M->nd_p : (int64_t)M->nd_n;
		w.wlen = w.wp ? (int64_t)M->nd_p : (int64_t)M->nd_n;
		w.rlen = w.wp ? (int64_t)M->nd_n : (int64_t)M->nd_p;
	} else if (x->kind == JN_KIND_N) {
		w.W = &p->lists[x->ln];
	} else {
		w.W = &p->lists[x->lp];
		w.wp = 1;
	}
	return w;
}

/* lane records and walk table of one view: one set per 32 chunks */
static void view_lanes(int64_t vi, void *v)
{
	const wjob_t *J = (const wjob_t *)v;
	const jn_plan_t *p = J->p;
	wview_t *V = &J->views[vi];
	const int U = V->U, LW = JN_WALK_LANE_WORDS(U);
	const int64_t w0 = V->w0, nw = V->nw, nchunk = V->nchunk, nsets = V->nsets;
	uint32_t *chunk = malloc((size_t)(nchunk ? nchunk : 1) * 3 * sizeof(uint32_t));   /* first ent index, count, walk */
	V->wtab = malloc((size_t)(nsets ? nsets : 1) * 32 * sizeof(uint32_t));
	V->set_walk0 = malloc((size_t)(nsets ? nsets : 1) * 2 * sizeof(uint32_t));
	if (!chunk || !V->wtab || !V->set_walk0) { free(chunk); V->status = 1; return; }
	{
		int64_t c = 0;
		for (int64_t w = 0; w < nw; w++) {
			const uint32_t a = p->walks[2 * (w0 + w)], len = p->walks[2 * (w0 + w) + 1] & 0xffffu;
			for (uint32_t o = 0; o < len; o += (uint32_t)U) {
				chunk[3 * c] = a + o;
				chunk[3 * c + 1] = len - o < (uint32_t)U ? len - o : (uint32_t)U;
				chunk[3 * c + 2] = (uint32_t)w;
				c++;
			}
		}
	}
	for (int64_t s = 0; s < nsets; s++) {
		uint32_t *L = J->lanes + V->lanes0 + s * 32 * LW;
		uint32_t *T = V->wtab + V->nwtab;
		int nwalk = 0;
		for (int l = 0; l < 32;) {
			/* the run of this set's lanes [l, l1) that hold chunks of one walk: its
			   entries (contiguous in the walk view) are dealt to the run's lanes in
			   turn, entry i to lane l + i mod nl at position i / nl */
			int l1 = l + 1;
			const int64_t c0 = s * 32 + l;
			if (c0 < nchunk)
				while (l1 < 32 && s * 32 + l1 < nchunk && chunk[3 * (s * 32 + l1) + 2] == chunk[3 * c0 + 2]) l1++;
			else
				l1 = 32;
			const int nl = l1 - l;
			uint32_t e0 = 0, ne = 0;
			if (c0 < nchunk) {
				T[nwalk++] = p->walks[2 * (w0 + chunk[3 * c0 + 2]) + 1] >> 16;
				e0 = chunk[3 * c0];
				for (int64_t c = c0; c < s * 32 + l1; c++) ne += chunk[3 * c + 1];
			}
			for (int r = 0; r < nl; r++) {
				uint32_t src[8], koff[8];
				for (int u = 0; u < U; u++) {
					const uint32_t i = (uint32_t)(u * nl + r);
					/* padding repeats the lane's first source with coefficient 0 */
					const uint32_t e = e0 + (i < ne ? i : (uint32_t)r);
					src[u] = c0 < nchunk ? p->ent[2 * e] & 0xffffu : 0u;
					koff[u] = i < ne ? (p->ent[2 * e + 1] & 0x3fffffffu) |
								   ((p->ent[2 * e + 1] >> 31) ? JN_WALK_NEG : JN_WALK_POS)
							 : 0u;
				}
				uint32_t mul = 0;
				for (int u = 0; u < U; u++) mul |= (koff[u] >> 30) << (2 * u);
				L[l + r] = (c0 < nchunk ? (uint32_t)(nwalk - 1) : 0u) | (mul << 16);
				for (int k = 0; k < U / 2; k++) L[(1 + k) * 32 + l + r] = src[2 * k] | (src[2 * k + 1] << 16);
				for (int u = 0; u < U; u++) L[(1 + U / 2 + u) * 32 + l + r] = koff[u];
			}
			l = l1;
		}
		V->set_walk0[2 * s] = (uint32_t)V->nwtab;
		V->set_walk0[2 * s + 1] = (uint32_t)nwalk;
		V->nwtab += nwalk;
	}
	free(chunk);
}

/* rows of one directed instruction, checked and cut into pieces: runs of
   whole row groups with at most JN_WALK_RS distinct destination rows (a
   group with more is split, and its element row read once per part) */
static void dir_pieces(int64_t di, void *v)
{
	const wjob_t *J = (const wjob_t *)v;
	const jn_plan_t *p = J->p;
	wdir_t *D = &J->dirs[di];
	const int q = D->q, dir = D->dir;
	const jn_instr_t *x = &p->instr[q];
	const jn_block_t *bi = &p->blocks[x->bin], *bo = &p->blocks[x->bout];
	const jn_block_t *bs = dir ? bo : bi, *bd = dir ? bi : bo;
	const wsides_t S = walk_sides(p, q);
	const jn_list_t *RL = S.RL;
	const int wp = S.wp;
	const int64_t nr = RL ? RL->len : (wp ? bo->Nn : bo->Np);
	row_t *R = malloc((size_t)(nr ? nr : 1) * sizeof(row_t));
	D->rows = malloc((size_t)(nr ? nr : 1) * sizeof(uint32_t));
	D->groups = malloc((size_t)(nr ? nr : 1) * sizeof(uint32_t));
	D->gblock = malloc((size_t)(nr ? nr : 1) * sizeof(int32_t));
	D->rdst = malloc((size_t)(nr ? nr : 1) * sizeof(uint32_t));      /* at most one new slot row per row */
	D->pieces = malloc((size_t)(nr ? nr : 1) * sizeof(jn_wpiece_t));
	D->prows = malloc((size_t)(nr ? nr : 1) * sizeof(int64_t));
	if (!R || !D->rows || !D->groups || !D->gblock || !D->rdst || !D->pieces || !D->prows) {
		free(R);
		D->status = 1;
		return;
	}
	if (RL) {
		for (int64_t e = 0; e < nr; e++) {
			const int32_t *t = RL->triples + 3 * e;
			R[e].src = (uint32_t)(dir ? t[1] : t[0]);
			R[e].dst = (uint32_t)(dir ? t[0] : t[1]);
			R[e].k = (uint32_t)t[2] & MASK31;
			R[e].sign = (uint32_t)t[2] >> 31;
		}
		qsort(R, (size_t)nr, sizeof(row_t), cmp_row);
	} else {
		for (int64_t r = 0; r < nr; r++) R[r] = (row_t){ (uint32_t)r, (uint32_t)r, 0u, 0u };
	}
	/* row index bounds: sources and destinations inside their blocks, k inside the element block */
	const int64_t src_rows = wp ? bs->Nn : bs->Np, dst_rows = wp ? bd->Nn : bd->Np;
	for (int64_t e = 0; e < nr; e++)
		if (R[e].src >= src_rows || R[e].dst >= dst_rows || R[e].src > 0xffffu || R[e].dst > 0xffffu || R[e].k >= S.rlen) {
			free(R);
			D->status = 2;
			return;
		}
	/* walk view and its bounds: destinations and sources inside their blocks, k inside the block */
	const wview_t *V = &J->views[D->view];
	const int64_t src_cols = wp ? bs->Np : bs->Nn, dst_cols = wp ? bd->Np : bd->Nn;
	for (int64_t w = 0; w < V->nw; w++) {
		const uint32_t a = p->walks[2 * (V->w0 + w)], len = p->walks[2 * (V->w0 + w) + 1] & 0xffffu;
		if ((p->walks[2 * (V->w0 + w) + 1] >> 16) >= dst_cols) { free(R); D->status = 3; return; }
		for (uint32_t e = a; e < a + len; e++)
			if ((p->ent[2 * e] & 0xffffu) >= src_cols || (p->ent[2 * e + 1] & MASK31) >= S.wlen) {
				free(R);
				D->status = 4;
				return;
			}
	}
	int64_t r0 = 0;
	while (r0 < nr) {
		int rs = 0;
		int64_t r1 = r0;
		const int64_t rdst0 = D->nrdst, row0 = D->nrows, group0 = D->ngroups;
		uint32_t *slot = D->rdst + rdst0;       /* the piece's destination rows */
		while (r1 < nr) {
			/* the next group [r1, g1) and the destinations it would add */
			int64_t g1 = r1;
			while (g1 < nr && R[g1].k == R[r1].k) g1++;
			int add = 0;
			for (int64_t e = r1; e < g1; e++) {
				if (e > r1 && R[e].dst == R[e - 1].dst) continue;
				int in = 0;
				for (int i = 0; i < rs; i++) in |= slot[i] == R[e].dst;
				add += !in;
			}
			if (rs > 0 && rs + add > JN_WALK_RS) break;
			/* take the group, or as much of it as fits */
			int64_t e = r1;
			for (; e < g1; e++) {
				int in = 0;
				for (int i = 0; i < rs; i++) in |= slot[i] == R[e].dst;
				if (!in) {
					if (rs == JN_WALK_RS) break;
					slot[rs++] = R[e].dst;
				}
			}
			D->groups[D->ngroups] = (uint32_t)(S.base + S.stride * (int64_t)R[r1].k);
			D->gblock[D->ngroups++] = x->me;
			r1 = e;
			if (e < g1) break;      /* a split group ends the piece */
		}
		/* row words: slot rows in order of first appearance */
		for (int64_t e = r0; e < r1; e++) {
			int sl = 0;
			while (slot[sl] != R[e].dst) sl++;
			const int end = e + 1 == r1 || R[e + 1].k != R[e].k;
			D->rows[D->nrows + (e - r0)] = R[e].src | ((uint32_t)sl << 16) | (end ? JN_WALK_GROUP_END : 0u) | (R[e].sign << 31);
		}
		D->nrows += r1 - r0;
		D->nrdst += rs;
		if (D->ngroups - group0 >= (1 << 23)) { free(R); D->status = 5; return; }
		jn_wpiece_t *P = &D->pieces[D->npieces];
		P->src_off = (int32_t)bs->offset;
		P->dst_off = (int32_t)bd->offset;
		P->src_stride = (int32_t)(wp ? bs->Np : bs->Nn);
		P->Nn_dst = (int32_t)bd->Nn;
		P->row0 = (int32_t)row0;
		P->rdst0 = (int32_t)rdst0;
		P->group0 = (int32_t)group0;
		P->meta = (uint32_t)rs | ((uint32_t)wp << 8) | ((uint32_t)(D->ngroups - group0) << 9);
		D->prows[D->npieces++] = r1 - r0;
		r0 = r1;
	}
	free(R);
}

static void wdir_free(wdir_t *D)
{
	free(D->rows); free(D->rdst); free(D->groups); free(D->gblock); free(D->pieces); free(D->prows);
	D->rows = D->rdst = D->groups = NULL;
	D->gblock = NULL;
	D->pieces = NULL;
	D->prows = NULL;
}

int jn_walk_build(jn_plan_t *p, char *err, size_t errlen)
{
	vec_t tasks = { 0, 0, 0, sizeof(jn_wtask_t) }, pieces = { 0, 0, 0, sizeof(jn_wpiece_t) };
	vec_t walks = { 0, 0, 0, sizeof(uint32_t) };
	vec_t rows = { 0, 0, 0, sizeof(uint32_t) }, rdst = { 0, 0, 0, sizeof(uint32_t) };
	vec_t groups = { 0, 0, 0, sizeof(uint32_t) }, gblock = { 0, 0, 0, sizeof(int32_t) };
	uint32_t *lanes = NULL;
	int64_t nlanes = 0;
	int *order = NULL, *view_of = NULL;
	wview_t *views = NULL;
	wdir_t *dirs = NULL;
	int64_t nviews = 0, ndirs = 0;
	double visits = 0.0, slots = 0.0;
	jn_walk_free(p);
	p->wtpos = malloc((size_t)(p->nmes ? p->nmes : 1) * sizeof(int64_t));
	view_of = malloc((size_t)(p->nlists ? p->nlists : 1) * 2 * sizeof(int));
	views = calloc((size_t)(p->nlists ? p->nlists : 1) * 2, sizeof(wview_t));
	dirs = calloc((size_t)(p->ninstr ? p->ninstr : 1) * 2, sizeof(wdir_t));
	if (!p->wtpos || !view_of || !views || !dirs) ERR("out of host memory");
	for (int v = 0; v < 2 * p->nlists; v++) view_of[v] = -1;
	if (p->dim >= 0x7fffffffll) ERR("dimension %lld: too large for the walk engine's 32-bit offsets", (long long)p->dim);
	/* transposed copies of the n x p blocks that proton-walk instructions use */
	for (int b = 0; b < p->nmes; b++) p->wtpos[b] = -1;
	p->n_wme = p->n_me;
	for (int q = 0; q < p->ninstr; q++) {
		const jn_instr_t *x = &p->instr[q];
		if (x->kind != JN_KIND_NP || p->lists[x->lp].len <= p->lists[x->ln].len || p->wtpos[x->me] >= 0) continue;
		p->wtpos[x->me] = p->n_wme;
		p->n_wme += p->mes[x->me].len;
	}
	if (p->n_wme >= 0x3fffffffll) ERR("%lld walk matrix elements: too many for the walk engine", (long long)p->n_wme);
	/* instructions in matrix-element-block order: the ~10 instructions (and
	   both directions of each) that read one block run one after another, so
	   L2 holds the block's rows while all of them gather from it */
	order = malloc((size_t)(p->ninstr > 0 ? p->ninstr : 1) * sizeof(int));
	if (!order) ERR("out of host memory");
	for (int q = 0; q < p->ninstr; q++) order[q] = q;
	qsort_r(order, (size_t)p->ninstr, sizeof(int), cmp_instr_block, p);
	/* the directed instructions in order, and the walk views in order of first use */
	for (int oq = 0; oq < p->ninstr; oq++) {
		const int q = order[oq];
		const jn_instr_t *x = &p->instr[q];
		const jn_block_t *bi = &p->blocks[x->bin], *bo = &p->blocks[x->bout];
		if (x->kind == JN_KIND_N && bi->Np != bo->Np) ERR("instruction %d: spectator rows differ", q);
		if (x->kind == JN_KIND_P && bi->Nn != bo->Nn) ERR("instruction %d: spectator columns differ", q);
		const wsides_t S = walk_sides(p, q);
		if (S.W->len == 0) continue;
		const int64_t nr = S.RL ? S.RL->len : (S.wp ? bo->Nn : bo->Np);
		for (int dir = 0; dir < 2; dir++) {
			if (dir == 1 && x->bin == x->bout) break;
			if (nr == 0) continue;
			const int key = 2 * (int)(S.W - p->lists) + dir;
			if (view_of[key] < 0) {
				wview_t *V = &views[nviews];
				V->W = S.W;
				V->dir = dir;
				V->w0 = dir ? S.W->walk_in : S.W->walk_out;
				V->nw = dir ? S.W->nwalk_in : S.W->nwalk_out;
				/* the chunk width with the fewest lane slots, counting a row's fixed
				   cost as about two entries */
				int U = 8;
				double best = 1e300;
				for (int u = 8; u >= 2; u /= 2) {
					const int64_t nc = chunks_for(p->walks, V->w0, V->nw, u);
					const double cost = (double)((nc + 31) / 32) * 32 * (u + 2);
					if (cost < best) { best = cost; U = u; }
				}
				V->U = U;
				V->nchunk = chunks_for(p->walks, V->w0, V->nw, U);
				V->nsets = (V->nchunk + 31) / 32;
				V->lanes0 = nlanes;
				nlanes += V->nsets * 32 * JN_WALK_LANE_WORDS(U);
				view_of[key] = (int)nviews++;
			}
			dirs[ndirs].q = q;
			dirs[ndirs].dir = dir;
			dirs[ndirs].view = view_of[key];
			ndirs++;
		}
	}
	if (nlanes > 0xffffffffll) ERR("the walk plan is too large");
	lanes = malloc((size_t)(nlanes ? nlanes : 1) * sizeof(uint32_t));
	if (!lanes) ERR("out of host memory");
	{
		wjob_t job = { p, views, dirs, lanes };
		jn_par_for(nviews, view_lanes, &job);
		jn_par_for(ndirs, dir_pieces, &job);
	}
	for (int64_t v = 0; v < nviews; v++)
		if (views[v].status) ERR("out of host memory");
	for (int64_t d = 0; d < ndirs; d++) {
		static const char *const what[] = { "", "out of host memory", "row index out of range",
						     "walk destination out of range", "walk entry out of range", "too many row groups" };
		if (dirs[d].status == 1) ERR("out of host memory");
		if (dirs[d].status) ERR("instruction %d: %s", dirs[d].q, what[dirs[d].status]);
	}
	/* join in instruction order: a view's walk table at its first use, then
	   the instruction's rows and pieces, and per piece one task per set */
	for (int64_t d = 0; d < ndirs; d++) {
		wdir_t *D = &dirs[d];
		wview_t *V = &views[D->view];
		const int U = V->U, LW = JN_WALK_LANE_WORDS(U);
		if (V->wtab) {
			if (vec_reserve(&walks, V->nwtab)) ERR("out of host memory");
			V->walks0 = walks.n;
			memcpy((uint32_t *)walks.a + walks.n, V->wtab, (size_t)V->nwtab * sizeof(uint32_t));
			walks.n += V->nwtab;
			free(V->wtab);
			V->wtab = NULL;
		}
		const int64_t row_base = rows.n, rdst_base = rdst.n, group_base = groups.n;
		if (vec_reserve(&rows, D->nrows) || vec_reserve(&rdst, D->nrdst) || vec_reserve(&groups, D->ngroups) ||
		    vec_reserve(&gblock, D->ngroups) || vec_reserve(&pieces, D->npieces) || vec_reserve(&tasks, D->npieces * V->nsets))
			ERR("out of host memory");
		memcpy((uint32_t *)rows.a + rows.n, D->rows, (size_t)D->nrows * sizeof(uint32_t));
		memcpy((uint32_t *)rdst.a + rdst.n, D->rdst, (size_t)D->nrdst * sizeof(uint32_t));
		memcpy((uint32_t *)groups.a + groups.n, D->groups, (size_t)D->ngroups * sizeof(uint32_t));
		memcpy((int32_t *)gblock.a + gblock.n, D->gblock, (size_t)D->ngroups * sizeof(int32_t));
		rows.n += D->nrows; rdst.n += D->nrdst; groups.n += D->ngroups; gblock.n += D->ngroups;
		for (int64_t k = 0; k < D->npieces; k++) {
			jn_wpiece_t P = D->pieces[k];
			P.row0 += (int32_t)row_base;
			P.rdst0 += (int32_t)rdst_base;
			P.group0 += (int32_t)group_base;
			if ((P.meta >> 8) & 1u) p->wxt = 1;
			const int64_t pi = pieces.n++;
			((jn_wpiece_t *)pieces.a)[pi] = P;
			for (int64_t s = 0; s < V->nsets; s++) {
				jn_wtask_t *T = (jn_wtask_t *)tasks.a + tasks.n++;
				T->piece = (uint32_t)pi;
				T->lanes = (uint32_t)(V->lanes0 + s * 32 * LW);
				T->walk0 = (uint32_t)(V->walks0 + V->set_walk0[2 * s]);
				T->meta = V->set_walk0[2 * s + 1] | ((uint32_t)U << 8);
				const int64_t used = (s + 1) * 32 <= V->nchunk ? 32 : V->nchunk - s * 32;
				visits += (double)D->prows[k] * (double)used * U;
				slots += (double)D->prows[k] * 32.0 * U;
			}
		}
		wdir_free(D);
	}
	/* tasks stay in this order: warps take the next one from a counter, so
	   warps that run at the same time work on neighbouring instructions and
	   share their matrix elements in L2 */
	/* the transposed view of x that proton walks read: block [n][p] */
	if (p->wxt) {
		p->wxperm = malloc((size_t)(p->dim ? p->dim : 1) * sizeof(int32_t));
		if (!p->wxperm) ERR("out of host memory");
		for (int b = 0; b < p->nblocks; b++) {
			const jn_block_t *B = &p->blocks[b];
			for (int64_t n = 0; n < B->Nn; n++)
				for (int64_t q = 0; q < B->Np; q++) p->wxperm[B->offset + n * B->Np + q] = (int32_t)(B->offset + q * B->Nn + n);
		}
	}
	/* spare row words: the kernel reads up to two words past a task's last row ahead of time */
	if (vec_reserve(&rows, JN_WALK_ROW_SPARE)) ERR("out of host memory");
	for (int k = 0; k < JN_WALK_ROW_SPARE; k++) ((uint32_t *)rows.a)[rows.n + k] = 0u;
	if (tasks.n > 0xf0000000ll || walks.n > 0xffffffffll || rows.n > 0x7fffffffll ||
	    rdst.n > 0x7fffffffll || groups.n > 0x7fffffffll || pieces.n > 0xffffffffll)
		ERR("the walk plan is too large");
	p->wtasks = tasks.a; p->nwtasks = tasks.n;
	p->wpieces = pieces.a; p->nwpieces = pieces.n;
	p->wlanes = lanes; p->n_wlanes = nlanes;
	p->wwalks = walks.a; p->n_wwalks = walks.n;
	p->wrows = rows.a; p->n_wrows = rows.n;         /* plus the spare words */
	p->wrdst = rdst.a; p->n_wrdst = rdst.n;
	p->wgroups = groups.a; p->n_wgroups = groups.n;
	p->wgblock = gblock.a;
	p->wvisits = visits;
	p->wlane_slots = slots;
	for (int64_t v = 0; v < nviews; v++) free(views[v].set_walk0);
	free(views); free(dirs); free(view_of); free(order);
	return 0;
fail:
	free(tasks.a); free(pieces.a); free(lanes); free(walks.a); free(rows.a); free(rdst.a); free(groups.a);
	free(gblock.a);
	if (views)
		for (int64_t v = 0; v < nviews; v++) { free(views[v].set_walk0); free(views[v].wtab); }
	if (dirs)
		for (int64_t d = 0; d < ndirs; d++) wdir_free(&dirs[d]);
	free(views); free(dirs); free(view_of); free(order);
	free(p->wtpos); free(p->wxperm);
	p->wtpos = NULL;
	p->wxperm = NULL;
	p->wxt = 0;
	p->n_wme = 0;
	return 1;
}
