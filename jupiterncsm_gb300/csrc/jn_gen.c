/*
 * jn_gen.c — synthetic NCSM problem generator in the Anicre / JupiterNCSM
 * on-disk formats.
 *
 * JupiterNCSM takes its M-scheme basis, its index lists and its combination
 * table from Anicre, an external program that is not part of the reference
 * tree.  The formats are defined by their consumers, and this file writes
 * exactly what those consumers parse:
 *
 *   comb.txt           combination table: "mp-states" ARRAYMP rows
 *                      (src/Utilities/combination_table/combination_table.c:419-468),
 *                      "Conn lists" ARRAY rows (:470-522), both
 *                      "Matrix-elements V" sections (:524-640) and
 *                      CALCBLOCK rows (src/Utilities/calculation_blocks/
 *                      calculation_blocks.c:31-84).  One shared 1-based id
 *                      space: basis blocks 1..nb first, because Bacchus'
 *                      vector files are named vec_<i+1> by basis-block
 *                      position (src/Bacchus/vector/vector.c:98-128).
 *   index_list_<id>    packed {int in, int out, int matrix_index} records,
 *                      sign of the term in bit 31 of matrix_index
 *                      (src/Minerva/index_triple/index_triple.h:6-11,
 *                      src/Aurora/index_list/index_list.c:55-56).
 *   <id>_matrix_elements  size_t n_dim, size_t p_dim, double[]
 *                      (src/Minerva/matrix_block/matrix_block.c:22-62).
 *   evaluation order   "BLOCK: in out list [list] me" rows as Mars writes
 *                      them (src/Mars/programs/mars.c:172-199).
 *   <t>_inds_index_lists/basis_energy_<E>
 *                      k-particle states of energy E as packed shorts, grouped
 *                      by M, which Mercury reads to enumerate connections
 *                      (src/Mercury/connection_list/connection_list.c:448-522).
 *   bacchus.conf       the Bacchus run file (src/Bacchus/settings/settings.c:79-211).
 *
 * Conventions (the ones the consumers pin down):
 *  - single-particle orbitals are ordered (e, l, j asc, m desc)
 *    (src/Neptune/bases/sp_states.c:7-35); orbital s is state 2s for a
 *    proton and 2s+1 for a neutron in Neptune's interleaved numbering;
 *    m and M are stored doubled.
 *  - a vector block is [Np][Nn] row-major, element n + Nn*p
 *    (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:58-63).
 *  - an index list for (species, k, E_in, M_in, E_out, M_out, depth) holds,
 *    for every Slater determinant |in> of sub-basis (E_in,M_in), every
 *    k-particle subset alpha of |in> with energy `depth`, and every k-particle
 *    state beta with energy depth+dE and M(beta) = M(alpha)+dM that fits, the
 *    triple (in, out, connection | sign), where |out> = +-O(beta,alpha)|in>.
 *  - the connection index follows Mercury's enumeration: alpha in
 *    basis_energy_<depth> order, then beta in basis_energy_<depth+dE> order
 *    among the states with M(alpha)+dM
 *    (src/Mercury/connection_list/connection_list.c:448-498); a
 *    proton x neutron block is indexed k_n + Nd_n*k_p (:108-147).
 *  - O(beta,alpha) = a+_{b1}..a+_{bk} a_{ak}..a_{a1}; with protons ordered
 *    before neutrons a mixed operator factorises into (proton part) x
 *    (neutron part) with no extra sign.
 *  - diagonal basis-block pairs carry both orders of every transition;
 *    off-diagonal pairs are listed once (in = lower block id) and Minerva
 *    applies the transpose (matrix_vector_multiplication.c:212-462).
 *
 * The interaction is synthetic and seeded: every M-scheme matrix element
 * <beta|V|alpha> is a normal deviate computed from a counter-based hash of
 * the unordered pair {alpha, beta}, so V is symmetric by construction and
 * independent of enumeration order.  M, parity and Tz conservation follow
 * from the basis (all blocks share total M and parity; species are kept
 * apart).  The harmonic-oscillator term hw * sum_i e_i is folded into the
 * diagonal two-body elements as hw (e_a + e_b)/(A-1).
 */
#include "jn_gen.h"
#include "jn_jt.h"

#include <errno.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#define MAXW 8            /* 512 orbitals per species */
#define SIGN_BIT 0x80000000u

typedef struct { int e, l, j, m; } sp_t;
typedef struct { uint64_t w[MAXW]; } mask_t;

/* ------------------------------------------------------------------ */
/* error handling: every failure returns a code and a message          */
/* ------------------------------------------------------------------ */
static char g_err[512];
const char *jn_gen_last_error(void) { return g_err; }
#define FAIL(code, ...) do { snprintf(g_err, sizeof g_err, __VA_ARGS__); return (code); } while (0)

static void *xcalloc(size_t n, size_t s) { void *p = calloc(n ? n : 1, s ? s : 1); return p; }

/* growable array */
typedef struct { void *a; size_t n, cap, es; } vec_t;
static int vpush(vec_t *v, const void *e)
{
	if (v->n == v->cap) {
		size_t nc = v->cap ? 2 * v->cap : 64;
		void *na = realloc(v->a, nc * v->es);
		if (!na) return -1;
		v->a = na; v->cap = nc;
	}
	memcpy((char *)v->a + v->n * v->es, e, v->es);
	v->n++;
	return 0;
}

/* ------------------------------------------------------------------ */
/* counter-based normal deviates (splitmix64 + Box-Muller)             */
/* ------------------------------------------------------------------ */
static uint64_t mix64(uint64_t z)
{
	z += 0x9e3779b97f4a7c15ull;
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

double jn_gen_pair_normal(uint64_t seed, uint64_t tag, uint64_t ka, uint64_t kb)
{
	uint64_t lo = ka < kb ? ka : kb, hi = ka < kb ? kb : ka;
	uint64_t h = mix64(seed ^ mix64(tag ^ mix64(lo ^ mix64(hi))));
	uint64_t h2 = mix64(h);
	/* 53-bit uniforms in (0,1] and [0,1) */
	double u1 = ((double)(h >> 11) + 1.0) * (1.0 / 9007199254740992.0);
	double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
	return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* ------------------------------------------------------------------ */
/* single-particle basis                                               */
/* ------------------------------------------------------------------ */
static int build_sp(int emax, sp_t **out)
{
	int n = 0;
	for (int e = 0; e <= emax; e++) n += (e + 1) * (e + 2);
	sp_t *sp = xcalloc(n, sizeof(sp_t));
	int i = 0;
	for (int e = 0; e <= emax; e++)
		for (int l = e & 1; l <= e; l += 2)
			for (int j = 2 * l - 1; j <= 2 * l + 1; j += 2) {
				if (j < 0) continue;
				for (int m = j; m >= -j; m -= 2) {
					sp[i].e = e; sp[i].l = l; sp[i].j = j; sp[i].m = m;
					i++;
				}
			}
	*out = sp;
	return n;
}

/* ------------------------------------------------------------------ */
/* k-particle states: sorted orbital tuples, grouped by energy, and    */
/* within an energy by M ascending then lexicographically.             */
/* ------------------------------------------------------------------ */
typedef struct {
	int k;
	int emax;               /* largest energy kept */
	int n;                  /* number of states */
	short *orb;             /* n*k orbitals */
	int *E, *M;
	int *ebeg;              /* states of energy E: [ebeg[E], ebeg[E+1]) */
	/* within energy E, M-segments: for lookup of (E,M) -> [beg,end) */
	int mmin, mmax;         /* doubled M range */
	int *mseg;              /* (emax+1) x (mmax-mmin+2)/... begins; see kst_range */
	int mstride;
	int *rank;              /* position of state inside its (E,M) segment */
} kst_t;

static const sp_t *g_sp_for_sort;
static int g_k_for_sort;
static int cmp_kstate(const void *a, const void *b)
{
	const short *x = a, *y = b;
	int k = g_k_for_sort;
	int ex = 0, ey = 0, mx = 0, my = 0;
	for (int i = 0; i < k; i++) {
		ex += g_sp_for_sort[x[i]].e; mx += g_sp_for_sort[x[i]].m;
		ey += g_sp_for_sort[y[i]].e; my += g_sp_for_sort[y[i]].m;
	}
	if (ex != ey) return ex - ey;
	if (mx != my) return mx - my;
	for (int i = 0; i < k; i++)
		if (x[i] != y[i]) return x[i] - y[i];
	return 0;
}

static void kst_free(kst_t *t)
{
	free(t->orb); free(t->E); free(t->M); free(t->ebeg); free(t->mseg); free(t->rank);
	memset(t, 0, sizeof *t);
}

static int build_kst(const sp_t *sp, int nsp, int k, int emax, kst_t *t)
{
	memset(t, 0, sizeof *t);
	t->k = k; t->emax = emax;
	vec_t v = { 0 }; v.es = sizeof(short) * k;
	short cur[3];
	/* nested enumeration of increasing tuples */
	if (k == 1) {
		for (int a = 0; a < nsp; a++) if (sp[a].e <= emax) { cur[0] = a; vpush(&v, cur); }
	} else if (k == 2) {
		for (int a = 0; a < nsp; a++) for (int b = a + 1; b < nsp; b++)
			if (sp[a].e + sp[b].e <= emax) { cur[0] = a; cur[1] = b; vpush(&v, cur); }
	} else {
		for (int a = 0; a < nsp; a++) for (int b = a + 1; b < nsp; b++) {
			if (sp[a].e + sp[b].e > emax) continue;
			for (int c = b + 1; c < nsp; c++)
				if (sp[a].e + sp[b].e + sp[c].e <= emax) {
					cur[0] = a; cur[1] = b; cur[2] = c; vpush(&v, cur);
				}
		}
	}
	g_sp_for_sort = sp; g_k_for_sort = k;
	qsort(v.a, v.n, v.es, cmp_kstate);
	t->n = (int)v.n;
	t->orb = v.a ? v.a : xcalloc(1, sizeof(short));
	t->E = xcalloc(t->n, sizeof(int));
	t->M = xcalloc(t->n, sizeof(int));
	t->rank = xcalloc(t->n, sizeof(int));
	int mmax = 0;
	for (int i = 0; i < t->n; i++) {
		int E = 0, M = 0;
		for (int q = 0; q < k; q++) { E += sp[t->orb[i * k + q]].e; M += sp[t->orb[i * k + q]].m; }
		t->E[i] = E; t->M[i] = M;
		if (abs(M) > mmax) mmax = abs(M);
	}
	t->mmin = -mmax; t->mmax = mmax;
	t->ebeg = xcalloc(emax + 2, sizeof(int));
	for (int E = 0, i = 0; E <= emax + 1; E++) {
		while (i < t->n && t->E[i] < E) i++;
		t->ebeg[E] = i;
	}
	t->mstride = (t->mmax - t->mmin) / 2 + 2;
	t->mseg = xcalloc((size_t)(emax + 1) * t->mstride, sizeof(int));
	for (int E = 0; E <= emax; E++) {
		int i = t->ebeg[E];
		for (int mi = 0; mi < t->mstride; mi++) {
			int M = t->mmin + 2 * mi;
			while (i < t->ebeg[E + 1] && t->M[i] < M) i++;
			t->mseg[(size_t)E * t->mstride + mi] = i;
		}
	}
	for (int i = 0; i < t->n; i++) {
		int beg, end;
		(void)end;
		int E = t->E[i], M = t->M[i];
		beg = t->mseg[(size_t)E * t->mstride + (M - t->mmin) / 2];
		t->rank[i] = i - beg;
	}
	return 0;
}

/* states of energy E and doubled M: [*beg, *end) */
static void kst_range(const kst_t *t, int E, int M, int *beg, int *end)
{
	*beg = *end = 0;
	if (E < 0 || E > t->emax) return;
	if (M < t->mmin || M > t->mmax || ((M - t->mmin) & 1)) return;
	int mi = (M - t->mmin) / 2;
	*beg = t->mseg[(size_t)E * t->mstride + mi];
	*end = (mi + 1 < t->mstride) ? t->mseg[(size_t)E * t->mstride + mi + 1] : t->ebeg[E + 1];
	if (*end > t->ebeg[E + 1]) *end = t->ebeg[E + 1];
}

/* index of a k-state given sorted orbitals (binary search inside its (E,M) segment) */
static int kst_find(const kst_t *t, const sp_t *sp, const short *o)
{
	int E = 0, M = 0, k = t->k;
	for (int q = 0; q < k; q++) { E += sp[o[q]].e; M += sp[o[q]].m; }
	int lo, hi;
	kst_range(t, E, M, &lo, &hi);
	while (lo < hi) {
		int mid = (lo + hi) / 2, c = 0;
		for (int q = 0; q < k && !c; q++) c = t->orb[mid * k + q] - o[q];
		if (c == 0) return mid;
		if (c < 0) lo = mid + 1; else hi = mid;
	}
	return -1;
}

/* ------------------------------------------------------------------ */
/* Slater determinants of one species, grouped in (E, M) sub-bases     */
/* ------------------------------------------------------------------ */
typedef struct {
	int E, M;
	int beg, n;             /* into sd arrays */
} subbasis_t;

typedef struct {
	int np;                 /* particles */
	int nsd;
	mask_t *mask;
	short *occ;             /* nsd*np sorted orbitals */
	int *E, *M;
	int nsub;
	subbasis_t *sub;
	/* hash: mask -> sd index */
	size_t hcap;
	int *htab;
} species_t;

static uint64_t mask_hash(const mask_t *m)
{
	uint64_t h = 0x12345678abcdefull;
	for (int i = 0; i < MAXW; i++) h = mix64(h ^ m->w[i]);
	return h;
}

static int mask_eq(const mask_t *a, const mask_t *b) { return memcmp(a, b, sizeof *a) == 0; }

static int sd_lookup(const species_t *s, const mask_t *m)
{
	size_t i = mask_hash(m) & (s->hcap - 1);
	while (s->htab[i] >= 0) {
		if (mask_eq(&s->mask[s->htab[i]], m)) return s->htab[i];
		i = (i + 1) & (s->hcap - 1);
	}
	return -1;
}

static const sp_t *g_sd_sp; static int g_sd_np;
static int cmp_sd(const void *a, const void *b)
{
	const short *x = a, *y = b;
	int ex = 0, ey = 0, mx = 0, my = 0;
	for (int i = 0; i < g_sd_np; i++) {
		ex += g_sd_sp[x[i]].e; mx += g_sd_sp[x[i]].m;
		ey += g_sd_sp[y[i]].e; my += g_sd_sp[y[i]].m;
	}
	if (ex != ey) return ex - ey;
	if (mx != my) return mx - my;
	for (int i = 0; i < g_sd_np; i++) if (x[i] != y[i]) return x[i] - y[i];
	return 0;
}

static void species_free(species_t *s)
{
	free(s->mask); free(s->occ); free(s->E); free(s->M); free(s->sub); free(s->htab);
	memset(s, 0, sizeof *s);
}

static int build_species(const sp_t *sp, int nsp, int np, int emax_total, species_t *s)
{
	memset(s, 0, sizeof *s);
	s->np = np;
	vec_t v = { 0 }; v.es = sizeof(short) * (np > 0 ? np : 1);
	if (np == 0) {
		short dummy = 0; vpush(&v, &dummy);
	} else {
		short cur[64];
		int idx[64];
		/* iterative enumeration of increasing np-tuples with energy cap */
		int d = 0; idx[0] = -1;
		int Eacc[65]; Eacc[0] = 0;
		while (d >= 0) {
			idx[d]++;
			if (idx[d] >= nsp) { d--; continue; }
			int E = Eacc[d] + sp[idx[d]].e;
			if (E > emax_total) {
				/* orbitals are sorted by e: no later orbital fits either */
				d--; continue;
			}
			if (d == np - 1) {
				for (int q = 0; q < np; q++) cur[q] = (short)idx[q];
				vpush(&v, cur);
			} else {
				Eacc[d + 1] = E;
				idx[d + 1] = idx[d];
				d++;
			}
		}
	}
	g_sd_sp = sp; g_sd_np = np;
	if (np > 0) qsort(v.a, v.n, v.es, cmp_sd);
	s->nsd = (int)v.n;
	s->occ = v.a;
	s->mask = xcalloc(s->nsd, sizeof(mask_t));
	s->E = xcalloc(s->nsd, sizeof(int));
	s->M = xcalloc(s->nsd, sizeof(int));
	for (int i = 0; i < s->nsd; i++) {
		int E = 0, M = 0;
		for (int q = 0; q < np; q++) {
			int o = s->occ[(size_t)i * np + q];
			s->mask[i].w[o >> 6] |= 1ull << (o & 63);
			E += sp[o].e; M += sp[o].m;
		}
		s->E[i] = E; s->M[i] = M;
	}
	vec_t sv = { 0 }; sv.es = sizeof(subbasis_t);
	for (int i = 0; i < s->nsd;) {
		subbasis_t b = { s->E[i], s->M[i], i, 0 };
		while (i < s->nsd && s->E[i] == b.E && s->M[i] == b.M) { i++; b.n++; }
		vpush(&sv, &b);
	}
	s->nsub = (int)sv.n; s->sub = sv.a;
	s->hcap = 1;
	while (s->hcap < 2 * (size_t)s->nsd + 2) s->hcap <<= 1;
	s->htab = malloc(s->hcap * sizeof(int));
	for (size_t i = 0; i < s->hcap; i++) s->htab[i] = -1;
	for (int i = 0; i < s->nsd; i++) {
		size_t h = mask_hash(&s->mask[i]) & (s->hcap - 1);
		while (s->htab[h] >= 0) h = (h + 1) & (s->hcap - 1);
		s->htab[h] = i;
	}
	return 0;
}

static int find_sub(const species_t *s, int E, int M)
{
	for (int i = 0; i < s->nsub; i++)
		if (s->sub[i].E == E && s->sub[i].M == M) return i;
	return -1;
}

/* ------------------------------------------------------------------ */
/* fermionic sign of O(beta,alpha)|sd>                                 */
/* ------------------------------------------------------------------ */
static int popc_below(const mask_t *m, int o)
{
	int c = 0;
	for (int w = 0; w < (o >> 6); w++) c += __builtin_popcountll(m->w[w]);
	if (o & 63) c += __builtin_popcountll(m->w[o >> 6] & ((1ull << (o & 63)) - 1));
	return c;
}

static int apply_op(const mask_t *in, const short *alpha, const short *beta, int k, mask_t *out)
{
	mask_t m = *in;
	int sign = 1;
	for (int q = 0; q < k; q++) {           /* a_{a1} first, then a_{a2} ... */
		int o = alpha[q];
		if (!((m.w[o >> 6] >> (o & 63)) & 1)) return 0;
		if (popc_below(&m, o) & 1) sign = -sign;
		m.w[o >> 6] &= ~(1ull << (o & 63));
	}
	for (int q = k - 1; q >= 0; q--) {      /* a+_{bk} first, ..., a+_{b1} last */
		int o = beta[q];
		if ((m.w[o >> 6] >> (o & 63)) & 1) return 0;
		if (popc_below(&m, o) & 1) sign = -sign;
		m.w[o >> 6] |= 1ull << (o & 63);
	}
	*out = m;
	return sign;
}

/* ------------------------------------------------------------------ */
/* problem tables                                                      */
/* ------------------------------------------------------------------ */
typedef struct { int Ep, Mp, En, Mn, ip, in; size_t np_, nn_; } bblock_t;

typedef struct {
	int species;            /* 0 proton, 1 neutron */
	int k;
	int Ein, Min, Eout, Mout, depth;
	size_t len;
	uint32_t *data;         /* len*3: in, out, matrix_index (file order) */
	int id;
} ilist_t;

typedef struct {
	int kp, kn;             /* particles of each species acted on */
	int dEp, dMp, dp, dEn, dMn, dn;
	size_t np_conn, nn_conn;
	int id;
} meblk_t;

typedef struct {
	int nparticles;
	int bin, bout;          /* basis block indices (0-based) */
	int lp, ln;             /* list indices or -1 */
	int me;                 /* ME block index */
	uint64_t mults;
} calc_t;

typedef struct {
	jn_gen_config cfg;
	int nsp;
	sp_t *sp;
	kst_t kst[4];
	species_t spc[2];
	int nb;
	bblock_t *bb;
	vec_t lists;            /* ilist_t */
	vec_t mes;              /* meblk_t */
	vec_t calcs;            /* calc_t */
	/* list lookup */
	size_t lcap; int *ltab;
	size_t mcap; int *mtab;
} gen_t;

static uint64_t lkey_hash(int sp_, int k, int Ein, int Min, int Eout, int Mout, int d)
{
	uint64_t h = mix64((uint64_t)sp_ * 7 + (uint64_t)k);
	h = mix64(h ^ (uint64_t)(uint32_t)Ein); h = mix64(h ^ (uint64_t)(uint32_t)Min);
	h = mix64(h ^ (uint64_t)(uint32_t)Eout); h = mix64(h ^ (uint64_t)(uint32_t)Mout);
	return mix64(h ^ (uint64_t)(uint32_t)d);
}

static int ltab_find(gen_t *g, int sp_, int k, int Ein, int Min, int Eout, int Mout, int d, int insert_idx)
{
	if (g->lcap == 0) {
		g->lcap = 1 << 16;
		g->ltab = malloc(g->lcap * sizeof(int));
		for (size_t i = 0; i < g->lcap; i++) g->ltab[i] = -1;
	}
	size_t i = lkey_hash(sp_, k, Ein, Min, Eout, Mout, d) & (g->lcap - 1);
	ilist_t *L = g->lists.a;
	while (g->ltab[i] >= 0) {
		ilist_t *c = &L[g->ltab[i]];
		if (c->species == sp_ && c->k == k && c->Ein == Ein && c->Min == Min && c->Eout == Eout &&
		    c->Mout == Mout && c->depth == d)
			return g->ltab[i];
		i = (i + 1) & (g->lcap - 1);
	}
	if (insert_idx >= 0) g->ltab[i] = insert_idx;
	return -1;
}

static void ltab_grow(gen_t *g)
{
	if (g->lists.n * 2 < g->lcap) return;
	free(g->ltab);
	g->lcap *= 2;
	g->ltab = malloc(g->lcap * sizeof(int));
	for (size_t i = 0; i < g->lcap; i++) g->ltab[i] = -1;
	ilist_t *L = g->lists.a;
	for (size_t q = 0; q < g->lists.n; q++) {
		size_t i = lkey_hash(L[q].species, L[q].k, L[q].Ein, L[q].Min, L[q].Eout, L[q].Mout, L[q].depth) & (g->lcap - 1);
		while (g->ltab[i] >= 0) i = (i + 1) & (g->lcap - 1);
		g->ltab[i] = (int)q;
	}
}

/* connection offsets for (k, depth, dE, dM): offset of alpha (global k-state index) */
static int conn_index(const kst_t *t, int alpha, int beta, int dE, int dM,
		      int *cache_valid, int *cache_key, int *offs)
{
	/* offsets recomputed when the (depth,dE,dM) key changes; alpha in energy depth */
	int depth = t->E[alpha];
	int key[3] = { depth, dE, dM };
	if (!*cache_valid || memcmp(cache_key, key, sizeof key) != 0) {
		int acc = 0;
		for (int a = t->ebeg[depth]; a < t->ebeg[depth + 1]; a++) {
			offs[a - t->ebeg[depth]] = acc;
			int b0, b1;
			kst_range(t, depth + dE, t->M[a] + dM, &b0, &b1);
			acc += b1 - b0;
		}
		offs[t->ebeg[depth + 1] - t->ebeg[depth]] = acc;
		memcpy(cache_key, key, sizeof key);
		*cache_valid = 1;
	}
	return offs[alpha - t->ebeg[depth]] + t->rank[beta];
}

static size_t conn_count(const kst_t *t, int depth, int dE, int dM)
{
	if (depth < 0 || depth > t->emax) return 0;
	size_t acc = 0;
	for (int a = t->ebeg[depth]; a < t->ebeg[depth + 1]; a++) {
		int b0, b1;
		kst_range(t, depth + dE, t->M[a] + dM, &b0, &b1);
		acc += (size_t)(b1 - b0);
	}
	return acc;
}

/* build one index list; returns list index or -1 when empty */
static int get_list(gen_t *g, int species, int k, int isub_in, int isub_out, int depth)
{
	species_t *s = &g->spc[species];
	subbasis_t *si = &s->sub[isub_in], *so = &s->sub[isub_out];
	int found = ltab_find(g, species, k, si->E, si->M, so->E, so->M, depth, -1);
	if (found >= 0) return ((ilist_t *)g->lists.a)[found].len ? found : -1;
	kst_t *t = &g->kst[k];
	int dE = so->E - si->E, dM = so->M - si->M;
	ilist_t L = { species, k, si->E, si->M, so->E, so->M, depth, 0, NULL, 0 };
	vec_t d = { 0 }; d.es = 3 * sizeof(uint32_t);
	int np = s->np;
	int cache_valid = 0, cache_key[3];
	int *offs = NULL;
	if (depth >= 0 && depth <= t->emax && k <= np && depth + dE >= 0 && depth + dE <= t->emax) {
		offs = xcalloc(t->ebeg[depth + 1] - t->ebeg[depth] + 1, sizeof(int));
		for (int i = 0; i < si->n; i++) {
			int sd = si->beg + i;
			const short *occ = s->occ + (size_t)sd * np;
			int sel[3], nsel = 0;
			/* k-subsets of occ in lexicographic order */
			for (sel[0] = 0; sel[0] < np; sel[0]++) {
				int lim1 = k > 1 ? np : sel[0] + 2;
				for (sel[1] = k > 1 ? sel[0] + 1 : sel[0] + 1; sel[1] < lim1; sel[1]++) {
					int lim2 = k > 2 ? np : sel[1] + 2;
					for (sel[2] = k > 2 ? sel[1] + 1 : sel[1] + 1; sel[2] < lim2; sel[2]++) {
						nsel++;
						short al[3];
						int Ea = 0, Ma = 0;
						for (int q = 0; q < k; q++) { al[q] = occ[sel[q]]; Ea += g->sp[al[q]].e; Ma += g->sp[al[q]].m; }
						if (Ea != depth) continue;
						int ia = kst_find(t, g->sp, al);
						if (ia < 0) continue;
						int b0, b1;
						kst_range(t, depth + dE, Ma + dM, &b0, &b1);
						for (int ib = b0; ib < b1; ib++) {
							mask_t out;
							int sg = apply_op(&s->mask[sd], al, t->orb + (size_t)ib * k, k, &out);
							if (!sg) continue;
							int j = sd_lookup(s, &out);
							if (j < 0) continue;
							if (j < so->beg || j >= so->beg + so->n) continue;
							uint32_t rec[3];
							uint32_t ci = (uint32_t)conn_index(t, ia, ib, dE, dM, &cache_valid, cache_key, offs);
							rec[0] = (uint32_t)i;
							rec[1] = (uint32_t)(j - so->beg);
							rec[2] = ci | (sg < 0 ? SIGN_BIT : 0u);
							vpush(&d, rec);
						}
					}
				}
			}
			(void)nsel;
		}
		free(offs);
	}
	L.len = d.n; L.data = d.a;
	int idx = (int)g->lists.n;
	vpush(&g->lists, &L);
	ltab_grow(g);
	if (ltab_find(g, species, k, si->E, si->M, so->E, so->M, depth, idx) >= 0) { /* already present */ }
	return L.len ? idx : -1;
}

static int get_me(gen_t *g, int kp, int kn, int dEp, int dMp, int dp, int dEn, int dMn, int dn)
{
	meblk_t *M = g->mes.a;
	for (size_t i = 0; i < g->mes.n; i++)
		if (M[i].kp == kp && M[i].kn == kn && M[i].dEp == dEp && M[i].dMp == dMp && M[i].dp == dp &&
		    M[i].dEn == dEn && M[i].dMn == dMn && M[i].dn == dn)
			return (int)i;
	meblk_t b = { kp, kn, dEp, dMp, dp, dEn, dMn, dn, 0, 0, 0 };
	b.np_conn = kp ? conn_count(&g->kst[kp], dp, dEp, dMp) : 0;
	b.nn_conn = kn ? conn_count(&g->kst[kn], dn, dEn, dMn) : 0;
	vpush(&g->mes, &b);
	return (int)g->mes.n - 1;
}

/* O(1) lookup of ME blocks through a small hash (many calc blocks share one) */
static int get_me_fast(gen_t *g, int kp, int kn, int dEp, int dMp, int dp, int dEn, int dMn, int dn)
{
	if (g->mcap == 0) {
		g->mcap = 1 << 14;
		g->mtab = malloc(g->mcap * sizeof(int));
		for (size_t i = 0; i < g->mcap; i++) g->mtab[i] = -1;
	}
	uint64_t h = mix64((uint64_t)(kp * 4 + kn));
	int v[6] = { dEp, dMp, dp, dEn, dMn, dn };
	for (int q = 0; q < 6; q++) h = mix64(h ^ (uint64_t)(uint32_t)v[q]);
	size_t i = h & (g->mcap - 1);
	meblk_t *M = g->mes.a;
	while (g->mtab[i] >= 0) {
		meblk_t *c = &M[g->mtab[i]];
		if (c->kp == kp && c->kn == kn && c->dEp == dEp && c->dMp == dMp && c->dp == dp &&
		    c->dEn == dEn && c->dMn == dMn && c->dn == dn)
			return g->mtab[i];
		i = (i + 1) & (g->mcap - 1);
	}
	if (g->mes.n * 2 >= g->mcap) {
		/* rebuild larger */
		free(g->mtab);
		g->mcap *= 2;
		g->mtab = malloc(g->mcap * sizeof(int));
		for (size_t q = 0; q < g->mcap; q++) g->mtab[q] = -1;
		M = g->mes.a;
		for (size_t q = 0; q < g->mes.n; q++) {
			uint64_t hh = mix64((uint64_t)(M[q].kp * 4 + M[q].kn));
			int vv[6] = { M[q].dEp, M[q].dMp, M[q].dp, M[q].dEn, M[q].dMn, M[q].dn };
			for (int r = 0; r < 6; r++) hh = mix64(hh ^ (uint64_t)(uint32_t)vv[r]);
			size_t j = hh & (g->mcap - 1);
			while (g->mtab[j] >= 0) j = (j + 1) & (g->mcap - 1);
			g->mtab[j] = (int)q;
		}
		i = h & (g->mcap - 1);
		while (g->mtab[i] >= 0) i = (i + 1) & (g->mcap - 1);
	}
	meblk_t b = { kp, kn, dEp, dMp, dp, dEn, dMn, dn, 0, 0, 0 };
	b.np_conn = kp ? conn_count(&g->kst[kp], dp, dEp, dMp) : 0;
	b.nn_conn = kn ? conn_count(&g->kst[kn], dn, dEn, dMn) : 0;
	vpush(&g->mes, &b);
	g->mtab[i] = (int)g->mes.n - 1;
	return (int)g->mes.n - 1;
}

/* ------------------------------------------------------------------ */
/* ground-state energies and shell capacities                          */
/* ------------------------------------------------------------------ */
static int min_energy(int np)
{
	int E = 0, e = 0, left = np;
	while (left > 0) { int c = (e + 1) * (e + 2); int t = left < c ? left : c; E += t * e; left -= t; e++; }
	return E;
}
static int top_shell(int np)
{
	int e = 0, left = np;
	if (np == 0) return 0;
	for (;;) { int c = (e + 1) * (e + 2); if (left <= c) return e; left -= c; e++; }
}

/* ------------------------------------------------------------------ */
/* enumerate calc blocks                                               */
/* ------------------------------------------------------------------ */
static void add_calc(gen_t *g, int bin, int bout, int kp, int kn, int dp, int dn)
{
	bblock_t *A = &g->bb[bin], *B = &g->bb[bout];
	int lp = -1, ln = -1;
	if (kp) { lp = get_list(g, 0, kp, A->ip, B->ip, dp); if (lp < 0) return; }
	if (kn) { ln = get_list(g, 1, kn, A->in, B->in, dn); if (ln < 0) return; }
	int me = get_me_fast(g, kp, kn, kp ? B->Ep - A->Ep : 0, kp ? B->Mp - A->Mp : 0, kp ? dp : 0,
			     kn ? B->En - A->En : 0, kn ? B->Mn - A->Mn : 0, kn ? dn : 0);
	meblk_t *mb = &((meblk_t *)g->mes.a)[me];
	if ((kp && !mb->np_conn) || (kn && !mb->nn_conn)) return;
	calc_t c = { kp + kn, bin, bout, lp, ln, me, 0 };
	ilist_t *L = g->lists.a;
	if (kp && kn) c.mults = (uint64_t)L[lp].len * L[ln].len;
	else if (kp) c.mults = (uint64_t)L[lp].len * A->nn_;
	else c.mults = (uint64_t)L[ln].len * A->np_;
	vpush(&g->calcs, &c);
}

static void enumerate_calcs(gen_t *g)
{
	int threebody = g->cfg.nbody >= 3;
	int Z = g->cfg.Z, N = g->cfg.N;
	for (int a = 0; a < g->nb; a++)
		for (int b = a; b < g->nb; b++) {
			bblock_t *A = &g->bb[a], *B = &g->bb[b];
			int sameP = (A->Ep == B->Ep && A->Mp == B->Mp);
			int sameN = (A->En == B->En && A->Mn == B->Mn);
			/* two-body: pp, nn, np */
			if (sameN && Z >= 2)
				for (int dp = 0; dp <= g->kst[2].emax; dp++) add_calc(g, a, b, 2, 0, dp, 0);
			if (sameP && N >= 2)
				for (int dn = 0; dn <= g->kst[2].emax; dn++) add_calc(g, a, b, 0, 2, 0, dn);
			if (Z >= 1 && N >= 1)
				for (int dp = 0; dp <= g->kst[1].emax; dp++)
					for (int dn = 0; dn <= g->kst[1].emax; dn++) add_calc(g, a, b, 1, 1, dp, dn);
			if (!threebody) continue;
			if (sameN && Z >= 3)
				for (int dp = 0; dp <= g->kst[3].emax; dp++) add_calc(g, a, b, 3, 0, dp, 0);
			if (sameP && N >= 3)
				for (int dn = 0; dn <= g->kst[3].emax; dn++) add_calc(g, a, b, 0, 3, 0, dn);
			if (Z >= 2 && N >= 1)
				for (int dp = 0; dp <= g->kst[2].emax; dp++)
					for (int dn = 0; dn <= g->kst[1].emax; dn++) add_calc(g, a, b, 2, 1, dp, dn);
			if (Z >= 1 && N >= 2)
				for (int dp = 0; dp <= g->kst[1].emax; dp++)
					for (int dn = 0; dn <= g->kst[2].emax; dn++) add_calc(g, a, b, 1, 2, dp, dn);
		}
}

/* ------------------------------------------------------------------ */
/* matrix-element values                                               */
/* ------------------------------------------------------------------ */
static uint64_t state_code(const short *o, int k, int nsp)
{
	uint64_t c = 0;
	for (int q = 0; q < k; q++) c = c * (uint64_t)(nsp + 1) + (uint64_t)(o[q] + 1);
	return c;
}

/* value of <beta|V|alpha> for a (kp protons, kn neutrons) term */
static double me_value(const gen_t *g, int kp, int kn, const short *ap, const short *bp,
		       const short *an, const short *bn, uint64_t seed, double sigma, int with_ho)
{
	uint64_t span = 1;
	for (int q = 0; q < kn; q++) span *= (uint64_t)(g->nsp + 1);
	uint64_t ka = state_code(ap, kp, g->nsp) * span + state_code(an, kn, g->nsp);
	uint64_t kb = state_code(bp, kp, g->nsp) * span + state_code(bn, kn, g->nsp);
	uint64_t tag = (uint64_t)(kp * 4 + kn);
	double v = sigma * jn_gen_pair_normal(seed, tag, ka, kb);
	if (with_ho && kp + kn == 2 && ka == kb) {
		int A = g->cfg.Z + g->cfg.N;
		double esum = 0;
		for (int q = 0; q < kp; q++) esum += g->sp[ap[q]].e;
		for (int q = 0; q < kn; q++) esum += g->sp[an[q]].e;
		v += g->cfg.hbar_omega * esum / (double)(A - 1);
	}
	return v;
}

/* enumerate connections of (k, depth, dE, dM) in Mercury order into (alpha,beta) pairs */
static size_t list_conns(const kst_t *t, int depth, int dE, int dM, int **pairs)
{
	size_t n = conn_count(t, depth, dE, dM), i = 0;
	int *p = xcalloc(2 * n, sizeof(int));
	if (n)
		for (int a = t->ebeg[depth]; a < t->ebeg[depth + 1]; a++) {
			int b0, b1;
			kst_range(t, depth + dE, t->M[a] + dM, &b0, &b1);
			for (int b = b0; b < b1; b++) { p[2 * i] = a; p[2 * i + 1] = b; i++; }
		}
	*pairs = p;
	return n;
}

/* quiet: leave the error text alone (the block writers on several threads) */
static int write_me_block(const gen_t *g, const meblk_t *b, const char *dir, uint64_t seed,
			  double sigma, int with_ho, int quiet)
{
	char path[4096];
	snprintf(path, sizeof path, "%s/%d_matrix_elements", dir, b->id);
	FILE *f = fopen(path, "wb");
	if (!f) {
		if (quiet) return JN_GEN_EIO;
		FAIL(JN_GEN_EIO, "cannot open %s: %s", path, strerror(errno));
	}
	size_t nd_n = b->kn ? b->nn_conn : 0, nd_p = b->kp ? b->np_conn : 0;
	fwrite(&nd_n, sizeof(size_t), 1, f);
	fwrite(&nd_p, sizeof(size_t), 1, f);
	int *pp = NULL, *pn = NULL;
	size_t cp = b->kp ? list_conns(&g->kst[b->kp], b->dp, b->dEp, b->dMp, &pp) : 1;
	size_t cn = b->kn ? list_conns(&g->kst[b->kn], b->dn, b->dEn, b->dMn, &pn) : 1;
	size_t row = cn;
	double *buf = xcalloc(row, sizeof(double));
	static const short none[3] = { 0, 0, 0 };
	for (size_t ip = 0; ip < cp; ip++) {
		const short *ap = none, *bp = none;
		if (b->kp) {
			ap = g->kst[b->kp].orb + (size_t)pp[2 * ip] * b->kp;
			bp = g->kst[b->kp].orb + (size_t)pp[2 * ip + 1] * b->kp;
		}
		for (size_t in = 0; in < cn; in++) {
			const short *an = none, *bn = none;
			if (b->kn) {
				an = g->kst[b->kn].orb + (size_t)pn[2 * in] * b->kn;
				bn = g->kst[b->kn].orb + (size_t)pn[2 * in + 1] * b->kn;
			}
			buf[in] = me_value(g, b->kp, b->kn, ap, bp, an, bn, seed, sigma, with_ho);
		}
		if (fwrite(buf, sizeof(double), row, f) != row) {
			fclose(f);
			free(buf); free(pp); free(pn);
			if (quiet) return JN_GEN_EIO;
			FAIL(JN_GEN_EIO, "short write %s", path);
		}
	}
	free(buf); free(pp); free(pn);
	if (fclose(f) != 0) {
		if (quiet) return JN_GEN_EIO;
		FAIL(JN_GEN_EIO, "close %s", path);
	}
	return 0;
}

/* The matrix-element blocks, written by all host cores (at most 32 threads,
 * fewer when JN_HOST_THREADS caps them).  Every element is a counter-based
 * deviate of its own indices and every block is its own file, so the files
 * do not depend on the thread count.  A failing block is written once more
 * on its own for the error text. */
typedef struct {
	const gen_t *g;
	const char *dir;
	const size_t *blk;      /* the blocks to write, in order */
	size_t n, next;
	int *rc;
} mejob_t;

static uint64_t me_seed(const gen_t *g, const meblk_t *b)
{
	return g->cfg.seed * 1000003ull + (uint64_t)(b->kp + b->kn);
}

static double me_sigma(const gen_t *g, const meblk_t *b)
{
	return (b->kp + b->kn == 3) ? g->cfg.sigma3 : g->cfg.sigma2;
}

static void *me_worker(void *v)
{
	mejob_t *j = (mejob_t *)v;
	const meblk_t *M = j->g->mes.a;
	for (;;) {
		const size_t i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
		if (i >= j->n) break;
		const meblk_t *b = &M[j->blk[i]];
		j->rc[i] = write_me_block(j->g, b, j->dir, me_seed(j->g, b), me_sigma(j->g, b), j->g->cfg.hbar_omega != 0.0, 1);
	}
	return NULL;
}

static int write_me_blocks(const gen_t *g, const char *dir)
{
	const meblk_t *M = g->mes.a;
	size_t n = 0;
	size_t *blk = xcalloc(g->mes.n, sizeof(size_t));
	int *rc = xcalloc(g->mes.n, sizeof(int));
	if (!blk || !rc) { free(blk); free(rc); FAIL(JN_GEN_ENOMEM, "out of memory"); }
	for (size_t i = 0; i < g->mes.n; i++) {
		if (!M[i].id) continue;
		if (g->cfg.antoine && M[i].kp + M[i].kn == 2) continue;   /* left to the J->M transform */
		blk[n++] = i;
	}
	long nt = sysconf(_SC_NPROCESSORS_ONLN);
	const char *cap = getenv("JN_HOST_THREADS");
	if (cap && atol(cap) > 0 && atol(cap) < nt) nt = atol(cap);
	if (nt > 32) nt = 32;
	if (nt < 1) nt = 1;
	mejob_t j = { g, dir, blk, n, 0, rc };
	pthread_t th[32];
	int started = 0;
	for (long t = 1; t < nt; t++)
		if (pthread_create(&th[started], NULL, me_worker, &j) == 0) started++;
	me_worker(&j);
	for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
	int out = 0;
	for (size_t i = 0; i < n && !out; i++)
		if (rc[i]) {
			const meblk_t *b = &M[blk[i]];
			out = write_me_block(g, b, dir, me_seed(g, b), me_sigma(g, b), g->cfg.hbar_omega != 0.0, 0);
			if (!out) {
				out = rc[i];
				snprintf(g_err, sizeof g_err, "writing matrix-element block %d failed", b->id);
			}
		}
	free(blk); free(rc);
	return out;
}

/* ------------------------------------------------------------------ */
/* output                                                              */
/* ------------------------------------------------------------------ */
static int mkdir_p(const char *p)
{
	char tmp[4096];
	snprintf(tmp, sizeof tmp, "%s", p);
	for (char *c = tmp + 1; *c; c++)
		if (*c == '/') { *c = 0; mkdir(tmp, 0755); *c = '/'; }
	if (mkdir(tmp, 0755) != 0 && errno != EEXIST) return -1;
	return 0;
}

static const char *ptype(int species, int k)
{
	static const char *n[2][4] = { { "", "p", "pp", "ppp" }, { "", "n", "nn", "nnn" } };
	return n[species][k];
}

static int write_basis_files(const gen_t *g, const char *dir)
{
	char path[4096];
	for (int species = 0; species < 2; species++)
		for (int k = 1; k <= 3; k++) {
			const kst_t *t = &g->kst[k];
			if (!t->n) continue;
			snprintf(path, sizeof path, "%s/anicr/%s_inds_index_lists", dir, ptype(species, k));
			if (mkdir_p(path)) FAIL(JN_GEN_EIO, "mkdir %s", path);
			for (int E = 0; E <= t->emax; E++) {
				snprintf(path, sizeof path, "%s/anicr/%s_inds_index_lists/basis_energy_%d", dir,
					 ptype(species, k), E);
				FILE *f = fopen(path, "wb");
				if (!f) FAIL(JN_GEN_EIO, "open %s", path);
				size_t n = (size_t)(t->ebeg[E + 1] - t->ebeg[E]) * k;
				if (n && fwrite(t->orb + (size_t)t->ebeg[E] * k, sizeof(short), n, f) != n) {
					fclose(f); FAIL(JN_GEN_EIO, "write %s", path);
				}
				fclose(f);
			}
		}
	return 0;
}

static int write_comb(const gen_t *g, const char *path, int *order_of_calcs)
{
	FILE *f = fopen(path, "w");
	if (!f) FAIL(JN_GEN_EIO, "open %s: %s", path, strerror(errno));
	const jn_gen_config *c = &g->cfg;
	fprintf(f, "# combination table written by jn_gen: Z=%d N=%d Nmax=%d 2M=%d parity=%d nbody=%d seed=%llu\n",
		c->Z, c->N, c->Nmax, c->M2, c->parity, c->nbody, (unsigned long long)c->seed);
	fprintf(f, "*** mp-states ***\n");
	fprintf(f, "#   Ep   Mp   En   Mn       Np       Nn        dim   (array id, bytes)\n");
	for (int b = 0; b < g->nb; b++) {
		const bblock_t *B = &g->bb[b];
		fprintf(f, "%6d %4d %4d %4d %8zu %8zu %10zu # ARRAYMP: %d= %zu\n", B->Ep, B->Mp, B->En, B->Mn,
			B->np_, B->nn_, B->np_ * B->nn_, b + 1, B->np_ * B->nn_ * sizeof(double));
	}
	fprintf(f, "*** Conn lists ***\n");
	fprintf(f, "# type E_in M_in E_out M_out depth length   (array id, bytes)\n");
	const ilist_t *L = g->lists.a;
	for (size_t i = 0; i < g->lists.n; i++) {
		if (!L[i].len) continue;
		fprintf(f, "%-4s %4d %4d %4d %4d %4d %10zu # ARRAY: %d= %zu\n", ptype(L[i].species, L[i].k), L[i].Ein,
			L[i].Min, L[i].Eout, L[i].Mout, L[i].depth, L[i].len, L[i].id, L[i].len * 12);
	}
	fprintf(f, "*** Matrix-elements V (cross p-n) ***\n");
	fprintf(f, "# p-type dEp dMp depth_p n-type dEn dMn depth_n n_p_comb n_n_comb length   (array id, bytes)\n");
	const meblk_t *M = g->mes.a;
	for (size_t i = 0; i < g->mes.n; i++) {
		if (!M[i].id || !M[i].kp || !M[i].kn) continue;
		fprintf(f, "%-4s %4d %4d %4d %-4s %4d %4d %4d %10zu %10zu %12zu # ARRAY: %d= %zu\n", ptype(0, M[i].kp),
			M[i].dEp, M[i].dMp, M[i].dp, ptype(1, M[i].kn), M[i].dEn, M[i].dMn, M[i].dn, M[i].np_conn,
			M[i].nn_conn, M[i].np_conn * M[i].nn_conn, M[i].id, M[i].np_conn * M[i].nn_conn * 8);
	}
	fprintf(f, "*** Matrix-elements V (same p/n) ***\n");
	fprintf(f, "# type dE dM depth n_comb length   (array id, bytes)\n");
	for (size_t i = 0; i < g->mes.n; i++) {
		if (!M[i].id || (M[i].kp && M[i].kn)) continue;
		int sp_ = M[i].kp ? 0 : 1, k = M[i].kp ? M[i].kp : M[i].kn;
		size_t n = M[i].kp ? M[i].np_conn : M[i].nn_conn;
		fprintf(f, "%-4s %4d %4d %4d %10zu %10zu # ARRAY: %d= %zu\n", ptype(sp_, k), M[i].kp ? M[i].dEp : M[i].dEn,
			M[i].kp ? M[i].dMp : M[i].dMn, M[i].kp ? M[i].dp : M[i].dn, n, n, M[i].id, n * 8);
	}
	fprintf(f, "*** Calc blocks ***\n");
	const calc_t *C = g->calcs.a;
	for (size_t q = 0; q < g->calcs.n; q++) {
		const calc_t *x = &C[order_of_calcs[q]];
		if (x->lp >= 0 && x->ln >= 0)
			fprintf(f, "MULT %llu # CALCBLOCK:%d: %d, %d, %d, %d, %d\n", (unsigned long long)x->mults, x->nparticles,
				x->bin + 1, x->bout + 1, L[x->ln].id, L[x->lp].id, M[x->me].id);
		else
			fprintf(f, "MULT %llu # CALCBLOCK:%d: %d, %d, %d, %d\n", (unsigned long long)x->mults, x->nparticles,
				x->bin + 1, x->bout + 1, x->lp >= 0 ? L[x->lp].id : L[x->ln].id, M[x->me].id);
	}
	fprintf(f, "*** End ***\n");
	if (fclose(f) != 0) FAIL(JN_GEN_EIO, "close %s", path);
	return 0;
}

static int write_eval_order(const gen_t *g, const char *path, int *order)
{
	FILE *f = fopen(path, "w");
	if (!f) FAIL(JN_GEN_EIO, "open %s: %s", path, strerror(errno));
	const calc_t *C = g->calcs.a;
	const ilist_t *L = g->lists.a;
	const meblk_t *M = g->mes.a;
	for (size_t q = 0; q < g->calcs.n; q++) {
		const calc_t *x = &C[order[q]];
		if (x->lp >= 0 && x->ln >= 0)
			fprintf(f, "BLOCK: %d %d %d %d %d\n", x->bin + 1, x->bout + 1, L[x->ln].id, L[x->lp].id, M[x->me].id);
		else
			fprintf(f, "BLOCK: %d %d %d %d\n", x->bin + 1, x->bout + 1, x->lp >= 0 ? L[x->lp].id : L[x->ln].id,
				M[x->me].id);
	}
	if (fclose(f) != 0) FAIL(JN_GEN_EIO, "close %s", path);
	return 0;
}

static int write_conf(const gen_t *g, const char *dir)
{
	char path[4096];
	snprintf(path, sizeof path, "%s/bacchus.conf", dir);
	FILE *f = fopen(path, "w");
	if (!f) FAIL(JN_GEN_EIO, "open %s", path);
	fprintf(f,
		"# Bacchus run file (libconfig syntax)\n"
		"interaction:\n{\n"
		"\tcombination_table_file = \"%s/comb.txt\";\n"
		"\tevaluation_order_file = \"%s/evaluation_order.txt\";\n"
		"\tindex_lists_base_directory = \"%s/index_lists\";\n"
		"\tmatrix_file_base_directory = \"%s/matrix_elements\";\n"
		"\tnum_neutrons = %d;\n"
		"\tnum_protons = %d;\n"
		"};\n"
		"lanczos:\n{\n"
		"\tkrylow_vector_directory = \"%s/krylow_vectors\";\n"
		"\tmax_num_lanczos_iterations = %d;\n"
		"\tconvergence_tolerance = 1e-6;\n"
		"\ttarget_eigenvector = 0;\n"
		"\teigenvector_directory = \"%s/eigen_vectors\";\n"
		"\tmax_memory_load = \"64GB\";\n"
		"};\n",
		dir, dir, dir, dir, g->cfg.N, g->cfg.Z, dir, g->cfg.lanczos_iterations > 0 ? g->cfg.lanczos_iterations : 200,
		dir);
	fclose(f);
	return 0;
}

static int write_lists(const gen_t *g, const char *dir)
{
	char path[4096];
	const ilist_t *L = g->lists.a;
	for (size_t i = 0; i < g->lists.n; i++) {
		if (!L[i].len) continue;
		snprintf(path, sizeof path, "%s/index_list_%d", dir, L[i].id);
		FILE *f = fopen(path, "wb");
		if (!f) FAIL(JN_GEN_EIO, "open %s: %s", path, strerror(errno));
		/* on-disk record is {in, out, matrix_index} */
		if (fwrite(L[i].data, 12, L[i].len, f) != L[i].len) { fclose(f); FAIL(JN_GEN_EIO, "write %s", path); }
		if (fclose(f) != 0) FAIL(JN_GEN_EIO, "close %s", path);
	}
	return 0;
}

/* the lists as Anicre writes them, the input of aurora.x
 * (src/Aurora/programs/aurora.c:64-96): raw {in, out, k} triples, or rows
 * "in out +k" / "in out -k" with the sign taken out of bit 31 */
static int write_anicre_lists(const gen_t *g, const char *outdir, int human_readable)
{
	char path[4096];
	const ilist_t *L = g->lists.a;
	for (size_t i = 0; i < g->lists.n; i++) {
		if (!L[i].len) continue;
		snprintf(path, sizeof path, "%s/anicr_lists/%s_inds_index_lists", outdir, ptype(L[i].species, L[i].k));
		if (mkdir_p(path)) FAIL(JN_GEN_EIO, "mkdir %s", path);
		snprintf(path, sizeof path, "%s/anicr_lists/%s_inds_index_lists/index_list_E_in%d_E_out%d_M_in%d_M_out%d_dE%d_dM%d_depth%d",
			 outdir, ptype(L[i].species, L[i].k), L[i].Ein, L[i].Eout, L[i].Min, L[i].Mout, L[i].Eout - L[i].Ein,
			 L[i].Mout - L[i].Min, L[i].depth);
		FILE *f = fopen(path, human_readable ? "w" : "wb");
		if (!f) FAIL(JN_GEN_EIO, "open %s: %s", path, strerror(errno));
		int bad = 0;
		if (!human_readable) {
			bad = fwrite(L[i].data, 12, L[i].len, f) != L[i].len;
		} else {
			for (size_t e = 0; e < L[i].len && !bad; e++) {
				const uint32_t k = L[i].data[3 * e + 2];
				bad = fprintf(f, "%d %d %c%u\n", (int)L[i].data[3 * e], (int)L[i].data[3 * e + 1],
					      (k & 0x80000000u) ? '-' : '+', k & 0x7fffffffu) < 0;
			}
		}
		if (fclose(f) != 0 || bad) FAIL(JN_GEN_EIO, "write %s", path);
	}
	return 0;
}

/* ------------------------------------------------------------------ */
/* public entry points                                                 */
/* ------------------------------------------------------------------ */
static void gen_free(gen_t *g)
{
	free(g->sp);
	for (int k = 0; k < 4; k++) kst_free(&g->kst[k]);
	species_free(&g->spc[0]); species_free(&g->spc[1]);
	free(g->bb);
	ilist_t *L = g->lists.a;
	for (size_t i = 0; i < g->lists.n; i++) free(L[i].data);
	free(g->lists.a); free(g->mes.a); free(g->calcs.a); free(g->ltab); free(g->mtab);
}

static const gen_t *g_sort_gen;
static int cmp_calc_order(const void *a, const void *b)
{
	/* evaluation order: by output block, then input block, then kind, then ids */
	const calc_t *C = g_sort_gen->calcs.a;
	const calc_t *x = &C[*(const int *)a], *y = &C[*(const int *)b];
	if (x->bout != y->bout) return x->bout - y->bout;
	if (x->bin != y->bin) return x->bin - y->bin;
	if (x->nparticles != y->nparticles) return x->nparticles - y->nparticles;
	if (x->me != y->me) return x->me - y->me;
	if (x->lp != y->lp) return x->lp - y->lp;
	return x->ln - y->ln;
}

static int fwrite_record(FILE *f, const void *data, int nbytes)
{
	return fwrite(&nbytes, 4, 1, f) != 1 || (nbytes && fwrite(data, (size_t)nbytes, 1, f) != 1) ||
	       fwrite(&nbytes, 4, 1, f) != 1;
}

int jn_gen_antoine(const char *path, int emax1, int emax2, int num_particles, double hbar_omega, uint64_t seed,
		   double sigma)
{
	if (num_particles < 2) FAIL(JN_GEN_EINVAL, "the Antoine kinetic column needs A >= 2 (A = %d)", num_particles);
	jn_jt_basis_t B;
	if (jn_jt_basis_build(emax1, emax2, &B)) FAIL(JN_GEN_EINVAL, "invalid JT basis emax1=%d emax2=%d", emax1, emax2);
	if (B.nconfig > 0x7fffffff / 24) { jn_jt_basis_free(&B); FAIL(JN_GEN_EINVAL, "too many configurations"); }
	const int ncol = 6;
	float *rows = xcalloc((size_t)B.nconfig * ncol, sizeof(float));
	const double A = num_particles;
	for (int i = 0; i < B.n; i++)
		for (int k = i; k < B.cfg_end[i]; k++) {
			float *r = rows + (size_t)jn_jt_config(&B, i, k) * ncol;
			if (i == k) {
				int E = B.shells[B.st[i].a].e + B.shells[B.st[i].b].e;
				r[0] = (float)(A * E / (2.0 * (A - 1.0)));
			}
			for (int c = 3; c < 6; c++) r[c] = (float)(sigma * jn_gen_pair_normal(seed, (uint64_t)c, i, k));
		}
	FILE *f = fopen(path, "wb");
	int rc = 0;
	if (!f) { rc = JN_GEN_EIO; snprintf(g_err, sizeof g_err, "open %s: %s", path, strerror(errno)); }
	else {
		struct { int ncol; float hw; int nrow; } hdr = { ncol, (float)hbar_omega, (int)B.nconfig };
		int title[2] = { emax1, emax2 };
		if (fwrite_record(f, title, sizeof title) || fwrite_record(f, &hdr, sizeof hdr) ||
		    fwrite_record(f, rows, (int)(B.nconfig * ncol * sizeof(float)))) {
			rc = JN_GEN_EIO; snprintf(g_err, sizeof g_err, "write %s", path);
		}
		if (fclose(f) && !rc) { rc = JN_GEN_EIO; snprintf(g_err, sizeof g_err, "close %s", path); }
	}
	free(rows);
	jn_jt_basis_free(&B);
	return rc;
}

/*
 * A jjj-coupled three-body interaction in the reference's ASCII format
 * (src/Neptune/input/read_3nf_ascii_format.c:14-279): <dir>/jjj.cnf lists the
 * single-particle shells ("i n l j tz", j doubled, tz -1 proton) and the
 * coupled states ("i a b c Jab Jabc", doubled), <dir>/jjj.mat one
 * "bra ket element" row per ordered pair of states in the same
 * (Jabc, Tz, parity) channel.  The states are those the three-body manager
 * can reach (src/Neptune/bases/jjj_coupled_3p.c:228-357): with shells
 * numbered as the manager numbers them (e; l and j descending; tz),
 * (s s s), (s1 s2 s1), (s1 s2 s2) and (s1 s2 s3) for s1 < s2 < s3, all
 * Jab and Jabc the triangle rules allow, three-particle energy <= e3max.
 * The file numbers its shells in another order (e; l and j ascending), so
 * the reader's shell matching and its a <-> b phase are exercised.  Elements
 * are normal deviates of width sigma, symmetric under bra <-> ket.
 */
typedef struct { int e, n, l, j, tz; } gshell_t;

int jn_gen_jjj_ascii(const char *dir, int emax, int e3max, uint64_t seed, double sigma, int64_t *num_states,
		     int64_t *num_elements)
{
	if (emax < 0 || emax > 7 || e3max < 0 || e3max > 3 * emax) FAIL(JN_GEN_EINVAL, "energies out of range (%d, %d)", emax, e3max);
	/* the manager's order and the file's order of the same shells */
	gshell_t mg[128], fl[128];
	int nm = 0, nf = 0;
	for (int e = 0; e <= emax; e++)
		for (int l = e; l >= (e & 1); l -= 2)
			for (int j = 2 * l + 1; j >= abs(2 * l - 1); j -= 2)
				for (int tz = -1; tz <= 1; tz += 2) { gshell_t g = { e, (e - l) / 2, l, j, tz }; mg[nm++] = g; }
	for (int e = 0; e <= emax; e++)
		for (int l = e & 1; l <= e; l += 2)
			for (int j = abs(2 * l - 1); j <= 2 * l + 1; j += 2)
				for (int tz = -1; tz <= 1; tz += 2) { gshell_t g = { e, (e - l) / 2, l, j, tz }; fl[nf++] = g; }
	int m2f[128];
	for (int a = 0; a < nm; a++)
		for (int b = 0; b < nf; b++)
			if (mg[a].e == fl[b].e && mg[a].l == fl[b].l && mg[a].j == fl[b].j && mg[a].tz == fl[b].tz) m2f[a] = b;
	if (mkdir_p(dir)) FAIL(JN_GEN_EIO, "mkdir %s", dir);
	/* states: (file a, file b, file c, jab, jabc) and the channel (jabc, tz, parity) */
	vec_t st = { 0 };
	st.es = 6 * sizeof(int);
	for (int a = 0; a < nm; a++)
		for (int b = a; b < nm; b++)
			for (int c = 0; c < nm; c++) {
				if (a == b ? c != a : !(c == a || c == b || c > b)) continue;
				if (mg[a].e + mg[b].e + mg[c].e > e3max) continue;
				const int ja = mg[a].j, jb = mg[b].j, jc = mg[c].j;
				const int tz = mg[a].tz + mg[b].tz + mg[c].tz, par = (mg[a].l + mg[b].l + mg[c].l) & 1;
				for (int jab = abs(ja - jb); jab <= ja + jb; jab += 2)
					for (int jabc = abs(jab - jc); jabc <= jab + jc; jabc += 2) {
						int fa = m2f[a], fb = m2f[b];
						if (fa > fb) { int t = fa; fa = fb; fb = t; }    /* the file's own a <= b */
						int r[6] = { fa, fb, m2f[c], jab, jabc, (jabc * 8 + (tz + 3)) * 2 + par };
						if (vpush(&st, r)) { free(st.a); FAIL(JN_GEN_ENOMEM, "out of memory"); }
					}
			}
	char path[4096];
	snprintf(path, sizeof path, "%s/jjj.cnf", dir);
	FILE *f = fopen(path, "w");
	if (!f) { free(st.a); FAIL(JN_GEN_EIO, "open %s: %s", path, strerror(errno)); }
	fprintf(f, "---single-particle-states---\n---i---n---l---j---tz---\n");
	for (int i = 0; i < nf; i++) fprintf(f, "%d %d %d %d %d\n", i, fl[i].n, fl[i].l, fl[i].j, fl[i].tz);
	fprintf(f, "---three-particle-states---\n---i---a---b---c---Jab-Jabc---\n");
	const int *S = (const int *)st.a;
	for (size_t i = 0; i < st.n; i++)
		fprintf(f, "%zu %d %d %d %d %d\n", i, S[6 * i], S[6 * i + 1], S[6 * i + 2], S[6 * i + 3], S[6 * i + 4]);
	if (fclose(f)) { free(st.a); FAIL(JN_GEN_EIO, "write %s", path); }
	/* channels: states grouped by their channel key, in state order */
	int maxch = 0;
	for (size_t i = 0; i < st.n; i++) if (S[6 * i + 5] > maxch) maxch = S[6 * i + 5];
	int *cnt = xcalloc(maxch + 2, sizeof(int)), *first = xcalloc(maxch + 2, sizeof(int));
	int *members = xcalloc(st.n ? st.n : 1, sizeof(int));
	for (size_t i = 0; i < st.n; i++) cnt[S[6 * i + 5]]++;
	for (int c = 1; c <= maxch + 1; c++) first[c] = first[c - 1] + cnt[c - 1];
	memset(cnt, 0, (maxch + 2) * sizeof(int));
	for (size_t i = 0; i < st.n; i++) { int c = S[6 * i + 5]; members[first[c] + cnt[c]++] = (int)i; }
	snprintf(path, sizeof path, "%s/jjj.mat", dir);
	f = fopen(path, "w");
	if (!f) { free(st.a); free(cnt); free(first); free(members); FAIL(JN_GEN_EIO, "open %s: %s", path, strerror(errno)); }
	fprintf(f, "---bra---ket---element---\n");
	int64_t ne = 0;
	for (int c = 0; c <= maxch; c++)
		for (int x = 0; x < cnt[c]; x++)
			for (int y = 0; y < cnt[c]; y++) {
				const int b = members[first[c] + x], k = members[first[c] + y];
				fprintf(f, "%d %d %.17g\n", b, k, sigma * jn_gen_pair_normal(seed, 3, (uint64_t)b, (uint64_t)k));
				ne++;
			}
	int bad = fclose(f) != 0;
	if (num_states) *num_states = (int64_t)st.n;
	if (num_elements) *num_elements = ne;
	free(st.a); free(cnt); free(first); free(members);
	if (bad) FAIL(JN_GEN_EIO, "write %s", path);
	return 0;
}

int jn_generate(const jn_gen_config *cfg, const char *outdir, jn_gen_summary *summary)
{
	gen_t G; memset(&G, 0, sizeof G);
	gen_t *g = &G;
	g->cfg = *cfg;
	g->lists.es = sizeof(ilist_t); g->mes.es = sizeof(meblk_t); g->calcs.es = sizeof(calc_t);
	if (cfg->Z < 0 || cfg->N < 0 || cfg->Z + cfg->N < 2 || cfg->Nmax < 0 || cfg->Z > 60 || cfg->N > 60)
		FAIL(JN_GEN_EINVAL, "invalid nucleus Z=%d N=%d Nmax=%d", cfg->Z, cfg->N, cfg->Nmax);
	if (cfg->nbody != 2 && cfg->nbody != 3) FAIL(JN_GEN_EINVAL, "nbody must be 2 or 3");
	int Ep0 = min_energy(cfg->Z), En0 = min_energy(cfg->N);
	int Etot = Ep0 + En0 + cfg->Nmax;
	int emax = (top_shell(cfg->Z) > top_shell(cfg->N) ? top_shell(cfg->Z) : top_shell(cfg->N)) + cfg->Nmax;
	g->nsp = build_sp(emax, &g->sp);
	if (g->nsp > 64 * MAXW) { gen_free(g); FAIL(JN_GEN_EINVAL, "too many orbitals (%d)", g->nsp); }
	int Epmax = Etot - En0, Enmax = Etot - Ep0;
	if (build_species(g->sp, g->nsp, cfg->Z, Epmax, &g->spc[0]) ||
	    build_species(g->sp, g->nsp, cfg->N, Enmax, &g->spc[1])) {
		gen_free(g); FAIL(JN_GEN_ENOMEM, "species enumeration failed");
	}
	/* k-particle states: an annihilated/created group of k particles of one species
	   has energy at most that species' largest energy */
	int emax_species = Epmax > Enmax ? Epmax : Enmax;
	for (int k = 1; k <= 3; k++) build_kst(g->sp, g->nsp, k, emax_species, &g->kst[k]);
	/* basis blocks: (Ep,Mp,En,Mn) with total energy, parity and M constraints;
	   order: proton sub-basis major, neutron minor */
	vec_t bv = { 0 }; bv.es = sizeof(bblock_t);
	for (int ip = 0; ip < g->spc[0].nsub; ip++)
		for (int in = 0; in < g->spc[1].nsub; in++) {
			subbasis_t *P = &g->spc[0].sub[ip], *Nn = &g->spc[1].sub[in];
			if (P->E + Nn->E > Etot) continue;
			if (((P->E + Nn->E) & 1) != (cfg->parity & 1)) continue;
			if (P->M + Nn->M != cfg->M2) continue;
			bblock_t b = { P->E, P->M, Nn->E, Nn->M, ip, in, (size_t)P->n, (size_t)Nn->n };
			vpush(&bv, &b);
		}
	g->nb = (int)bv.n; g->bb = bv.a;
	if (!g->nb) { gen_free(g); FAIL(JN_GEN_EINVAL, "empty basis"); }
	enumerate_calcs(g);
	/* ids: basis blocks, then lists, then ME blocks (dense 1-based space) */
	int id = g->nb + 1;
	ilist_t *L = g->lists.a;
	for (size_t i = 0; i < g->lists.n; i++) if (L[i].len) L[i].id = id++;
	meblk_t *M = g->mes.a;
	/* only ME blocks referenced by a calc block get an id */
	char *used = xcalloc(g->mes.n, 1);
	calc_t *C = g->calcs.a;
	for (size_t q = 0; q < g->calcs.n; q++) used[C[q].me] = 1;
	for (size_t i = 0; i < g->mes.n; i++) if (used[i]) M[i].id = id++;
	free(used);
	int *order = xcalloc(g->calcs.n, sizeof(int));
	for (size_t q = 0; q < g->calcs.n; q++) order[q] = (int)q;
	g_sort_gen = g;
	qsort(order, g->calcs.n, sizeof(int), cmp_calc_order);

	int rc = 0;
	char path[4096];
	if (mkdir_p(outdir)) { rc = JN_GEN_EIO; snprintf(g_err, sizeof g_err, "mkdir %s", outdir); goto done; }
	snprintf(path, sizeof path, "%s/index_lists", outdir);
	if (mkdir_p(path)) { rc = JN_GEN_EIO; snprintf(g_err, sizeof g_err, "mkdir %s", path); goto done; }
	if (!cfg->me_only) {
		if ((rc = write_lists(g, path))) goto done;
		snprintf(path, sizeof path, "%s/comb.txt", outdir);
		if ((rc = write_comb(g, path, order))) goto done;
		snprintf(path, sizeof path, "%s/evaluation_order.txt", outdir);
		if ((rc = write_eval_order(g, path, order))) goto done;
		if ((rc = write_conf(g, outdir))) goto done;
		if (cfg->write_basis_files && (rc = write_basis_files(g, outdir))) goto done;
		if (cfg->anicre_lists && (rc = write_anicre_lists(g, outdir, cfg->anicre_lists == 2))) goto done;
	}
	{
		const char *medir = cfg->me_subdir && cfg->me_subdir[0] ? cfg->me_subdir : "matrix_elements";
		snprintf(path, sizeof path, "%s/%s", outdir, medir);
		if (mkdir_p(path)) { rc = JN_GEN_EIO; snprintf(g_err, sizeof g_err, "mkdir %s", path); goto done; }
		if ((rc = write_me_blocks(g, path))) goto done;
	}
	if (cfg->antoine) {
		snprintf(path, sizeof path, "%s/antoine_2nf.bin", outdir);
		if ((rc = jn_gen_antoine(path, emax, Etot, cfg->Z + cfg->N, cfg->hbar_omega, cfg->seed * 1000003ull + 2,
					 cfg->sigma2)))
			goto done;
	}
	if (summary) {
		memset(summary, 0, sizeof *summary);
		summary->emax_single = emax;
		summary->emax_pair = Etot;
		summary->num_basis_blocks = g->nb;
		for (int b = 0; b < g->nb; b++) summary->dimension += g->bb[b].np_ * g->bb[b].nn_;
		for (size_t i = 0; i < g->lists.n; i++) if (L[i].len) { summary->num_lists++; summary->list_entries += L[i].len; }
		for (size_t i = 0; i < g->mes.n; i++) if (M[i].id) {
			summary->num_me_blocks++;
			size_t len = M[i].kp && M[i].kn ? M[i].np_conn * M[i].nn_conn : (M[i].kp ? M[i].np_conn : M[i].nn_conn);
			summary->me_elements += len;
		}
		summary->num_calc_blocks = g->calcs.n;
		summary->num_orbitals = g->nsp;
		summary->num_proton_sds = g->spc[0].nsd;
		summary->num_neutron_sds = g->spc[1].nsd;
		for (size_t q = 0; q < g->calcs.n; q++) summary->multiplications += C[q].mults;
	}
done:
	free(order);
	gen_free(g);
	return rc;
}

void jn_gen_default_config(jn_gen_config *cfg)
{
	memset(cfg, 0, sizeof *cfg);
	cfg->Z = 2; cfg->N = 2; cfg->Nmax = 4; cfg->M2 = 0; cfg->parity = 0; cfg->nbody = 2;
	cfg->seed = 20261203ull; cfg->hbar_omega = 20.0; cfg->sigma2 = 1.0; cfg->sigma3 = 0.1;
	cfg->write_basis_files = 1; cfg->lanczos_iterations = 200;
}

#ifdef JN_GEN_MAIN
static void usage(const char *p)
{
	fprintf(stderr,
		"usage: %s --out DIR [--Z n] [--N n] [--nmax n] [--M2 n] [--parity 0|1] [--nbody 2|3]\n"
		"          [--seed s] [--hw MeV] [--sigma2 s] [--sigma3 s] [--me-only SUBDIR] [--no-basis-files]\n"
		"          [--antoine]\n", p);
}
int main(int argc, char **argv)
{
	jn_gen_config c; jn_gen_default_config(&c);
	const char *out = NULL;
	for (int i = 1; i < argc; i++) {
		const char *a = argv[i];
		const char *v = i + 1 < argc ? argv[i + 1] : NULL;
		if (!strcmp(a, "--out") && v) { out = v; i++; }
		else if (!strcmp(a, "--Z") && v) { c.Z = atoi(v); i++; }
		else if (!strcmp(a, "--N") && v) { c.N = atoi(v); i++; }
		else if (!strcmp(a, "--nmax") && v) { c.Nmax = atoi(v); i++; }
		else if (!strcmp(a, "--M2") && v) { c.M2 = atoi(v); i++; }
		else if (!strcmp(a, "--parity") && v) { c.parity = atoi(v); i++; }
		else if (!strcmp(a, "--nbody") && v) { c.nbody = atoi(v); i++; }
		else if (!strcmp(a, "--seed") && v) { c.seed = strtoull(v, NULL, 10); i++; }
		else if (!strcmp(a, "--hw") && v) { c.hbar_omega = atof(v); i++; }
		else if (!strcmp(a, "--sigma2") && v) { c.sigma2 = atof(v); i++; }
		else if (!strcmp(a, "--sigma3") && v) { c.sigma3 = atof(v); i++; }
		else if (!strcmp(a, "--me-only") && v) { c.me_only = 1; c.me_subdir = v; i++; }
		else if (!strcmp(a, "--no-basis-files")) c.write_basis_files = 0;
		else if (!strcmp(a, "--antoine")) c.antoine = 1;
		else { usage(argv[0]); return 2; }
	}
	if (!out) { usage(argv[0]); return 2; }
	jn_gen_summary s;
	int rc = jn_generate(&c, out, &s);
	if (rc) { fprintf(stderr, "jn_gen: %s\n", jn_gen_last_error()); return 1; }
	printf("dimension %zu blocks %d lists %zu entries %zu me_blocks %zu me_elements %zu calc_blocks %zu mults %llu"
	       " emax_single %d emax_pair %d\n",
	       s.dimension, s.num_basis_blocks, s.num_lists, s.list_entries, s.num_me_blocks, s.me_elements,
	       s.num_calc_blocks, (unsigned long long)s.multiplications, s.emax_single, s.emax_pair);
	return 0;
}
#endif
