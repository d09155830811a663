/*
 * jn_transform.c — host plan of the two-body J -> M transform (see
 * jn_transform.h for the reduction that makes it a per-element short sum).
 *
 * Reference parts restated here, in the order the plan builds them:
 *   combination table matrix-element rows   src/Utilities/combination_table/combination_table.c:530-640
 *   Antoine file and kinetic term           src/Neptune/input/read_2nf_antoine_format.c:70-236
 *   single-particle order (e, l, j, m desc)  src/Neptune/bases/sp_states.c:7-70
 *   two-particle M-scheme bases              src/Neptune/bases/m_scheme_2p_basis.c:175-204, 498-581
 *   coefficients S = N * CG * CG             src/Neptune/jt_transformation/jt_transformation.c:207-341
 *   connections                              src/Mercury/connection_list/connection_list.c:61-180, 380-431
 *   bra/ket pair order and phase             src/Mercury/transform_2nf_block_manager/transform_2nf_block_manager.c:411-515
 */
#include "jn_transform.h"

#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define TERR(...) do { snprintf(err, errlen, __VA_ARGS__); goto fail; } while (0)

typedef struct { void *a; size_t n, cap, es; } tvec_t;

static int tpush(tvec_t *v, const void *e)
{
	if (v->n == v->cap) {
		size_t c = v->cap ? 2 * v->cap : 64;
		void *p = realloc(v->a, c * v->es);
		if (!p) return -1;
		v->a = p; v->cap = c;
	}
	memcpy((char *)v->a + v->n * v->es, e, v->es);
	v->n++;
	return 0;
}

/* ------------------------------------------------------------------ */
/* single-particle orbitals up to emax1                                */
/* ------------------------------------------------------------------ */
typedef struct { int e, l, j, m, tse; } orb_t;

static int build_orbitals(int emax, orb_t **out)
{
	int n = 0, tse = 0;
	for (int pass = 0; pass < 2; pass++) {
		n = 0; tse = 0;
		for (int e = 0; e <= emax; e++)
			for (int l = e & 1; l <= e; l += 2)
				for (int j = abs(2 * l - 1); j <= 2 * l + 1; j += 2, tse++)
					for (int m = j; m >= -j; m -= 2) {
						if (pass) { orb_t o = { e, l, j, m, tse }; (*out)[n] = o; }
						n++;
					}
		if (!pass) *out = (orb_t *)calloc(n, sizeof(orb_t));
	}
	return n;
}

/* ------------------------------------------------------------------ */
/* Anicre basis files, read once per (species, particles, energy)      */
/* ------------------------------------------------------------------ */
typedef struct { char sp; int k, E; int64_t n; int16_t *s; } bfile_t;

typedef struct {
	const char *dir;
	tvec_t files;           /* bfile_t *, each allocated once so that pointers stay valid */
} bcache_t;

static void bcache_free(bcache_t *c)
{
	for (size_t i = 0; i < c->files.n; i++) {
		bfile_t *f = ((bfile_t **)c->files.a)[i];
		free(f->s);
		free(f);
	}
	free(c->files.a);
	c->files.a = NULL;
	c->files.n = 0;
}

static const bfile_t *bfile(bcache_t *c, char sp, int k, int E, int norb, char *err, size_t errlen)
{
	bfile_t **f = (bfile_t **)c->files.a;
	for (size_t i = 0; i < c->files.n; i++)
		if (f[i]->sp == sp && f[i]->k == k && f[i]->E == E) return f[i];
	char path[4352];
	snprintf(path, sizeof path, "%s/%.*s_inds_index_lists/basis_energy_%d", c->dir, k, sp == 'p' ? "ppp" : "nnn", E);
	FILE *fp = fopen(path, "rb");
	if (!fp) { snprintf(err, errlen, "Could not open file \"%s\". %s", path, strerror(errno)); return NULL; }
	fseek(fp, 0, SEEK_END);
	long bytes = ftell(fp);
	fseek(fp, 0, SEEK_SET);
	if (bytes < 0 || bytes % (2 * k)) { fclose(fp); snprintf(err, errlen, "%s: size is not a multiple of %d", path, 2 * k); return NULL; }
	bfile_t nf = { sp, k, E, bytes / (2 * k), (int16_t *)malloc(bytes ? bytes : 1) };
	if (bytes && fread(nf.s, 1, bytes, fp) != (size_t)bytes) {
		fclose(fp); free(nf.s); snprintf(err, errlen, "%s: short read", path); return NULL;
	}
	fclose(fp);
	for (int64_t i = 0; i < nf.n * k; i++)
		if (nf.s[i] < 0 || nf.s[i] >= norb) {
			int bad = nf.s[i];
			free(nf.s);
			snprintf(err, errlen, "%s: orbital %d outside the %d orbitals of the single-particle energy limit", path,
				 bad, norb);
			return NULL;
		}
	bfile_t *keep = (bfile_t *)malloc(sizeof *keep);
	if (!keep || (*keep = nf, tpush(&c->files, &keep))) {
		free(nf.s); free(keep); snprintf(err, errlen, "out of memory"); return NULL;
	}
	return keep;
}

/* ------------------------------------------------------------------ */
/* two-particle M-scheme bases, one per (Tz, Ep, En)                    */
/* ------------------------------------------------------------------ */
typedef struct {
	int tz, Ep, En;
	int64_t first;          /* first pair-state id */
	int64_t n;
	int nn;                 /* Tz = 0: neutron states of the En file (LUT row length) */
	int64_t lut;            /* Tz = 0: first LUT entry */
	int minM, maxM;
} pbasis_t;

typedef struct { int a, b, M; int64_t pos; } pstate_t;

static int cmp_pstate(const void *x, const void *y)
{
	const pstate_t *p = (const pstate_t *)x, *q = (const pstate_t *)y;
	if (p->M != q->M) return p->M < q->M ? -1 : 1;
	if (p->a != q->a) return p->a < q->a ? -1 : 1;
	if (p->b != q->b) return p->b < q->b ? -1 : 1;
	return 0;
}

typedef struct {
	const orb_t *orb;
	int norb;
	const jn_jt_basis_t *jt;
	int jmax;               /* largest J of the reference's loop: 2 emax1 + 1 */
	int *jt_index;          /* (2J+T) x nshells x nshells -> coupled state or -1 */
	tvec_t bases;           /* pbasis_t */
	tvec_t ms;              /* jn_mstate_t */
	tvec_t cs;              /* double */
	tvec_t ca;              /* int32 */
	tvec_t lut;             /* int32 */
	double dense_flops;
} tbuild_t;

/* the sign convention of jt_transformation.c:321 (C remainder: -1 % 2 != 1) */
static int is_odd_ref(int x) { return x % 2 == 1; }

/* S(J,T) and alpha for the pair of interleaved states a < b
 * (jt_transformation.c:267-341) */
static void expand_pair(tbuild_t *t, int a, int b, int tz, jn_mstate_t *m)
{
	const orb_t *oa = &t->orb[a >> 1], *ob = &t->orb[b >> 1];
	int tza = (a & 1) ? 1 : -1, tzb = (b & 1) ? 1 : -1;
	int ta = oa->tse, tb = ob->tse;
	int ja = oa->j, jb = ob->j, ma = oa->m, mb = ob->m;
	int swapped = 0;
	if (ta > tb) {          /* the coupled state is (tb, ta): exchange the particles */
		swapped = 1;
		int x;
		x = ta; ta = tb; tb = x;
		x = ja; ja = jb; jb = x;
		x = ma; ma = mb; mb = x;
		x = tza; tza = tzb; tzb = x;
	}
	const int M = ma + mb;
	int jlo = abs(ja - jb) / 2, jhi = (ja + jb) / 2;
	if (abs(M) / 2 > jlo) jlo = abs(M) / 2;
	if (jhi > t->jmax) jhi = t->jmax;
	if (jhi > t->jt->nJ - 1) jhi = t->jt->nJ - 1;
	m->M = (int16_t)M;
	m->jlo = (int16_t)jlo;
	m->nj = (int16_t)(jhi >= jlo ? jhi - jlo + 1 : 0);
	m->coef = (int32_t)t->cs.n;
	const int tlo = abs(tz) / 2;
	const int ns = t->jt->nshells;
	for (int J = jlo; J <= jhi; J++)
		for (int T = 0; T <= 1; T++) {
			double s = 0.0;
			int32_t alpha = -1;
			if (T >= tlo) {
				int idx = t->jt_index[((size_t)(2 * J + T) * ns + ta) * ns + tb];
				if (idx >= 0) {
					double norm = 0.0;
					if (ta != tb) norm = 1.0;
					else if (is_odd_ref(J + T)) norm = sqrt(2.0);
					if (is_odd_ref((ja + jb) / 2 - J - T) && swapped) norm = -norm;
					if (fabs(norm) >= 1e-10) {
						double cg1 = jn_cg(ja, jb, 2 * J, ma, mb, ma + mb);
						double cg2 = jn_cg(1, 1, 2 * T, tza, tzb, tza + tzb);
						s = norm * cg1 * cg2;
						if (fabs(s) < 1e-10) s = 0.0;
					}
					if (s != 0.0) alpha = idx;
				}
			}
			tpush(&t->cs, &s);
			tpush(&t->ca, &alpha);
		}
}

static int m_of(const tbuild_t *t, int interleaved) { return t->orb[interleaved >> 1].m; }

/* the pair basis for (tz, Ep, En), built on first use; returns its index */
static int pair_basis(tbuild_t *t, bcache_t *bc, int tz, int Ep, int En, char *err, size_t errlen)
{
	pbasis_t *B = (pbasis_t *)t->bases.a;
	for (size_t i = 0; i < t->bases.n; i++)
		if (B[i].tz == tz && B[i].Ep == Ep && B[i].En == En) return (int)i;
	pbasis_t nb = { tz, Ep, En, (int64_t)t->ms.n, 0, 0, -1, 0, 0 };
	pstate_t *st = NULL;
	int64_t n = 0;
	if (tz != 0) {
		/* one species: the file's pairs in file order, which must come grouped by
		   ascending M (m_scheme_2p_basis.c:498-520, cut_out_M_block :260-282) */
		const bfile_t *f = bfile(bc, tz < 0 ? 'p' : 'n', 2, tz < 0 ? Ep : En, t->norb, err, errlen);
		if (!f) return -1;
		n = f->n;
		st = (pstate_t *)calloc(n ? n : 1, sizeof(pstate_t));
		const int odd = tz > 0;
		for (int64_t i = 0; i < n; i++) {
			int o0 = f->s[2 * i], o1 = f->s[2 * i + 1];
			int a = 2 * (o0 < o1 ? o0 : o1) + odd, b = 2 * (o0 < o1 ? o1 : o0) + odd;
			st[i].a = a; st[i].b = b; st[i].M = m_of(t, a) + m_of(t, b); st[i].pos = i;
			if (i && st[i].M < st[i - 1].M) {
				free(st);
				snprintf(err, errlen, "%cp basis of energy %d is not ordered by M", tz < 0 ? 'p' : 'n', tz < 0 ? Ep : En);
				return -1;
			}
		}
	} else {
		/* protons x neutrons, sorted by (M, a, b) (m_scheme_2p_basis.c:522-581) */
		const bfile_t *fp = bfile(bc, 'p', 1, Ep, t->norb, err, errlen);
		if (!fp) return -1;
		const bfile_t *fn = bfile(bc, 'n', 1, En, t->norb, err, errlen);
		if (!fn) return -1;
		n = fp->n * fn->n;
		nb.nn = (int)fn->n;
		st = (pstate_t *)calloc(n ? n : 1, sizeof(pstate_t));
		for (int64_t i = 0; i < fp->n; i++)
			for (int64_t k = 0; k < fn->n; k++) {
				int p = 2 * fp->s[i], q = 2 * fn->s[k] + 1;
				pstate_t *s = &st[i * fn->n + k];
				s->a = p < q ? p : q; s->b = p < q ? q : p; s->M = m_of(t, p) + m_of(t, q);
				s->pos = i * fn->n + k;
			}
		qsort(st, n, sizeof(pstate_t), cmp_pstate);
	}
	nb.n = n;
	if (n) { nb.minM = st[0].M; nb.maxM = st[n - 1].M; }
	/* pair states in basis order; the position inside the M block */
	int64_t run = 0;
	for (int64_t i = 0; i < n; i++) {
		if (i && st[i].M != st[i - 1].M) run = i;
		jn_mstate_t m;
		memset(&m, 0, sizeof m);
		expand_pair(t, st[i].a, st[i].b, tz, &m);
		m.mindex = (int32_t)(i - run);
		m.phase = 1;
		tpush(&t->ms, &m);
	}
	if (tz == 0) {
		/* LUT: (proton position, neutron position) -> pair state; the ket/bra is
		   ordered (2n+1, 2p) and flips sign when that is descending
		   (transform_2nf_block_manager.c:435-450) */
		nb.lut = (int64_t)t->lut.n;
		int32_t *tmp = (int32_t *)calloc(n ? n : 1, sizeof(int32_t));
		for (int64_t i = 0; i < n; i++) tmp[st[i].pos] = (int32_t)(nb.first + i);
		const bfile_t *fp = bfile(bc, 'p', 1, Ep, t->norb, err, errlen);
		const bfile_t *fn = bfile(bc, 'n', 1, En, t->norb, err, errlen);
		for (int64_t i = 0; i < fp->n; i++)
			for (int64_t k = 0; k < fn->n; k++) {
				int32_t id = tmp[i * fn->n + k];
				int neg = 2 * fn->s[k] + 1 > 2 * fp->s[i];
				int32_t v = neg ? -id - 1 : id;
				tpush(&t->lut, &v);
			}
		free(tmp);
	}
	free(st);
	if (t->ms.n > 0x7fffffff || t->cs.n > 0x7fffffff) { snprintf(err, errlen, "too many pair states"); return -1; }
	if (tpush(&t->bases, &nb)) { snprintf(err, errlen, "out of memory"); return -1; }
	return (int)t->bases.n - 1;
}

/* ------------------------------------------------------------------ */
/* combination-table matrix-element rows                                */
/* ------------------------------------------------------------------ */
static int split_words(char *line, char **w, int max)
{
	int n = 0;
	for (char *s = strtok(line, " \t\r\n"); s && n < max; s = strtok(NULL, " \t\r\n")) w[n++] = s;
	return n;
}

static int parse_id(const char *s)
{
	int id = 0;
	while (*s && *s != '=') {
		if (*s < '0' || *s > '9') return -1;
		id = 10 * id + (*s++ - '0');
	}
	return id;
}

static int count_char(const char *s, char c)
{
	int n = 0;
	for (; *s; s++) n += *s == c;
	return n;
}

static int read_me_rows(const char *comb, tvec_t *out, char *err, size_t errlen)
{
	FILE *f = fopen(comb, "r");
	if (!f) { snprintf(err, errlen, "Could not open %s: %s", comb, strerror(errno)); return -1; }
	char line[4096];
	int sec = 0;    /* 1 cross p-n, 2 same p/n */
	while (fgets(line, sizeof line, f)) {
		if (strstr(line, "***")) {
			sec = strstr(line, "Matrix-elements V (cross p-n)") ? 1 : strstr(line, "Matrix-elements V (same p/n)") ? 2 : 0;
			continue;
		}
		if (!sec || !strstr(line, "ARRAY:")) continue;
		char *w[32];
		int nw = split_words(line, w, 32);
		jn_meblock_info_t b;
		memset(&b, 0, sizeof b);
		if (sec == 1) {
			if (nw < 14) { fclose(f); snprintf(err, errlen, "%s: short cross p-n row", comb); return -1; }
			b.np = count_char(w[0], 'p'); b.nn = count_char(w[4], 'n');
			b.dEp = atoi(w[1]); b.dMp = atoi(w[2]); b.dp = atoi(w[3]);
			b.dEn = atoi(w[5]); b.dMn = atoi(w[6]); b.dn = atoi(w[7]);
			b.Np = strtoull(w[8], NULL, 10); b.Nn = strtoull(w[9], NULL, 10);
			b.id = parse_id(w[13]);
		} else {
			if (nw < 9) { fclose(f); snprintf(err, errlen, "%s: short same p/n row", comb); return -1; }
			int k = (int)strlen(w[0]);
			if (w[0][0] == 'p') { b.np = k; b.dEp = atoi(w[1]); b.dMp = atoi(w[2]); b.dp = atoi(w[3]); b.Np = strtoull(w[4], NULL, 10); }
			else { b.nn = k; b.dEn = atoi(w[1]); b.dMn = atoi(w[2]); b.dn = atoi(w[3]); b.Nn = strtoull(w[4], NULL, 10); }
			b.id = parse_id(w[8]);
		}
		if (b.id <= 0) { fclose(f); snprintf(err, errlen, "%s: bad array id", comb); return -1; }
		if (tpush(out, &b)) { fclose(f); snprintf(err, errlen, "out of memory"); return -1; }
	}
	fclose(f);
	return 0;
}

int jn_read_me_blocks(const char *comb, jn_meblock_info_t **rows, int *n, char *err, size_t errlen)
{
	tvec_t v = { 0 };
	v.es = sizeof(jn_meblock_info_t);
	*rows = NULL;
	*n = 0;
	if (read_me_rows(comb, &v, err, errlen)) {
		free(v.a);
		return -1;
	}
	*rows = (jn_meblock_info_t *)v.a;
	*n = (int)v.n;
	return 0;
}

/* ------------------------------------------------------------------ */
/* Antoine file (three Fortran records)                                 */
/* ------------------------------------------------------------------ */
static int read_record(FILE *f, void **buf, int *len)
{
	int a, b;
	if (fread(&a, 4, 1, f) != 1 || a < 0) return -1;
	*buf = malloc(a ? a : 1);
	if (a && fread(*buf, 1, a, f) != (size_t)a) { free(*buf); *buf = NULL; return -1; }
	if (fread(&b, 4, 1, f) != 1 || a != b) { free(*buf); *buf = NULL; return -1; }
	*len = a;
	return 0;
}

static int read_antoine(jn_tplan_t *p, const char *path, int include_kinetic, char *err, size_t errlen)
{
	FILE *f = fopen(path, "rb");
	if (!f) { snprintf(err, errlen, "Could not open file \"%s\". %s.", path, strerror(errno)); return -1; }
	void *r1 = NULL, *r2 = NULL, *r3 = NULL;
	int l1, l2, l3;
	int rc = -1;
	if (read_record(f, &r1, &l1)) { snprintf(err, errlen, "%s: no title record", path); goto out; }
	if (read_record(f, &r2, &l2) || l2 != 12) { snprintf(err, errlen, "%s: bad header record", path); goto out; }
	struct { int ncol; float hw; int nrow; } h;
	memcpy(&h, r2, 12);
	if (h.ncol < 6 || h.nrow < 0) { snprintf(err, errlen, "%s: header ncol=%d nrow=%d", path, h.ncol, h.nrow); goto out; }
	if ((int64_t)h.nrow != p->jt.nconfig) {
		snprintf(err, errlen, "%s has %d rows but the coupled basis (single-particle energy %d, two-particle energy %d) "
			 "has %lld configurations", path, h.nrow, p->emax1, p->emax2, (long long)p->jt.nconfig);
		goto out;
	}
	if (read_record(f, &r3, &l3) || (int64_t)l3 != (int64_t)h.nrow * h.ncol * 4) {
		snprintf(err, errlen, "%s: element record does not hold %d x %d floats", path, h.nrow, h.ncol);
		goto out;
	}
	const float *raw = (const float *)r3;
	const int64_t nc = h.nrow;
	p->V = (double *)malloc(3 * (nc ? nc : 1) * sizeof(double));
	const int cols[3] = { 3, 5, 4 };        /* Tz = -2, 0, +2 */
	const double A = (double)(p->Z + p->N);
	for (int64_t i = 0; i < nc; i++) {
		double kin = 0.0;
		if (include_kinetic) kin = (2.0) * (double)h.hw * (double)raw[(int64_t)h.ncol * i] / A;
		for (int t = 0; t < 3; t++) {
			double v = (double)raw[(int64_t)h.ncol * i + cols[t]];
			p->V[t * nc + i] = include_kinetic ? v + kin : v;
		}
	}
	rc = 0;
out:
	free(r1); free(r2); free(r3);
	fclose(f);
	return rc;
}

/* ------------------------------------------------------------------ */
/* connections                                                          */
/* ------------------------------------------------------------------ */
static int state_M(const tbuild_t *t, const int16_t *s, int k)
{
	int M = 0;
	for (int i = 0; i < k; i++) M += t->orb[s[i]].m;
	return M;
}

/* annihilated states of `ann` x created states of `cre` with M + dM, in
 * Mercury's order (connection_list.c:380-431) */
static int connections(const tbuild_t *t, const bfile_t *ann, const bfile_t *cre, int dM, tvec_t *pairs)
{
	const int k = ann->k;
	for (int64_t i = 0; i < ann->n; i++) {
		int Mc = state_M(t, ann->s + i * k, k) + dM;
		int64_t c = 0;
		while (c < cre->n && state_M(t, cre->s + c * k, k) != Mc) c++;
		for (; c < cre->n && state_M(t, cre->s + c * k, k) == Mc; c++) {
			int32_t pr[2] = { (int32_t)i, (int32_t)c };
			if (tpush(pairs, pr)) return -1;
		}
	}
	return 0;
}

void jn_tplan_free(jn_tplan_t *p)
{
	if (!p) return;
	jn_jt_basis_free(&p->jt);
	free(p->V); free(p->info); free(p->tb); free(p->tb_info); free(p->ms); free(p->coef_s); free(p->coef_a);
	free(p->conn_ket); free(p->conn_bra); free(p->conn_sign); free(p->pc); free(p->nc); free(p->lut);
	free(p->z1_info); free(p->z1_count);
	memset(p, 0, sizeof *p);
}

int jn_tplan_build(jn_tplan_t *p, const char *comb, const char *lists_dir, int Z, int N, int emax1, int emax2,
		   const char *antoine, int include_kinetic, char *err, size_t errlen)
{
	memset(p, 0, sizeof *p);
	tbuild_t t;
	memset(&t, 0, sizeof t);
	bcache_t bc;
	memset(&bc, 0, sizeof bc);
	orb_t *orb = NULL;
	tvec_t rows = { 0 }, tb = { 0 }, tbi = { 0 }, c1 = { 0 }, pcv = { 0 }, ncv = { 0 }, pairs = { 0 };
	rows.es = sizeof(jn_meblock_info_t); tb.es = sizeof(jn_tblock_t); tbi.es = sizeof(int);
	c1.es = 3 * sizeof(int32_t); pcv.es = sizeof(jn_pconn_t); ncv.es = sizeof(jn_nconn_t); pairs.es = 2 * sizeof(int32_t);
	t.bases.es = sizeof(pbasis_t); t.ms.es = sizeof(jn_mstate_t); t.cs.es = sizeof(double); t.ca.es = sizeof(int32_t);
	t.lut.es = sizeof(int32_t);
	bc.dir = lists_dir; bc.files.es = sizeof(bfile_t *);

	if (Z < 0 || N < 0 || Z + N < 2) TERR("the transform needs at least two particles (Z=%d N=%d)", Z, N);
	if (emax1 < 0 || emax2 < 0 || emax1 > 30 || emax2 > 60) TERR("energies out of range (%d, %d)", emax1, emax2);
	p->Z = Z; p->N = N; p->emax1 = emax1; p->emax2 = emax2;
	p->jmax = 2 * emax1 + 1;                /* J_max / 2 of transform_2nf_block_manager.c:98 */
	if (jn_jt_basis_build(emax1, emax2, &p->jt)) TERR("coupled basis (%d, %d) failed", emax1, emax2);
	if (read_antoine(p, antoine, include_kinetic, err, errlen)) goto fail;
	if (read_me_rows(comb, &rows, err, errlen)) goto fail;
	p->nblocks = (int)rows.n;
	p->info = (jn_meblock_info_t *)rows.a;
	rows.a = NULL;

	t.norb = build_orbitals(emax1, &orb);
	t.orb = orb;
	t.jt = &p->jt;
	t.jmax = p->jmax;
	{
		const int ns = p->jt.nshells;
		size_t nidx = (size_t)2 * p->jt.nJ * ns * ns;
		t.jt_index = (int *)malloc(nidx * sizeof(int));
		for (size_t i = 0; i < nidx; i++) t.jt_index[i] = -1;
		for (int i = 0; i < p->jt.n; i++) {
			const jn_jt_state_t *s = &p->jt.st[i];
			t.jt_index[((size_t)(2 * s->J + s->T) * ns + s->a) * ns + s->b] = i;
		}
	}

	p->z1_info = (int *)calloc(p->nblocks ? p->nblocks : 1, sizeof(int));
	p->z1_count = (int64_t *)calloc(p->nblocks ? p->nblocks : 1, sizeof(int64_t));
	int64_t nelem = 0;
	for (int i = 0; i < p->nblocks; i++) {
		const jn_meblock_info_t *b = &p->info[i];
		if (b->np + b->nn == 1) {
			/* one-body blocks are written as zeros of their connection count */
			const char sp = b->np ? 'p' : 'n';
			const int depth = b->np ? b->dp : b->dn, dE = b->np ? b->dEp : b->dEn, dM = b->np ? b->dMp : b->dMn;
			const bfile_t *ann = bfile(&bc, sp, 1, depth, t.norb, err, errlen);
			const bfile_t *cre = ann ? bfile(&bc, sp, 1, depth + dE, t.norb, err, errlen) : NULL;
			if (!cre) goto fail;
			pairs.n = 0;
			if (connections(&t, ann, cre, dM, &pairs)) TERR("out of memory");
			p->z1_info[p->n1] = i;
			p->z1_count[p->n1++] = (int64_t)pairs.n;
			continue;
		}
		if (b->np + b->nn != 2) continue;
		jn_tblock_t d;
		memset(&d, 0, sizeof d);
		d.out = nelem;
		const int tz = b->nn - b->np;
		d.tz = tz / 2 + 1;
		if (b->np == 1 && b->nn == 1) {
			/* protons x neutrons: p major, n minor (connection_list.c:108-147) */
			int kb = pair_basis(&t, &bc, 0, b->dp, b->dn, err, errlen);
			if (kb < 0) goto fail;
			int bb = pair_basis(&t, &bc, 0, b->dp + b->dEp, b->dn + b->dEn, err, errlen);
			if (bb < 0) goto fail;
			const pbasis_t *KB = &((pbasis_t *)t.bases.a)[kb], *BB = &((pbasis_t *)t.bases.a)[bb];
			const bfile_t *pa = bfile(&bc, 'p', 1, b->dp, t.norb, err, errlen);
			const bfile_t *pcr = pa ? bfile(&bc, 'p', 1, b->dp + b->dEp, t.norb, err, errlen) : NULL;
			const bfile_t *na = pcr ? bfile(&bc, 'n', 1, b->dn, t.norb, err, errlen) : NULL;
			const bfile_t *ncr = na ? bfile(&bc, 'n', 1, b->dn + b->dEn, t.norb, err, errlen) : NULL;
			if (!ncr) goto fail;
			pairs.n = 0;
			if (connections(&t, pa, pcr, b->dMp, &pairs)) TERR("out of memory");
			int64_t npc = (int64_t)pairs.n;
			d.conn = (int32_t)pcv.n;
			for (size_t q = 0; q < pairs.n; q++) {
				const int32_t *pr = (const int32_t *)pairs.a + 2 * q;
				jn_pconn_t c = { pr[0], pr[1], (int32_t)KB->lut, (int32_t)BB->lut, KB->nn, BB->nn };
				if (tpush(&pcv, &c)) TERR("out of memory");
			}
			pairs.n = 0;
			if (connections(&t, na, ncr, b->dMn, &pairs)) TERR("out of memory");
			int64_t nnc = (int64_t)pairs.n;
			d.nconn = (int32_t)ncv.n;
			for (size_t q = 0; q < pairs.n; q++) {
				const int32_t *pr = (const int32_t *)pairs.a + 2 * q;
				jn_nconn_t c = { pr[0], pr[1] };
				if (tpush(&ncv, &c)) TERR("out of memory");
			}
			if ((uint64_t)npc != b->Np || (uint64_t)nnc != b->Nn)
				TERR("matrix block %d should have %llu x %llu connections but has %lld x %lld", b->id,
				     (unsigned long long)b->Np, (unsigned long long)b->Nn, (long long)npc, (long long)nnc);
			/* every ket/bra pair must keep its M (the block manager reads D_M at the ket's M) */
			for (int64_t q = 0; q < npc; q++) {
				const jn_pconn_t *c = &((jn_pconn_t *)pcv.a)[d.conn + q];
				for (int64_t r = 0; r < nnc; r++) {
					const jn_nconn_t *e = &((jn_nconn_t *)ncv.a)[d.nconn + r];
					int32_t ki = ((int32_t *)t.lut.a)[c->ket_lut + (int64_t)c->p_ann * c->ket_nn + e->n_ann];
					int32_t bi = ((int32_t *)t.lut.a)[c->bra_lut + (int64_t)c->p_cre * c->bra_nn + e->n_cre];
					if (ki < 0) ki = -ki - 1;
					if (bi < 0) bi = -bi - 1;
					if (((jn_mstate_t *)t.ms.a)[ki].M != ((jn_mstate_t *)t.ms.a)[bi].M)
						TERR("matrix block %d connects different total M", b->id);
				}
			}
			d.kind = 1;
			d.nn = (int32_t)nnc;
			d.count = npc * nnc;
		} else {
			/* one species, two particles */
			const char sp = b->np ? 'p' : 'n';
			const int depth = b->np ? b->dp : b->dn, dE = b->np ? b->dEp : b->dEn, dM = b->np ? b->dMp : b->dMn;
			int kb = pair_basis(&t, &bc, tz, b->np ? depth : 0, b->np ? 0 : depth, err, errlen);
			if (kb < 0) goto fail;
			int bb = pair_basis(&t, &bc, tz, b->np ? depth + dE : 0, b->np ? 0 : depth + dE, err, errlen);
			if (bb < 0) goto fail;
			const bfile_t *ann = bfile(&bc, sp, 2, depth, t.norb, err, errlen);
			const bfile_t *cre = ann ? bfile(&bc, sp, 2, depth + dE, t.norb, err, errlen) : NULL;
			if (!cre) goto fail;
			pairs.n = 0;
			if (connections(&t, ann, cre, dM, &pairs)) TERR("out of memory");
			const uint64_t want = b->np ? b->Np : b->Nn;
			if ((uint64_t)pairs.n != want)
				TERR("matrix block %d should have %llu connections but has %zu", b->id, (unsigned long long)want,
				     pairs.n);
			const pbasis_t *KB = &((pbasis_t *)t.bases.a)[kb], *BB = &((pbasis_t *)t.bases.a)[bb];
			d.conn = (int32_t)c1.n;
			for (size_t q = 0; q < pairs.n; q++) {
				const int32_t *pr = (const int32_t *)pairs.a + 2 * q;
				int32_t e[3];
				e[0] = (int32_t)(KB->first + pr[0]);
				e[1] = (int32_t)(BB->first + pr[1]);
				const int16_t *ks = ann->s + 2 * (int64_t)pr[0], *bs = cre->s + 2 * (int64_t)pr[1];
				int sign = (ks[0] > ks[1] ? -1 : 1) * (bs[0] > bs[1] ? -1 : 1);
				e[2] = sign;
				if (((jn_mstate_t *)t.ms.a)[e[0]].M != ((jn_mstate_t *)t.ms.a)[e[1]].M)
					TERR("matrix block %d connects different total M", b->id);
				if (tpush(&c1, e)) TERR("out of memory");
			}
			d.kind = 0;
			d.count = (int64_t)pairs.n;
		}
		nelem += d.count;
		if (tpush(&tb, &d) || tpush(&tbi, &i)) TERR("out of memory");
	}
	if (pcv.n > 0x7fffffff || ncv.n > 0x7fffffff || c1.n > 0x7fffffff) TERR("too many connections");

	/* flops of the reference's dense formulation for every decoupled (energies, Tz, M) */
	{
		const pbasis_t *B = (const pbasis_t *)t.bases.a;
		const jn_tblock_t *T = (const jn_tblock_t *)tb.a;
		tvec_t seen = { 0 };
		seen.es = 2 * sizeof(int);
		for (size_t i = 0; i < tb.n; i++) {
			const jn_meblock_info_t *b = &p->info[((int *)tbi.a)[i]];
			const int tz = b->nn - b->np;
			int kb = -1, bb = -1;
			for (size_t q = 0; q < t.bases.n; q++) {
				if (B[q].tz != tz) continue;
				if (B[q].Ep == (tz <= 0 ? b->dp : 0) && B[q].En == (tz >= 0 ? b->dn : 0)) kb = (int)q;
				if (B[q].Ep == (tz <= 0 ? b->dp + b->dEp : 0) && B[q].En == (tz >= 0 ? b->dn + b->dEn : 0)) bb = (int)q;
			}
			int dup = 0;
			for (size_t q = 0; q < seen.n; q++)
				if (((int *)seen.a)[2 * q] == kb && ((int *)seen.a)[2 * q + 1] == bb) dup = 1;
			if (dup || kb < 0 || bb < 0) continue;
			int pr[2] = { kb, bb };
			tpush(&seen, pr);
			int lo = B[kb].minM > B[bb].minM ? B[kb].minM : B[bb].minM;
			int hi = B[kb].maxM < B[bb].maxM ? B[kb].maxM : B[bb].maxM;
			for (int M = lo; M <= hi; M += 2) {
				double mk = 0, mb = 0;
				for (int64_t s = 0; s < B[kb].n; s++) mk += ((jn_mstate_t *)t.ms.a)[B[kb].first + s].M == M;
				for (int64_t s = 0; s < B[bb].n; s++) mb += ((jn_mstate_t *)t.ms.a)[B[bb].first + s].M == M;
				for (int J = abs(M) / 2; J <= t.jmax && J < p->jt.nJ; J++)
					for (int TT = abs(tz) / 2; TT <= 1; TT++) {
						double n = p->jt.blk_count[2 * J + TT];
						t.dense_flops += 2.0 * (n * n * mk + n * mb * mk);
					}
			}
		}
		free(seen.a);
		(void)T;
	}

	p->n2 = (int)tb.n;
	p->tb = (jn_tblock_t *)tb.a; tb.a = NULL;
	p->tb_info = (int *)tbi.a; tbi.a = NULL;
	p->nelem = nelem;
	p->nms = (int64_t)t.ms.n;
	p->ms = (jn_mstate_t *)t.ms.a; t.ms.a = NULL;
	p->ncoef = (int64_t)t.cs.n;
	p->coef_s = (double *)t.cs.a; t.cs.a = NULL;
	p->coef_a = (int32_t *)t.ca.a; t.ca.a = NULL;
	p->nconn1 = (int64_t)c1.n;
	p->conn_ket = (int32_t *)malloc((c1.n ? c1.n : 1) * sizeof(int32_t));
	p->conn_bra = (int32_t *)malloc((c1.n ? c1.n : 1) * sizeof(int32_t));
	p->conn_sign = (int32_t *)malloc((c1.n ? c1.n : 1) * sizeof(int32_t));
	for (size_t q = 0; q < c1.n; q++) {
		const int32_t *e = (const int32_t *)c1.a + 3 * q;
		p->conn_ket[q] = e[0]; p->conn_bra[q] = e[1]; p->conn_sign[q] = e[2];
	}
	p->npc = (int64_t)pcv.n; p->pc = (jn_pconn_t *)pcv.a; pcv.a = NULL;
	p->nnc = (int64_t)ncv.n; p->nc = (jn_nconn_t *)ncv.a; ncv.a = NULL;
	p->nlut = (int64_t)t.lut.n; p->lut = (int32_t *)t.lut.a; t.lut.a = NULL;
	p->dense_flops = t.dense_flops;
	free(c1.a); free(pairs.a); free(t.jt_index); free(t.bases.a); free(orb);
	bcache_free(&bc);
	return 0;
fail:
	free(rows.a); free(tb.a); free(tbi.a); free(c1.a); free(pcv.a); free(ncv.a); free(pairs.a);
	free(t.jt_index); free(t.bases.a); free(t.ms.a); free(t.cs.a); free(t.ca.a); free(t.lut.a); free(orb);
	bcache_free(&bc);
	jn_tplan_free(p);
	return -1;
}
