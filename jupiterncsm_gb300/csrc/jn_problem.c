/*
 * jn_problem.c — reads the reference's run file, combination table,
 * evaluation order, index lists and matrix-element blocks, validates them,
 * and builds the output-owned device plan described in jn_problem.h.
 *
 * Parsing follows the reference consumers:
 *   bacchus.conf   src/Bacchus/settings/settings.c:79-211 (libconfig keys)
 *   comb.txt       src/Utilities/combination_table/combination_table.c:419-640
 *                  (titles :679-703, id strings "12=" :705-713)
 *   BLOCK rows     src/Minerva/evaluation_order/evaluation_order.c:175-243
 *   index lists    src/Minerva/index_list/index_list.c:69-97
 *   ME blocks      src/Minerva/matrix_block/matrix_block.c:22-62
 * Where the reference calls error() and exits, these functions return a
 * non-zero status and a message.
 */
#define _GNU_SOURCE
#include "jn_problem.h"

#include <ctype.h>
#include <errno.h>
#include <fcntl.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <unistd.h>

#define ERR(...) do { if (err) snprintf(err, errlen, __VA_ARGS__); goto fail; } while (0)

static int split_words(char *s, char **w, int maxw)
{
	int n = 0;
	while (*s && n < maxw) {
		while (*s && isspace((unsigned char)*s)) s++;
		if (!*s) break;
		w[n++] = s;
		while (*s && !isspace((unsigned char)*s)) s++;
		if (*s) *s++ = 0;
	}
	return n;
}

/* "12=" -> 12, digits up to '=' (combination_table.c:705-713) */
static long id_string(const char *s)
{
	long v = 0;
	while (*s && *s != '=') {
		if (*s < '0' || *s > '9') return -1;
		v = 10 * v + (*s++ - '0');
	}
	return v;
}

/* ------------------------------------------------------------------ */
/* run file: the libconfig subset Bacchus uses                          */
/* ------------------------------------------------------------------ */
static char *slurp(const char *path, size_t *len)
{
	FILE *f = fopen(path, "rb");
	if (!f) return NULL;
	fseek(f, 0, SEEK_END);
	long n = ftell(f);
	fseek(f, 0, SEEK_SET);
	char *b = malloc((size_t)n + 1);
	if (!b) { fclose(f); return NULL; }
	size_t got = fread(b, 1, (size_t)n, f);
	fclose(f);
	b[got] = 0;
	if (len) *len = got;
	return b;
}

/* find `key = value;` inside group `group:{ ... }`; returns pointer to value text */
static int rf_lookup(const char *text, const char *group, const char *key, char *out, size_t outlen)
{
	const char *g = text;
	size_t gl = strlen(group), kl = strlen(key);
	while ((g = strstr(g, group)) != NULL) {
		const char *after = g + gl;
		int boundary = (g == text || !(isalnum((unsigned char)g[-1]) || g[-1] == '_'));
		while (*after == ' ' || *after == '\t' || *after == '\n' || *after == '\r') after++;
		if (boundary && (*after == ':' || *after == '=')) {
			const char *open = strchr(after, '{');
			if (!open) return 0;
			int depth = 1;
			const char *p = open + 1;
			const char *end = p;
			while (*end && depth) { if (*end == '{') depth++; else if (*end == '}') depth--; end++; }
			while (p < end) {
				/* skip comments */
				if (*p == '#' || (p[0] == '/' && p[1] == '/')) { while (p < end && *p != '\n') p++; continue; }
				if (!strncmp(p, key, kl) && (p == open + 1 || !(isalnum((unsigned char)p[-1]) || p[-1] == '_')) &&
				    !(isalnum((unsigned char)p[kl]) || p[kl] == '_')) {
					const char *v = p + kl;
					while (*v == ' ' || *v == '\t') v++;
					if (*v != '=' && *v != ':') { p++; continue; }
					v++;
					while (*v == ' ' || *v == '\t') v++;
					size_t i = 0;
					if (*v == '"') {
						v++;
						while (*v && *v != '"' && i + 1 < outlen) out[i++] = *v++;
					} else {
						while (*v && *v != ';' && *v != '\n' && *v != ',' && i + 1 < outlen) out[i++] = *v++;
						while (i && isspace((unsigned char)out[i - 1])) i--;
					}
					out[i] = 0;
					return 1;
				}
				p++;
			}
			return 0;
		}
		g += gl;
	}
	return 0;
}

int jn_read_runfile(const char *path, jn_runfile_t *rf, char *err, size_t errlen)
{
	char v[4096];
	char *text = slurp(path, NULL);
	memset(rf, 0, sizeof *rf);
	if (!text) ERR("could not read run file %s: %s", path, strerror(errno));
#define REQ_STR(grp, key, dst) do { if (!rf_lookup(text, grp, key, v, sizeof v)) ERR("No %s.%s found in \"%s\"", grp, key, path); snprintf(dst, sizeof dst, "%s", v); } while (0)
#define REQ_NUM(grp, key) (rf_lookup(text, grp, key, v, sizeof v) ? 1 : 0)
	REQ_STR("interaction", "combination_table_file", rf->comb);
	REQ_STR("interaction", "evaluation_order_file", rf->order);
	REQ_STR("interaction", "index_lists_base_directory", rf->lists);
	REQ_STR("interaction", "matrix_file_base_directory", rf->mes);
	if (!REQ_NUM("interaction", "num_neutrons")) ERR("No interaction.num_neutrons found in \"%s\"", path);
	rf->N = atoi(v);
	if (!REQ_NUM("interaction", "num_protons")) ERR("No interaction.num_protons found in \"%s\"", path);
	rf->Z = atoi(v);
	REQ_STR("lanczos", "krylow_vector_directory", rf->krylov);
	if (!REQ_NUM("lanczos", "max_num_lanczos_iterations")) ERR("No lanczos.max_num_lanczos_iterations found in \"%s\"", path);
	rf->max_iterations = atol(v);
	if (!REQ_NUM("lanczos", "convergence_tolerance")) ERR("No lanczos.convergence_tolerance found in \"%s\"", path);
	rf->tolerance = atof(v);
	if (!REQ_NUM("lanczos", "target_eigenvector")) ERR("No lanczos.target_eigenvector found in \"%s\"", path);
	rf->target_eigenvector = atol(v);
	rf->converge_eigenvectors = 0;
	if (REQ_NUM("lanczos", "converge_eigenvectors")) rf->converge_eigenvectors = (!strcmp(v, "true") || !strcmp(v, "TRUE"));
	REQ_STR("lanczos", "eigenvector_directory", rf->eigvec);
	/* additive GPU group, ignored by the reference */
	rf->num_eigenvalues = 10;
	rf->precision = 64;
	rf->reorthogonalize = 1;
	if (REQ_NUM("gpu", "num_eigenvalues")) rf->num_eigenvalues = atoi(v);
	if (REQ_NUM("gpu", "precision")) rf->precision = (strstr(v, "32") ? 32 : 64);
	if (REQ_NUM("gpu", "reorthogonalize")) rf->reorthogonalize = !(strstr(v, "partial") || !strcmp(v, "false"));
	free(text);
	return 0;
fail:
	free(text);
	return 1;
}

/* ------------------------------------------------------------------ */
/* combination table                                                   */
/* ------------------------------------------------------------------ */
typedef struct { long id; char type; long length; } listset_t;
typedef struct { long id; long len_comb; } meset_t;

static int is_title(const char *row) { return strstr(row, "***") != NULL; }

typedef struct {
	jn_block_t *b; int nb, cb;
	listset_t *l; int nl, cl;
	meset_t *m; int nm, cm;
} comb_t;

static int read_comb(const char *path, comb_t *c, char *err, size_t errlen)
{
	FILE *f = fopen(path, "r");
	char *line = NULL;
	size_t cap = 0;
	memset(c, 0, sizeof *c);
	if (!f) ERR("Could not open \"%s\". %s", path, strerror(errno));
	int section = 0; /* 1 mp-states, 2 conn lists, 3 cross, 4 same */
	while (getline(&line, &cap, f) >= 0) {
		if (is_title(line)) {
			section = strstr(line, "mp-states") ? 1 : strstr(line, "Conn lists") ? 2 :
				  strstr(line, "Matrix-elements V (cross p-n)") ? 3 :
				  strstr(line, "Matrix-elements V (same p/n)") ? 4 : 0;
			continue;
		}
		char *w[40];
		if (section == 1 && strstr(line, "ARRAYMP:")) {
			int n = split_words(line, w, 40);
			if (n < 10) ERR("malformed mp-states row in %s", path);
			if (c->nb == c->cb) { c->cb = c->cb ? 2 * c->cb : 64; c->b = realloc(c->b, c->cb * sizeof *c->b); }
			jn_block_t *b = &c->b[c->nb++];
			memset(b, 0, sizeof *b);
			b->Ep = atoi(w[0]); b->Mp = atoi(w[1]); b->En = atoi(w[2]); b->Mn = atoi(w[3]);
			b->Np = atoll(w[4]); b->Nn = atoll(w[5]);
			b->id = (int)id_string(w[9]);
			if (b->id <= 0 || b->Np < 0 || b->Nn < 0) ERR("malformed mp-states row in %s", path);
		} else if (section == 2 && strstr(line, "ARRAY:")) {
			int n = split_words(line, w, 40);
			if (n < 10) ERR("malformed Conn lists row in %s", path);
			if (w[0][0] != 'n' && w[0][0] != 'p') ERR("Not a particle type %s", w[0]);
			if (c->nl == c->cl) { c->cl = c->cl ? 2 * c->cl : 256; c->l = realloc(c->l, c->cl * sizeof *c->l); }
			listset_t *l = &c->l[c->nl++];
			l->type = w[0][0]; l->length = atol(w[6]); l->id = id_string(w[9]);
			if (l->id <= 0) ERR("malformed Conn lists row in %s", path);
		} else if ((section == 3 || section == 4) && strstr(line, "ARRAY:")) {
			int n = split_words(line, w, 40);
			int need = section == 3 ? 14 : 9;
			if (n < need) ERR("malformed matrix-element row in %s", path);
			if (c->nm == c->cm) { c->cm = c->cm ? 2 * c->cm : 256; c->m = realloc(c->m, c->cm * sizeof *c->m); }
			meset_t *m = &c->m[c->nm++];
			m->id = id_string(w[section == 3 ? 13 : 8]);
			m->len_comb = section == 3 ? atol(w[8]) * atol(w[9]) : atol(w[4]);
			if (m->id <= 0) ERR("malformed matrix-element row in %s", path);
		}
	}
	free(line);
	fclose(f);
	if (!c->nb) { if (err) snprintf(err, errlen, "no basis blocks in %s", path); return 1; }
	return 0;
fail:
	free(line);
	if (f) fclose(f);
	return 1;
}

/* ------------------------------------------------------------------ */
/* plan                                                                */
/* ------------------------------------------------------------------ */
typedef struct { long *v; long n, cap; } ivec_t;

static int32_t *read_list_file(const char *dir, long id, int64_t *len, char *err, size_t errlen)
{
	char path[8192];
	snprintf(path, sizeof path, "%s/index_list_%ld", dir, id);
	FILE *f = fopen(path, "rb");
	int32_t *d = NULL;
	if (!f) ERR("Could not open file %s. %s", path, strerror(errno));
	fseek(f, 0, SEEK_END);
	long nb = ftell(f);
	fseek(f, 0, SEEK_SET);
	if (nb < 0 || nb % 12) ERR("%s does not hold whole index triples (%ld bytes)", path, nb);
	*len = nb / 12;
	d = malloc(nb ? (size_t)nb : 12);
	if (!d) ERR("out of host memory reading %s", path);
	if ((long)fread(d, 12, (size_t)*len, f) != *len) ERR("Could not read the index_list elements from %s", path);
	fclose(f);
	return d;
fail:
	if (f) fclose(f);
	free(d);
	return NULL;
}

/* one index list per work item */
typedef struct { jn_plan_t *p; const char *dir; uint8_t *bad; } list_job_t;

static void list_read_item(int64_t l, void *v)
{
	const list_job_t *j = (const list_job_t *)v;
	jn_list_t *L = &j->p->lists[l];
	L->triples = read_list_file(j->dir, L->id, &L->len, NULL, 0);
	if (!L->triples) j->bad[l] = 1;
}

/* fn(i, arg) for every i < n, on up to 32 host threads taking items from a
 * shared counter */
typedef struct {
	int64_t n, next;
	void (*fn)(int64_t, void *);
	void *arg;
} par_t;

static void *par_worker(void *v)
{
	par_t *p = (par_t *)v;
	for (;;) {
		const int64_t i = __atomic_fetch_add(&p->next, 1, __ATOMIC_RELAXED);
		if (i >= p->n) break;
		p->fn(i, p->arg);
	}
	return NULL;
}

void jn_par_for(int64_t n, void (*fn)(int64_t, void *), void *arg)
{
	long nt = sysconf(_SC_NPROCESSORS_ONLN);
	const char *cap = getenv("JN_HOST_THREADS");     /* optional cap on the host threads */
	if (cap && atol(cap) > 0 && atol(cap) < nt) nt = atol(cap);
	if (nt > 32) nt = 32;
	if (nt > n) nt = (long)n;          /* no idle threads for short loops */
	if (nt < 1) nt = 1;
	par_t p = { n, 0, fn, arg };
	pthread_t th[32];
	int started = 0;
	for (long t = 1; t < nt; t++)
		if (pthread_create(&th[started], NULL, par_worker, &p) == 0) started++;
	par_worker(&p);
	for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

/* The header of one matrix-element file (two uint64 dimensions, the
 * reference's matrix_block.c:22-62 layout) and its element count, checked
 * against the file's size. */
static int me_file_header(const char *dir, long id, uint64_t *nd_n, uint64_t *nd_p, int64_t *len, char *err,
			  size_t errlen)
{
	char path[8192];
	snprintf(path, sizeof path, "%s/%ld_matrix_elements", dir, id);
	FILE *f = fopen(path, "rb");
	uint64_t hdr[2];
	if (!f) ERR("Could not open block file %s. %s", path, strerror(errno));
	if (fread(hdr, sizeof(uint64_t), 2, f) != 2) ERR("Could not read dimensions from matrix file %ld", id);
	*nd_n = hdr[0]; *nd_p = hdr[1];
	uint64_t n = hdr[0] == 0 ? hdr[1] : hdr[1] == 0 ? hdr[0] : hdr[0] * hdr[1];
	if (hdr[0] && hdr[1] && n / hdr[0] != hdr[1]) ERR("matrix file %ld: dimension overflow", id);
	if (n > ((uint64_t)1 << 56)) ERR("matrix file %ld: dimension overflow", id);
	if (fseeko(f, 0, SEEK_END) != 0) ERR("Could not read matrix elements form matrix file %ld", id);
	off_t fsz = ftello(f);
	if (fsz < 0 || (uint64_t)fsz < 16 + 8 * n) ERR("Could not read matrix elements form matrix file %ld", id);
	fclose(f);
	*len = (int64_t)n;
	return 0;
fail:
	if (f) fclose(f);
	return 1;
}

/* Every block's elements, read by all host cores straight into out + offset:
 * work items are pieces of at most ME_READ_CHUNK elements of one file. */
#define ME_READ_CHUNK ((int64_t)1 << 22)

typedef struct { int b; int64_t e0, e1; } me_piece_t;

typedef struct {
	const jn_plan_t *p;
	const char *dir;
	double *out;
	const me_piece_t *pc;
	uint8_t *bad;
} me_read_t;

static void me_read_piece(int64_t i, void *v)
{
	me_read_t *r = (me_read_t *)v;
	const me_piece_t *pc = &r->pc[i];
	const jn_me_t *M = &r->p->mes[pc->b];
	char path[8192];
	snprintf(path, sizeof path, "%s/%d_matrix_elements", r->dir, M->id);
	int fd = open(path, O_RDONLY);
	if (fd < 0) { r->bad[i] = 1; return; }
	char *dst = (char *)(r->out + M->offset + pc->e0);
	size_t want = (size_t)(pc->e1 - pc->e0) * sizeof(double);
	off_t at = 16 + (off_t)pc->e0 * (off_t)sizeof(double);
	while (want > 0) {
		ssize_t got = pread(fd, dst, want, at);
		if (got < 0 && errno == EINTR) continue;
		if (got <= 0) { r->bad[i] = 1; break; }
		dst += got; at += got; want -= (size_t)got;
	}
	close(fd);
}

static int me_read_all(const jn_plan_t *p, const char *dir, double *out, char *err, size_t errlen)
{
	int64_t n = 0;
	for (int b = 0; b < p->nmes; b++) n += (p->mes[b].len + ME_READ_CHUNK - 1) / ME_READ_CHUNK;
	me_piece_t *pc = malloc((n ? n : 1) * sizeof *pc);
	uint8_t *bad = calloc(n ? n : 1, 1);
	if (!pc || !bad) {
		free(pc); free(bad);
		if (err) snprintf(err, errlen, "out of host memory reading %s", dir);
		return 1;
	}
	n = 0;
	for (int b = 0; b < p->nmes; b++)
		for (int64_t e = 0; e < p->mes[b].len; e += ME_READ_CHUNK) {
			pc[n].b = b; pc[n].e0 = e;
			pc[n].e1 = e + ME_READ_CHUNK < p->mes[b].len ? e + ME_READ_CHUNK : p->mes[b].len;
			n++;
		}
	me_read_t r = { p, dir, out, pc, bad };
	jn_par_for(n, me_read_piece, &r);
	int rc = 0;
	for (int64_t i = 0; i < n && !rc; i++)
		if (bad[i]) {
			if (err) snprintf(err, errlen, "Could not read matrix elements form matrix file %d", p->mes[pc[i].b].id);
			rc = 1;
		}
	free(pc); free(bad);
	return rc;
}

int jn_plan_read_me(const jn_plan_t *p, const char *dir, double *out, char *err, size_t errlen)
{
	for (int b = 0; b < p->nmes; b++) {
		const jn_me_t *M = &p->mes[b];
		uint64_t nd_n, nd_p;
		int64_t len;
		if (me_file_header(dir, M->id, &nd_n, &nd_p, &len, err, errlen)) return 1;
		if (nd_n != M->nd_n || nd_p != M->nd_p || len != M->len) {
			if (err) snprintf(err, errlen, "matrix file %d in %s has dimensions (%llu, %llu), the plan (%llu, %llu)", M->id,
					  dir, (unsigned long long)nd_n, (unsigned long long)nd_p, (unsigned long long)M->nd_n,
					  (unsigned long long)M->nd_p);
			return 1;
		}
	}
	return me_read_all(p, dir, out, err, errlen);
}

static int build_csr(const int32_t *tri, int64_t len, int32_t nrows, int by_out, uint32_t *rowptr, uint32_t *ent)
{
	/* stable counting sort on the destination index; entries (source | destination << 16, matrix_index) */
	memset(rowptr, 0, (size_t)(nrows + 1) * sizeof(uint32_t));
	for (int64_t e = 0; e < len; e++) rowptr[(by_out ? tri[3 * e + 1] : tri[3 * e]) + 1]++;
	for (int32_t r = 0; r < nrows; r++) rowptr[r + 1] += rowptr[r];
	uint32_t *fill = malloc((size_t)(nrows + 1) * sizeof(uint32_t));
	if (!fill) return 1;
	memcpy(fill, rowptr, (size_t)(nrows + 1) * sizeof(uint32_t));
	for (int64_t e = 0; e < len; e++) {
		int32_t dst = by_out ? tri[3 * e + 1] : tri[3 * e];
		uint32_t at = fill[dst]++;
		/* source index in the low half, destination in the high half, in both views */
		ent[2 * at] = by_out ? ((uint32_t)tri[3 * e] | ((uint32_t)tri[3 * e + 1] << 16))
				     : ((uint32_t)tri[3 * e + 1] | ((uint32_t)tri[3 * e] << 16));
		ent[2 * at + 1] = (uint32_t)tri[3 * e + 2];
	}
	free(fill);
	return 0;
}

/* both CSR views of one list, with absolute entry indices; lists write
 * disjoint parts of rowptr and ent, so all host cores build them */
typedef struct { jn_plan_t *p; uint8_t *bad; } csr_job_t;

static void csr_list(int64_t l, void *v)
{
	const csr_job_t *j = (const csr_job_t *)v;
	jn_plan_t *p = j->p;
	jn_list_t *L = &p->lists[l];
	if (build_csr(L->triples, L->len, L->nout, 1, p->rowptr + L->csr_out_ptr, p->ent + 2 * L->ent_out) ||
	    build_csr(L->triples, L->len, L->nin, 0, p->rowptr + L->csr_in_ptr, p->ent + 2 * L->ent_in)) {
		j->bad[l] = 1;
		return;
	}
	/* the CSR row pointers are list-local: make them absolute entry indices */
	for (int32_t r = 0; r <= L->nout; r++) p->rowptr[L->csr_out_ptr + r] += (uint32_t)L->ent_out;
	for (int32_t r = 0; r <= L->nin; r++) p->rowptr[L->csr_in_ptr + r] += (uint32_t)L->ent_in;
}

void jn_plan_free(jn_plan_t *p)
{
	if (!p) return;
	free(p->blocks);
	free(p->instr);
	for (int i = 0; i < p->nlists; i++) free(p->lists[i].triples);
	free(p->lists);
	free(p->mes);
	free(p->rowptr); free(p->ent); free(p->me);
	free(p->terms); free(p->tiles); free(p->units); free(p->unit_terms);
	free(p->btiles); free(p->pieces); free(p->tterms); free(p->walks); free(p->items);
	free(p->term_dst);
	jn_panels_free(p);
	jn_walk_free(p);
	memset(p, 0, sizeof *p);
}

/* max |M| of every matrix-element block (1 for each when me is NULL), one
 * block per work item on all host cores.  A comparison skips NaN as fmax
 * does, without fmax's library call per element. */
typedef struct { const jn_plan_t *p; const double *me; double *m; } bmax_t;

static void block_max_item(int64_t b, void *v)
{
	const bmax_t *j = (const bmax_t *)v;
	const jn_me_t *M = &j->p->mes[b];
	const double *a = j->me + M->offset;
	double m = 0.0;
	for (int64_t e = 0; e < M->len; e++) {
		const double x = fabs(a[e]);
		if (x > m) m = x;
	}
	j->m[b] = m;
}

static double *block_max(const jn_plan_t *p, const double *me)
{
	double *m = calloc(p->nmes ? p->nmes : 1, sizeof(double));
	if (!m) return NULL;
	if (!me) {
		for (int b = 0; b < p->nmes; b++) m[b] = 1.0;
		return m;
	}
	bmax_t j = { p, me, m };
	jn_par_for(p->nmes, block_max_item, &j);
	return m;
}

double jn_plan_abs_bound(const jn_plan_t *p, const double *me)
{
	const uint32_t *rp = p->rowptr;
	double *tmax = calloc(p->nterms ? p->nterms : 1, sizeof(double));
	double *mmax = block_max(p, me);            /* once per block, not once per term */
	if (!tmax || !mmax) {
		free(tmax); free(mmax);
		return INFINITY;
	}
	for (int t = 0; t < p->nterms; t++) tmax[t] = mmax[p->instr[p->terms[t].instr].me];
	free(mmax);
	/* terms grouped by destination block */
	int *cnt = calloc((size_t)p->nblocks + 1, sizeof(int));
	int *byb = malloc((p->nterms > 0 ? (size_t)p->nterms : 1) * sizeof(int));
	for (int t = 0; t < p->nterms; t++) cnt[p->term_dst[t] + 1]++;
	for (int b = 0; b < p->nblocks; b++) cnt[b + 1] += cnt[b];
	int *fl = malloc((p->nblocks + 1) * sizeof(int));
	memcpy(fl, cnt, (p->nblocks + 1) * sizeof(int));
	for (int t = 0; t < p->nterms; t++) byb[fl[p->term_dst[t]]++] = t;
	free(fl);
	double best = 0, *bound = NULL;
	size_t bcap = 0;
	for (int b = 0; b < p->nblocks; b++) {
		const jn_block_t *B = &p->blocks[b];
		size_t E = (size_t)(B->Np * B->Nn);
		if (!E) continue;
		if (E > bcap) { bcap = E; bound = realloc(bound, bcap * sizeof(double)); }
		memset(bound, 0, E * sizeof(double));
		for (int q = cnt[b]; q < cnt[b + 1]; q++) {
			const int t = byb[q];
			const jn_term_t *T = &p->terms[t];
			for (int64_t r = 0; r < B->Np; r++) {
				double np = T->kind == JN_KIND_N ? 1.0 : (double)(rp[T->p_ptr + r + 1] - rp[T->p_ptr + r]);
				if (np == 0) continue;
				for (int64_t c = 0; c < B->Nn; c++) {
					double nn = T->kind == JN_KIND_P ? 1.0 : (double)(rp[T->n_ptr + c + 1] - rp[T->n_ptr + c]);
					bound[r * B->Nn + c] += np * nn * tmax[t];
				}
			}
		}
		for (size_t e = 0; e < E; e++) best = fmax(best, bound[e]);
	}
	free(bound); free(tmax); free(cnt); free(byb);
	return best;
}

/* warp pieces: R rows x W columns of one destination block, R*W <= 32 */
#define PIECE_LANES 32

/* estimated warp time of term t on the piece rows [r0,r1) x cols [c0,c1):
 * every lane owns one element, so the warp runs as long as its longest
 * lane.  Zero when the term contributes nothing to the piece. */
static double term_cost(const jn_plan_t *p, const jn_term_t *t, int r0, int r1, int c0, int c1)
{
	const uint32_t *rp = p->rowptr;
	double np = 0, nn = 0, npmax = 0, nnmax = 0;
	if (t->kind != JN_KIND_N) {
		for (int r = r0; r < r1; r++) {
			double v = rp[t->p_ptr + r + 1] - rp[t->p_ptr + r];
			np += v;
			if (v > npmax) npmax = v;
		}
		if (np == 0) return 0;
	}
	if (t->kind != JN_KIND_P) {
		for (int c = c0; c < c1; c++) {
			double v = rp[t->n_ptr + c + 1] - rp[t->n_ptr + c];
			nn += v;
			if (v > nnmax) nnmax = v;
		}
		if (nn == 0) return 0;
	}
	if (t->kind == JN_KIND_P) return 4.0 + npmax;
	if (t->kind == JN_KIND_N) return 4.0 + nnmax;
	return 4.0 + npmax * (1.0 + nnmax);
}

/* indices by cost, heaviest first, ties by index (qsort_r: the costs come
 * with the call, so concurrent plan builds share no state) */
static int cmp_cost_desc(const void *a, const void *b, void *cost)
{
	const double *c = (const double *)cost;
	double x = c[*(const int *)a], y = c[*(const int *)b];
	if (x != y) return x < y ? 1 : -1;
	return *(const int *)a - *(const int *)b;
}

/* shared-memory accumulator budget of one CTA, in 64-bit elements */
#define TILE_SMEM_ELEMS 8192
/* work of one lane in one task, at most (multiply-adds plus per-output cost) */
#define LANE_VISITS 96
/* fixed per-task cost in the work model, in multiply-add units */
#define TASK_OVERHEAD 6.0

typedef struct { jn_piece_t t; double cost; } task_cost_t;

static int cmp_task_cost(const void *a, const void *b)
{
	const task_cost_t *x = a, *y = b;
	if (x->cost != y->cost) return x->cost < y->cost ? 1 : -1;
	if (x->t.head != y->t.head) return x->t.head < y->t.head ? -1 : 1;
	if (x->t.lane_base != y->t.lane_base) return x->t.lane_base < y->t.lane_base ? -1 : 1;
	return x->t.loop_base < y->t.loop_base ? -1 : (x->t.loop_base > y->t.loop_base);
}

/*
 * Block tiles and warp tasks.  Every destination block is cut into row
 * ranges whose accumulator fits in shared memory.  Each term touching a
 * range becomes warp tasks in the orientation that keeps more lanes busy:
 *   NP  lanes over the neutron entries, each walking Pout(row) for one row
 *       (EN), or lanes over the proton entries, each walking Nout(col) for
 *       one column (EP);
 *   P   lanes over columns, walking Pout(row) (PC);
 *   N   lanes over rows, walking Nout(col) (NR).
 * Tasks are packed into tiles of similar work, longest first.  Also computes
 * abs_bound, the largest sum of |M| over the contributions to one element,
 * which bounds |y| by abs_bound * max|x| for the fixed-point scale.
 */
/* the first walk in [lo, hi) whose destination row is at least `row`; a
 * view's walks are stored in ascending destination-row order */
static int64_t first_walk_from(const uint32_t *W, int64_t lo, int64_t hi, uint32_t row)
{
	while (lo < hi) {
		const int64_t m = lo + (hi - lo) / 2;
		if ((W[2 * m + 1] >> 16) < row) lo = m + 1;
		else hi = m;
	}
	return lo;
}

/* The first pass of the block-tile plan for one destination block: its
 * |M| bound, its row ranges and their warp tasks with their costs.  Blocks
 * are independent, so all host cores build them; the caller concatenates
 * them in block order. */
typedef struct { int b; int64_t r0, r1; int64_t t0, t1; double cost; } tile_range_t;

typedef struct {
	tile_range_t *ranges;
	int nranges;
	task_cost_t *tasks;
	int64_t ntasks;
	double abs_bound;       /* largest bound of the block's elements */
	int max_el;             /* largest tile of the block, in shared-memory elements */
	int status;             /* 1: out of host memory; 2: a row wider than a shared-memory tile */
} blk_tiles_t;

typedef struct {
	const jn_plan_t *p;
	const int *cnt, *byb;
	const double *tmax;
	blk_tiles_t *out;
} tiles_job_t;

static void tiles_block(int64_t bi, void *v)
{
	const tiles_job_t *J = (const tiles_job_t *)v;
	const jn_plan_t *p = J->p;
	const int b = (int)bi;
	const jn_block_t *B = &p->blocks[b];
	blk_tiles_t *o = &J->out[b];
	const uint32_t *rp = p->rowptr;
	const int *cnt = J->cnt, *byb = J->byb;
	const double *tmax = J->tmax;
	if (B->Np == 0 || B->Nn == 0) return;
	const int64_t stride = B->Nn | 1;
	/* |M| bound per element of this block (needed by every engine, tiles or not) */
	const size_t E = (size_t)(B->Np * B->Nn);
	double *bound = calloc(E ? E : 1, sizeof(double));
	if (!bound) { o->status = 1; return; }
	for (int q = cnt[b]; q < cnt[b + 1]; q++) {
		const jn_term_t *T = &p->terms[byb[q]];
		for (int64_t r = 0; r < B->Np; r++) {
			double np = T->kind == JN_KIND_N ? 1.0 : (double)(rp[T->p_ptr + r + 1] - rp[T->p_ptr + r]);
			if (np == 0) continue;
			for (int64_t c = 0; c < B->Nn; c++) {
				double nn = T->kind == JN_KIND_P ? 1.0 : (double)(rp[T->n_ptr + c + 1] - rp[T->n_ptr + c]);
				bound[r * B->Nn + c] += np * nn * tmax[byb[q]];
			}
		}
	}
	for (size_t e = 0; e < E; e++) o->abs_bound = fmax(o->abs_bound, bound[e]);
	free(bound);
	if (stride > TILE_SMEM_ELEMS) { o->status = 2; return; }
	int64_t tcap = 0;
	int rcap = 0;
#define PUSH_TASK(TERM, KIND, COUNT, LANE_BASE, LOOP_BASE, LOOP_LEN, COST)                     \
	do {                                                                                   \
		if (o->ntasks == tcap) {                                                       \
			const int64_t nc_ = tcap ? 2 * tcap : 4096;                            \
			task_cost_t *g_ = realloc(o->tasks, (size_t)nc_ * sizeof *g_);         \
			if (!g_) { o->status = 1; return; }                                    \
			o->tasks = g_;                                                         \
			tcap = nc_;                                                            \
		}                                                                              \
		task_cost_t *q_ = &o->tasks[o->ntasks++];                                      \
		q_->t.head = (uint32_t)(TERM) | ((uint32_t)(KIND) << 24) | ((uint32_t)((COUNT) - 1) << 27); \
		q_->t.lane_base = (uint32_t)(LANE_BASE); q_->t.loop_base = (uint32_t)(LOOP_BASE); \
		q_->t.loop_len = (uint32_t)(LOOP_LEN);                                         \
		q_->cost = TASK_OVERHEAD + (COST);                                             \
	} while (0)
	const int64_t R = TILE_SMEM_ELEMS / stride;
	for (int64_t r0 = 0; r0 < B->Np; r0 += R) {
		const int64_t r1 = r0 + R < B->Np ? r0 + R : B->Np;
		if (o->nranges == rcap) {
			const int nc = rcap ? 2 * rcap : 16;
			tile_range_t *g = realloc(o->ranges, (size_t)nc * sizeof *g);
			if (!g) { o->status = 1; return; }
			o->ranges = g;
			rcap = nc;
		}
		tile_range_t *rg = &o->ranges[o->nranges++];
		rg->b = b; rg->r0 = r0; rg->r1 = r1; rg->t0 = o->ntasks;
		for (int q = cnt[b]; q < cnt[b + 1]; q++) {
			const int ti = byb[q];
			const jn_term_t *T = &p->terms[ti];
			const uint32_t *W = p->walks;
			/* P-walks with destination rows in [r0, r1) */
			int64_t pa = T->pw0, pb = T->pw0;
			if (T->kind != JN_KIND_N) {
				pa = first_walk_from(W, T->pw0, T->pw1, (uint32_t)r0);
				pb = first_walk_from(W, pa, T->pw1, (uint32_t)r1);
			}
			const int64_t nR = pb - pa, nC = T->nw1 - T->nw0;
			int lanes_on_n;
			int64_t lane0, nlane, loop0, nloop;
			int kind;
			if (T->kind == JN_KIND_NP) {
				if (!nR || !nC) continue;
				lanes_on_n = nC >= nR;
				kind = lanes_on_n ? JN_TASK_NP_A : JN_TASK_NP_B;
				lane0 = lanes_on_n ? T->nw0 : pa; nlane = lanes_on_n ? nC : nR;
				loop0 = lanes_on_n ? pa : T->nw0; nloop = lanes_on_n ? nR : nC;
			} else if (T->kind == JN_KIND_P) {
				if (!nR) continue;
				lanes_on_n = B->Nn >= nR;          /* lanes over columns */
				kind = lanes_on_n ? JN_TASK_P_A : JN_TASK_P_B;
				lane0 = lanes_on_n ? 0 : pa; nlane = lanes_on_n ? B->Nn : nR;
				loop0 = lanes_on_n ? pa : 0; nloop = lanes_on_n ? nR : B->Nn;
			} else {
				if (!nC) continue;
				lanes_on_n = nC >= r1 - r0;         /* lanes over N-walks */
				kind = lanes_on_n ? JN_TASK_N_A : JN_TASK_N_B;
				lane0 = lanes_on_n ? T->nw0 : r0; nlane = lanes_on_n ? nC : r1 - r0;
				loop0 = lanes_on_n ? r0 : T->nw0; nloop = lanes_on_n ? r1 - r0 : nC;
			}
			/* walk lengths (1 for a dense column or row) of the two sides */
#define LANE_LEN(i) ((kind == JN_TASK_P_A || kind == JN_TASK_N_B) ? 1.0 : (double)(W[2 * (i) + 1] & 0xffff))
#define LOOP_LEN(i) ((kind == JN_TASK_P_B || kind == JN_TASK_N_A) ? 1.0 : (double)(W[2 * (i) + 1] & 0xffff))
			for (int64_t l0 = 0; l0 < nlane; l0 += 32) {
				const int64_t cntl = nlane - l0 < 32 ? nlane - l0 : 32;
				double lane_max = 0;
				for (int64_t i = 0; i < cntl; i++) lane_max = fmax(lane_max, LANE_LEN(lane0 + l0 + i));
				/* split the loop so that one task stays short */
				int64_t s0 = 0;
				double acc = 0;
				for (int64_t sI = 0; sI < nloop; sI++) {
					acc += LOOP_LEN(loop0 + sI) * lane_max + 4.0;
					if (acc >= LANE_VISITS || sI == nloop - 1) {
						PUSH_TASK(ti, kind, cntl, lane0 + l0, loop0 + s0, sI + 1 - s0, acc);
						s0 = sI + 1;
						acc = 0;
					}
				}
			}
#undef LANE_LEN
#undef LOOP_LEN
		}
		rg->t1 = o->ntasks;
		const int64_t el = (r1 - r0) * stride;
		if (el > o->max_el) o->max_el = (int)el;
	}
#undef PUSH_TASK
}

/* compact term descriptions read by the tile kernel */
static int build_tterms(jn_plan_t *p, char *err, size_t errlen)
{
	p->tterms = calloc(p->nterms ? p->nterms : 1, sizeof(jn_tterm_t));
	if (!p->tterms) {
		if (err) snprintf(err, errlen, "out of host memory");
		return 1;
	}
	for (int t = 0; t < p->nterms; t++) {
		const jn_term_t *T = &p->terms[t];
		if (T->src_off > 0x7fffffffll) {
			if (err) snprintf(err, errlen, "vector too long for 32-bit block offsets");
			return 1;
		}
		p->tterms[t].me_off = T->me_off;
		p->tterms[t].src_off = (int32_t)T->src_off;
		p->tterms[t].nd = T->nd;
		p->tterms[t].Nn_src = T->Nn_src;
		p->tterms[t].transpose = T->transpose;
	}
	return 0;
}

/* The second pass for one row range: its tiles of similar work and their
 * warp items.  Every task becomes one piece at its own task index, so
 * ranges (disjoint task runs) are built on all host cores; tile item ranges
 * are local to the range until the caller joins them. */
typedef struct { uint32_t first, width_n; double cost; } tile_item_t;

typedef struct {
	jn_btile_t *tiles;
	double *tile_cost;
	int ntiles;
	uint32_t *items;        /* pairs {first piece, width | pieces << 8} */
	int64_t nitems;
	int status;             /* 1: out of host memory */
} range_tiles_t;

typedef struct {
	jn_plan_t *p;
	const tile_range_t *ranges;
	task_cost_t *tasks;
	double tile_target;
	range_tiles_t *out;
} pass2_job_t;

static void tiles_range(int64_t ri, void *v)
{
	const pass2_job_t *J = (const pass2_job_t *)v;
	jn_plan_t *p = J->p;
	const tile_range_t *rg = &J->ranges[ri];
	const jn_block_t *B = &p->blocks[rg->b];
	task_cost_t *tasks = J->tasks;
	range_tiles_t *o = &J->out[ri];
	const int64_t nall = rg->t1 - rg->t0;
	tile_item_t *items = malloc((nall ? nall : 1) * sizeof *items);
	o->items = malloc((nall ? nall : 1) * 2 * sizeof(uint32_t));
	if (!items || !o->items) { free(items); o->status = 1; return; }
	int tcap = 0;
	int nt = (int)ceil(rg->cost / J->tile_target);
	if (nt < 1) nt = 1;
	double per = rg->cost / nt, acc = 0;
	int64_t begin = rg->t0;
	for (int64_t k = rg->t0; k < rg->t1; k++) {
		acc += tasks[k].cost;
		if (!(acc >= per || k == rg->t1 - 1)) continue;
		if (o->ntiles == tcap) {
			const int nc = tcap ? 2 * tcap : 8;
			jn_btile_t *g = realloc(o->tiles, (size_t)nc * sizeof *g);
			if (g) o->tiles = g;
			double *gc = realloc(o->tile_cost, (size_t)nc * sizeof *gc);
			if (gc) o->tile_cost = gc;
			if (!g || !gc) { free(items); o->status = 1; return; }
			tcap = nc;
		}
		jn_btile_t *Tl = &o->tiles[o->ntiles];
		Tl->dst_off = B->offset; Tl->Nn = (int32_t)B->Nn; Tl->row0 = (int32_t)rg->r0;
		Tl->nrows = (int32_t)(rg->r1 - rg->r0); Tl->stride = (int32_t)(B->Nn | 1);
		/* group by (kind, width), heaviest first inside a group */
		int64_t n = k + 1 - begin;
		for (int64_t q = begin; q <= k; q++) {
			uint32_t c = JN_TASK_COUNT(tasks[q].t.head);
			uint32_t w = c <= 8 ? 8 : c <= 16 ? 16 : 32;
			/* sort key: kind, width, then cost */
			tasks[q].cost += 1e12 * (double)(JN_TASK_KIND(tasks[q].t.head) * 4 + (w >> 3));
		}
		qsort(tasks + begin, n, sizeof *tasks, cmp_task_cost);
		int64_t nitems = 0;
		double tcost = 0;
		for (int64_t q = begin; q <= k;) {
			const uint32_t kind = JN_TASK_KIND(tasks[q].t.head);
			const uint32_t c = JN_TASK_COUNT(tasks[q].t.head);
			const uint32_t w = c <= 8 ? 8 : c <= 16 ? 16 : 32, per_item = 32 / w;
			tile_item_t *it = &items[nitems++];
			it->first = (uint32_t)q;
			it->cost = 0;
			uint32_t m = 0;
			while (q <= k && m < per_item && JN_TASK_KIND(tasks[q].t.head) == kind &&
			       (JN_TASK_COUNT(tasks[q].t.head) <= 8 ? 8u : JN_TASK_COUNT(tasks[q].t.head) <= 16 ? 16u : 32u) == w) {
				double cst = fmod(tasks[q].cost, 1e12);
				if (cst > it->cost) it->cost = cst;
				p->pieces[q] = tasks[q].t;
				q++;
				m++;
			}
			it->width_n = w | (m << 8);
			tcost += it->cost;
		}
		/* heaviest items first for the warps' dynamic fetch */
		for (int64_t i = 1; i < nitems; i++) {
			tile_item_t t = items[i];
			int64_t j = i - 1;
			while (j >= 0 && items[j].cost < t.cost) { items[j + 1] = items[j]; j--; }
			items[j + 1] = t;
		}
		Tl->pc0 = o->nitems;
		for (int64_t i = 0; i < nitems; i++) {
			o->items[2 * o->nitems] = items[i].first;
			o->items[2 * o->nitems + 1] = items[i].width_n;
			o->nitems++;
		}
		Tl->pc1 = o->nitems;
		o->tile_cost[o->ntiles++] = tcost;
		begin = k + 1;
		acc = 0;
	}
	free(items);
}

static int build_block_tiles(jn_plan_t *p, const int *term_dst, int target_units, char *err, size_t errlen)
{
	double *tmax = calloc(p->nterms ? p->nterms : 1, sizeof(double));
	double *mmax = block_max(p, p->me);         /* once per block, not once per term */
	if (!tmax || !mmax) {
		free(tmax); free(mmax);
		if (err) snprintf(err, errlen, "out of host memory");
		return 1;
	}
	for (int t = 0; t < p->nterms; t++) tmax[t] = mmax[p->instr[p->terms[t].instr].me];
	free(mmax);
	int *cnt = calloc(p->nblocks + 1, sizeof(int));
	for (int t = 0; t < p->nterms; t++) cnt[term_dst[t] + 1]++;
	for (int b = 0; b < p->nblocks; b++) cnt[b + 1] += cnt[b];
	int *byb = malloc((p->nterms ? p->nterms : 1) * sizeof(int)), *fl = malloc((p->nblocks + 1) * sizeof(int));
	memcpy(fl, cnt, (p->nblocks + 1) * sizeof(int));
	for (int t = 0; t < p->nterms; t++) byb[fl[term_dst[t]]++] = t;
	free(fl);
	/* pass 1: tasks of every (block, row range), with their costs, built per
	   block on all host cores and concatenated in block order; the running
	   cost total is summed in that order */
	blk_tiles_t *bt = calloc(p->nblocks ? p->nblocks : 1, sizeof *bt);
	if (!bt) {
		free(tmax); free(cnt); free(byb);
		if (err) snprintf(err, errlen, "out of host memory");
		return 1;
	}
	tiles_job_t job = { p, cnt, byb, tmax, bt };
	jn_par_for(p->nblocks, tiles_block, &job);
	int64_t ntasks = 0;
	int nranges = 0, status = 0, wide = -1;
	for (int b = 0; b < p->nblocks; b++) {
		if (bt[b].status == 1) status = 1;
		if (bt[b].status == 2 && wide < 0) wide = b;
		ntasks += bt[b].ntasks;
		nranges += bt[b].nranges;
	}
	if (wide >= 0 && !status) {
		/* a block row wider than one shared-memory tile: no block tiles, so
		   engine 3 (and what runs on it) is unavailable for this plan; the
		   bound and the term descriptions, which other engines use, are built */
		p->abs_bound = 0;
		for (int b = 0; b < p->nblocks; b++) {
			p->abs_bound = fmax(p->abs_bound, bt[b].abs_bound);
			free(bt[b].tasks); free(bt[b].ranges);
		}
		free(bt); free(tmax); free(cnt); free(byb);
		p->max_tile_elems = 0;
		p->btiles_off = 1;
		snprintf(p->btiles_why, sizeof p->btiles_why,
			 "basis block %d has %lld neutron states: more than one shared-memory row of the block-tile engine (%d)",
			 p->blocks[wide].id, (long long)p->blocks[wide].Nn, TILE_SMEM_ELEMS - 1);
		return build_tterms(p, err, errlen);
	}
	tile_range_t *ranges = status ? NULL : malloc((nranges ? nranges : 1) * sizeof *ranges);
	task_cost_t *tasks = status ? NULL : malloc((ntasks ? ntasks : 1) * sizeof *tasks);
	if (!status && (!ranges || !tasks)) status = 1;
	if (status) {
		for (int b = 0; b < p->nblocks; b++) { free(bt[b].tasks); free(bt[b].ranges); }
		free(bt); free(tmax); free(cnt); free(byb); free(tasks); free(ranges);
		if (err) snprintf(err, errlen, "out of host memory");
		return 1;
	}
	double total = 0;
	p->max_tile_elems = 0;
	p->abs_bound = 0;
	ntasks = 0;
	nranges = 0;
	for (int b = 0; b < p->nblocks; b++) {
		p->abs_bound = fmax(p->abs_bound, bt[b].abs_bound);
		if (bt[b].max_el > p->max_tile_elems) p->max_tile_elems = bt[b].max_el;
		for (int k = 0; k < bt[b].nranges; k++) {
			tile_range_t rg = bt[b].ranges[k];
			const double before = total;
			const int64_t t0 = ntasks;
			for (int64_t i = rg.t0; i < rg.t1; i++) {
				tasks[ntasks] = bt[b].tasks[i];
				total += tasks[ntasks++].cost;
			}
			rg.t0 = t0;
			rg.t1 = ntasks;
			rg.cost = total - before;
			ranges[nranges++] = rg;
		}
		free(bt[b].tasks); free(bt[b].ranges);
	}
	free(bt);
	if (p->nterms >= (1 << 24)) {
		free(tmax); free(cnt); free(byb); free(tasks); free(ranges);
		if (err) snprintf(err, errlen, "too many terms for the packed task format");
		return 1;
	}
	if (build_tterms(p, err, errlen)) {
		free(tmax); free(cnt); free(byb); free(tasks); free(ranges);
		return 1;
	}
	/* pass 2: tiles of similar work.  Inside a tile, tasks of one kind and
	 * similar width are packed into warp items (one task per 8, 16 or 32
	 * lanes), heaviest items first; tiles are ordered heaviest first too. */
	int ntile_target = target_units > 0 ? target_units / 2 : 152 * 24;
	if (ntile_target < 1) ntile_target = 1;
	double tile_target = total / ntile_target;
	if (tile_target < 64 * 32) tile_target = 64 * 32;
	p->pieces = malloc((ntasks ? ntasks : 1) * sizeof(jn_piece_t));
	p->items = malloc((ntasks ? ntasks : 1) * 2 * sizeof(uint32_t));
	range_tiles_t *rt = calloc(nranges ? nranges : 1, sizeof *rt);
	int ntl = 0;
	status = !p->pieces || !p->items || !rt;
	if (!status) {
		pass2_job_t job2 = { p, ranges, tasks, tile_target, rt };
		jn_par_for(nranges, tiles_range, &job2);
		for (int ri = 0; ri < nranges; ri++) {
			status |= rt[ri].status;
			ntl += rt[ri].ntiles;
		}
	}
	jn_btile_t *tiles = status ? NULL : malloc((ntl ? ntl : 1) * sizeof(jn_btile_t));
	double *tile_cost = status ? NULL : malloc((ntl ? ntl : 1) * sizeof(double));
	if (!status && (!tiles || !tile_cost)) status = 1;
	if (status) {
		if (rt)
			for (int ri = 0; ri < nranges; ri++) { free(rt[ri].tiles); free(rt[ri].tile_cost); free(rt[ri].items); }
		free(rt); free(tiles); free(tile_cost);
		free(tmax); free(cnt); free(byb); free(tasks); free(ranges);
		if (err) snprintf(err, errlen, "out of host memory");
		return 1;
	}
	/* every task is one piece, in task order; items and tiles are joined in range order */
	p->npieces = ntasks;
	p->nitems = 0;
	ntl = 0;
	for (int ri = 0; ri < nranges; ri++) {
		const range_tiles_t *o = &rt[ri];
		for (int i = 0; i < o->ntiles; i++) {
			tiles[ntl] = o->tiles[i];
			tiles[ntl].pc0 += p->nitems;
			tiles[ntl].pc1 += p->nitems;
			tile_cost[ntl++] = o->tile_cost[i];
		}
		memcpy(p->items + 2 * p->nitems, o->items, (size_t)o->nitems * 2 * sizeof(uint32_t));
		p->nitems += o->nitems;
		free(o->tiles); free(o->tile_cost); free(o->items);
	}
	free(rt);
	/* tiles heaviest first: persistent CTAs fetch them in this order */
	{
		int *ord = malloc((ntl ? ntl : 1) * sizeof(int));
		for (int i = 0; i < ntl; i++) ord[i] = i;
		qsort_r(ord, ntl, sizeof(int), cmp_cost_desc, tile_cost);
		p->btiles = malloc((ntl ? ntl : 1) * sizeof(jn_btile_t));
		for (int i = 0; i < ntl; i++) p->btiles[i] = tiles[ord[i]];
		p->nbtiles = ntl;
		free(ord);
	}
	free(tiles); free(tile_cost);
	free(tmax); free(cnt); free(byb); free(tasks); free(ranges);
	return 0;
}

/* Engine 2's plan: output tiles of 32 columns, their chunks of terms
 * (work units) and the chunk partial-sum layout, longest units first.  Built
 * when engine 2 is selected (jn_set_engine), not at open. */
int jn_plan_build_units(jn_plan_t *p, int target_units, char *err, size_t errlen)
{
	if (p->units) return 0;
	const int *term_dst = p->term_dst;
	/* terms grouped per destination block, in evaluation order */
	int *count = calloc(p->nblocks + 1, sizeof(int));
	for (int t = 0; t < p->nterms; t++) count[term_dst[t] + 1]++;
	for (int b = 0; b < p->nblocks; b++) count[b + 1] += count[b];
	int *byblk = malloc((p->nterms ? p->nterms : 1) * sizeof(int));
	int *fillp = malloc((p->nblocks + 1) * sizeof(int));
	memcpy(fillp, count, (p->nblocks + 1) * sizeof(int));
	for (int t = 0; t < p->nterms; t++) byblk[fillp[term_dst[t]]++] = t;
	free(fillp);
	/* pass 1: tiles and their costs */
	int tcap = 1024;
	p->tiles = malloc(tcap * sizeof(jn_tile_t));
	double *tile_cost = malloc(tcap * sizeof(double));
	double total_cost = 0;
	for (int b = 0; b < p->nblocks; b++) {
		jn_block_t *B = &p->blocks[b];
		if (B->Np == 0 || B->Nn == 0) continue;
		int64_t cw = B->Nn < PIECE_LANES ? B->Nn : PIECE_LANES;
		int64_t R = B->Nn >= PIECE_LANES ? 1 : PIECE_LANES / B->Nn;
		for (int64_t r0 = 0; r0 < B->Np; r0 += R)
			for (int64_t c0 = 0; c0 < B->Nn; c0 += cw) {
				if (p->ntiles == tcap) {
					tcap *= 2;
					p->tiles = realloc(p->tiles, tcap * sizeof(jn_tile_t));
					tile_cost = realloc(tile_cost, tcap * sizeof(double));
				}
				jn_tile_t *T = &p->tiles[p->ntiles];
				memset(T, 0, sizeof *T);
				T->dst_off = B->offset;
				T->Nn = (int32_t)B->Nn;
				T->row0 = (int32_t)r0; T->nrows = (int32_t)((r0 + R <= B->Np) ? R : B->Np - r0);
				T->col0 = (int32_t)c0; T->ncols = (int32_t)((c0 + cw <= B->Nn) ? cw : B->Nn - c0);
				T->pad = b;     /* destination block while planning */
				double cost = 0;
				for (int q = count[b]; q < count[b + 1]; q++)
					cost += term_cost(p, &p->terms[byblk[q]], T->row0, T->row0 + T->nrows, T->col0, T->col0 + T->ncols);
				tile_cost[p->ntiles++] = cost;
				total_cost += cost;
			}
	}
	if (target_units <= 0) target_units = 152 * 48;
	double target = total_cost / target_units;
	if (target < 256) target = 256;
	/* pass 2: chunks */
	int64_t ucap = 4096, tcap2 = 1 << 16;
	p->units = malloc(ucap * sizeof(jn_unit_t));
	p->unit_terms = malloc(tcap2 * sizeof(int32_t));
	int64_t partial = 0;
	for (int ti = 0; ti < p->ntiles; ti++) {
		jn_tile_t *T = &p->tiles[ti];
		int b = T->pad;
		T->pad = 0;
		T->unit0 = p->nunits;
		int nchunk = (int)ceil(tile_cost[ti] / target);
		if (nchunk < 1) nchunk = 1;
		double per = tile_cost[ti] / nchunk, acc = 0;
		int nb_terms = count[b + 1] - count[b];
		double *cst = malloc((nb_terms ? nb_terms : 1) * sizeof(double));
		int lastnz = -1;
		for (int q = 0; q < nb_terms; q++) {
			cst[q] = term_cost(p, &p->terms[byblk[count[b] + q]], T->row0, T->row0 + T->nrows, T->col0,
					   T->col0 + T->ncols);
			if (cst[q] > 0) lastnz = q;
		}
		int64_t begin = p->n_unit_terms;
		int chunks = 0;
		for (int q = 0; q <= lastnz; q++) {
			if (cst[q] == 0) continue;
			if (p->n_unit_terms == tcap2) { tcap2 *= 2; p->unit_terms = realloc(p->unit_terms, tcap2 * sizeof(int32_t)); }
			p->unit_terms[p->n_unit_terms++] = byblk[count[b] + q];
			acc += cst[q];
			if (acc >= per * (chunks + 1) || q == lastnz) {
				if (p->nunits == ucap) { ucap *= 2; p->units = realloc(p->units, ucap * sizeof(jn_unit_t)); }
				jn_unit_t *U = &p->units[p->nunits++];
				U->tile = ti; U->chunk = chunks++;
				U->t0 = begin; U->t1 = p->n_unit_terms;
				begin = p->n_unit_terms;
			}
		}
		free(cst);
		T->nchunks = chunks;
		T->partial = partial;
		partial += (int64_t)chunks * T->nrows * T->ncols;
	}
	p->n_partial = partial;
	/* longest units first: the warps that start first take the heaviest work */
	{
		double *uc = malloc((p->nunits ? p->nunits : 1) * sizeof(double));
		int *ord = malloc((p->nunits ? p->nunits : 1) * sizeof(int));
		for (int u = 0; u < p->nunits; u++) {
			const jn_unit_t *U = &p->units[u];
			const jn_tile_t *T = &p->tiles[U->tile];
			double cst = 0;
			for (int64_t q = U->t0; q < U->t1; q++)
				cst += term_cost(p, &p->terms[p->unit_terms[q]], T->row0, T->row0 + T->nrows, T->col0,
						 T->col0 + T->ncols);
			uc[u] = cst;
			ord[u] = u;
		}
		qsort_r(ord, p->nunits, sizeof(int), cmp_cost_desc, uc);
		jn_unit_t *sorted = malloc((p->nunits ? p->nunits : 1) * sizeof(jn_unit_t));
		for (int u = 0; u < p->nunits; u++) sorted[u] = p->units[ord[u]];
		free(p->units);
		p->units = sorted;
		free(uc); free(ord);
	}
	free(tile_cost); free(byblk); free(count);
	if (!p->units || !p->tiles || !p->unit_terms) {
		if (err) snprintf(err, errlen, "out of host memory for the work units");
		return 1;
	}
	return 0;
}

/* one list's bound checks: the first entry whose in / out index leaves the
 * sub-bases (-1 if none), and the largest connection index */
typedef struct { const jn_plan_t *p; int64_t *bad_e; uint64_t *kmax; } list_check_t;

static void list_check_item(int64_t l, void *v)
{
	const list_check_t *j = (const list_check_t *)v;
	const jn_list_t *L = &j->p->lists[l];
	int64_t bad = -1;
	uint64_t km = 0;
	for (int64_t e = 0; e < L->len; e++) {
		const int32_t a = L->triples[3 * e], b = L->triples[3 * e + 1];
		if (bad < 0 && (a < 0 || a >= L->nin || b < 0 || b >= L->nout)) bad = e;
		const uint64_t k = (uint32_t)L->triples[3 * e + 2] & 0x7fffffffu;
		if (k > km) km = k;
	}
	j->bad_e[l] = bad;
	j->kmax[l] = km;
}

/* The matrix elements some product reads (the compulsory traffic): the
 * entries' matrix indices for single-species instructions, every (k_n, k_p)
 * pair of the two lists for NP ones.  One work item per matrix block, so no
 * two threads mark the same bytes. */
typedef struct {
	const jn_plan_t *p;
	const int *iptr, *ilist;        /* instructions of each block */
	uint8_t *mark;
	int64_t *count;
	uint8_t *bad;
} census_t;

static void census_block(int64_t b, void *v)
{
	census_t *cs = (census_t *)v;
	const jn_plan_t *p = cs->p;
	const jn_me_t *M = &p->mes[b];
	uint8_t *mk = cs->mark + M->offset;
	for (int q = cs->iptr[b]; q < cs->iptr[b + 1]; q++) {
		const jn_instr_t *x = &p->instr[cs->ilist[q]];
		if (x->kind != JN_KIND_NP) {
			const jn_list_t *L = &p->lists[x->kind == JN_KIND_N ? x->ln : x->lp];
			for (int64_t e = 0; e < L->len; e++) mk[(uint32_t)L->triples[3 * e + 2] & 0x7fffffffu] = 1;
			continue;
		}
		/* every (k_n, k_p) pair of the two lists is visited: mark the product of the distinct sets */
		const jn_list_t *Ln = &p->lists[x->ln], *Lp = &p->lists[x->lp];
		if (!Ln->len || !Lp->len) continue;     /* no pairs; the indices were not range-checked */
		int64_t *kn = malloc((Ln->len ? Ln->len : 1) * sizeof(int64_t));
		int64_t *kp = malloc((Lp->len ? Lp->len : 1) * sizeof(int64_t));
		uint8_t *seen_n = calloc(M->nd_n + 1, 1), *seen_p = calloc(M->nd_p + 1, 1);
		if (!kn || !kp || !seen_n || !seen_p) {
			free(kn); free(kp); free(seen_n); free(seen_p);
			cs->bad[b] = 1;
			return;
		}
		size_t nn = 0, np_ = 0;
		for (int64_t e = 0; e < Ln->len; e++) {
			uint32_t k = (uint32_t)Ln->triples[3 * e + 2] & 0x7fffffffu;
			if (!seen_n[k]) { seen_n[k] = 1; kn[nn++] = k; }
		}
		for (int64_t e = 0; e < Lp->len; e++) {
			uint32_t k = (uint32_t)Lp->triples[3 * e + 2] & 0x7fffffffu;
			if (!seen_p[k]) { seen_p[k] = 1; kp[np_++] = k; }
		}
		for (size_t a = 0; a < np_; a++)
			for (size_t c = 0; c < nn; c++) mk[kn[c] + (int64_t)M->nd_n * kp[a]] = 1;
		free(kn); free(kp); free(seen_n); free(seen_p);
	}
	int64_t n = 0;
	for (int64_t e = 0; e < M->len; e++) n += mk[e];
	cs->count[b] = n;
}

static int me_census(jn_plan_t *p)
{
	const int nb = p->nmes;
	uint8_t *mark = calloc(p->n_me ? p->n_me : 1, 1);
	int *iptr = calloc((size_t)nb + 1, sizeof(int));
	int *ilist = malloc((p->ninstr ? p->ninstr : 1) * sizeof(int));
	int64_t *count = calloc(nb ? nb : 1, sizeof(int64_t));
	uint8_t *bad = calloc(nb ? nb : 1, 1);
	int rc = 1;
	if (!mark || !iptr || !ilist || !count || !bad) goto out;
	for (int i = 0; i < p->ninstr; i++) iptr[p->instr[i].me + 1]++;
	for (int b = 0; b < nb; b++) iptr[b + 1] += iptr[b];
	{
		int *fill = malloc(((size_t)nb + 1) * sizeof(int));
		if (!fill) goto out;
		memcpy(fill, iptr, ((size_t)nb + 1) * sizeof(int));
		for (int i = 0; i < p->ninstr; i++) ilist[fill[p->instr[i].me]++] = i;
		free(fill);
	}
	census_t cs = { p, iptr, ilist, mark, count, bad };
	jn_par_for(nb, census_block, &cs);
	rc = 0;
	for (int b = 0; b < nb; b++) rc |= bad[b];
	p->me_referenced = 0;
	for (int b = 0; b < nb; b++) p->me_referenced += count[b];
out:
	free(mark); free(iptr); free(ilist); free(count); free(bad);
	return rc;
}

int jn_plan_build(jn_plan_t *p, const char *comb_path, const char *order_path, const char *lists_dir,
		  const char *me_dir, int Z, int N, int target_units, char *err, size_t errlen)
{
	comb_t c;
	FILE *f = NULL;
	char *line = NULL;
	size_t cap = 0;
	long maxid = 0;
	int *slot_of_id = NULL;     /* id -> block / list / me slot */
	char *kind_of_id = NULL;    /* 'b' 'l' 'm' */
	int rc;
	memset(p, 0, sizeof *p);
	p->Z = Z; p->N = N;
	if ((rc = read_comb(comb_path, &c, err, errlen))) return rc;
	for (int i = 0; i < c.nb; i++) if (c.b[i].id > maxid) maxid = c.b[i].id;
	for (int i = 0; i < c.nl; i++) if (c.l[i].id > maxid) maxid = c.l[i].id;
	for (int i = 0; i < c.nm; i++) if (c.m[i].id > maxid) maxid = c.m[i].id;
	slot_of_id = malloc((maxid + 1) * sizeof(int));
	kind_of_id = calloc(maxid + 1, 1);
	for (long i = 0; i <= maxid; i++) slot_of_id[i] = -1;
	p->nblocks = c.nb;
	p->blocks = c.b; c.b = NULL;
	int64_t off = 0;
	for (int i = 0; i < p->nblocks; i++) {
		jn_block_t *b = &p->blocks[i];
		if (kind_of_id[b->id]) ERR("array id %d used twice in %s", b->id, comb_path);
		kind_of_id[b->id] = 'b'; slot_of_id[b->id] = i;
		b->offset = off;
		off += b->Np * b->Nn;
	}
	p->dim = off;
	for (int i = 0; i < c.nl; i++) {
		if (kind_of_id[c.l[i].id]) ERR("array id %ld used twice in %s", c.l[i].id, comb_path);
		kind_of_id[c.l[i].id] = 'l'; slot_of_id[c.l[i].id] = -2 - i; /* resolved lazily */
	}
	for (int i = 0; i < c.nm; i++) {
		if (kind_of_id[c.m[i].id]) ERR("array id %ld used twice in %s", c.m[i].id, comb_path);
		kind_of_id[c.m[i].id] = 'm'; slot_of_id[c.m[i].id] = -2 - i;
	}

	/* evaluation order */
	f = fopen(order_path, "r");
	if (!f) ERR("Could not open evaluation order file %s. %s", order_path, strerror(errno));
	int icap = 0;
	while (getline(&line, &cap, f) >= 0) {
		char *b = strstr(line, "BLOCK:");
		if (!b || strstr(line, "UNLOAD_")) continue;
		char *w[16];
		int n = split_words(b, w, 16);
		if (n != 5 && n != 6) ERR("malformed evaluation-order row \"%s\"", b);
		long v[5];
		for (int q = 1; q < n; q++) {
			char *end;
			v[q - 1] = strtol(w[q], &end, 10);
			if (*end || v[q - 1] <= 0 || v[q - 1] > maxid) ERR("unknown array id \"%s\" in evaluation order", w[q]);
		}
		jn_instr_t in = { 0, -1, -1, -1, -1, -1 };
		if (kind_of_id[v[0]] != 'b' || kind_of_id[v[1]] != 'b') ERR("BLOCK row names a non-vector array");
		in.bin = slot_of_id[v[0]]; in.bout = slot_of_id[v[1]];
		long lids[2] = { v[2], n == 6 ? v[3] : 0 };
		long meid = n == 6 ? v[4] : v[3];
		if (kind_of_id[meid] != 'm') ERR("BLOCK row names %ld as matrix elements but it is not one", meid);
		int nl = n == 6 ? 2 : 1;
		int lslot[2] = { -1, -1 };
		char ltype[2] = { 0, 0 };
		for (int q = 0; q < nl; q++) {
			if (kind_of_id[lids[q]] != 'l') ERR("BLOCK row names %ld as an index list but it is not one", lids[q]);
			int s = slot_of_id[lids[q]];
			if (s < 0) {
				int ci = -2 - s;
				if (p->nlists % 256 == 0) p->lists = realloc(p->lists, (p->nlists + 256) * sizeof(jn_list_t));
				jn_list_t *L = &p->lists[p->nlists];
				memset(L, 0, sizeof *L);
				L->id = (int)lids[q]; L->type = c.l[ci].type; L->nin = L->nout = -1;
				s = slot_of_id[lids[q]] = p->nlists++;          /* read below */
			}
			lslot[q] = s;
			ltype[q] = p->lists[s].type;
		}
		if (nl == 2) {
			in.kind = JN_KIND_NP;
			if (ltype[0] == 'n') { in.ln = lslot[0]; in.lp = lslot[1]; } else { in.ln = lslot[1]; in.lp = lslot[0]; }
			if (p->lists[in.ln].type != 'n' || p->lists[in.lp].type != 'p')
				ERR("neutron-proton BLOCK row needs one neutron and one proton list");
		} else if (ltype[0] == 'n') { in.kind = JN_KIND_N; in.ln = lslot[0]; }
		else { in.kind = JN_KIND_P; in.lp = lslot[0]; }
		int ms = slot_of_id[meid];
		if (ms < 0) {
			if (p->nmes % 256 == 0) p->mes = realloc(p->mes, (p->nmes + 256) * sizeof(jn_me_t));
			jn_me_t *M = &p->mes[p->nmes];
			memset(M, 0, sizeof *M);
			M->id = (int)meid;
			ms = slot_of_id[meid] = p->nmes++;
		}
		in.me = ms;
		if (p->ninstr == icap) { icap = icap ? 2 * icap : 1024; p->instr = realloc(p->instr, icap * sizeof(jn_instr_t)); }
		p->instr[p->ninstr++] = in;
	}
	fclose(f); f = NULL;
	if (!p->ninstr) ERR("evaluation order %s holds no BLOCK rows", order_path);

	/* the index lists, read by all host cores; a failing list is read once
	   more on its own for its message, the first in order of appearance */
	{
		uint8_t *bad = calloc(p->nlists ? p->nlists : 1, 1);
		if (!bad) ERR("out of host memory");
		list_job_t lj = { p, lists_dir, bad };
		jn_par_for(p->nlists, list_read_item, &lj);
		int first = -1;
		for (int l = 0; l < p->nlists && first < 0; l++)
			if (bad[l]) first = l;
		free(bad);
		if (first >= 0) {
			jn_list_t *L = &p->lists[first];
			L->triples = read_list_file(lists_dir, L->id, &L->len, err, errlen);
			if (!L->triples) goto fail;
			ERR("index list %d could not be read", L->id);
		}
	}

	/* matrix elements */
	int64_t me_total = 0;
	for (int i = 0; i < p->nmes; i++) {
		jn_me_t *M = &p->mes[i];
		if (me_file_header(me_dir, M->id, &M->nd_n, &M->nd_p, &M->len, err, errlen)) goto fail;
		M->offset = me_total;
		me_total += M->len;
	}
	p->n_me = me_total;
	p->me = malloc((me_total ? me_total : 1) * sizeof(double));
	if (!p->me) ERR("out of host memory for matrix elements");
	if (me_read_all(p, me_dir, p->me, err, errlen)) goto fail;
	p->me_elements = me_total;

	/* validation and list dimensions */
	for (int i = 0; i < p->ninstr; i++) {
		jn_instr_t *x = &p->instr[i];
		jn_block_t *bi = &p->blocks[x->bin], *bo = &p->blocks[x->bout];
		jn_me_t *M = &p->mes[x->me];
		if (x->kind == JN_KIND_N && bi->Np != bo->Np) ERR("instruction %d: neutron term between blocks of different proton dimension", i);
		if (x->kind == JN_KIND_P && bi->Nn != bo->Nn) ERR("instruction %d: proton term between blocks of different neutron dimension", i);
		if (x->kind == JN_KIND_NP && M->nd_n == 0) ERR("instruction %d: matrix block %d has no neutron dimension", i, M->id);
		if (x->kind != JN_KIND_NP) M->single = 1;
		int slots[2] = { x->ln, x->lp };
		for (int q = 0; q < 2; q++) {
			if (slots[q] < 0) continue;
			jn_list_t *L = &p->lists[slots[q]];
			int32_t nin = (int32_t)(L->type == 'n' ? bi->Nn : bi->Np);
			int32_t nout = (int32_t)(L->type == 'n' ? bo->Nn : bo->Np);
			if (L->nin < 0) { L->nin = nin; L->nout = nout; }
			else if (L->nin != nin || L->nout != nout)
				ERR("index list %d is used between sub-bases of different sizes", L->id);
		}
	}
	{
		/* per list, on all host cores: the first entry outside the sub-bases
		   and the largest connection index (lists are shared by many
		   instructions, so each is scanned once) */
		int64_t *bad_e = malloc((p->nlists ? p->nlists : 1) * sizeof(int64_t));
		uint64_t *kmax = malloc((p->nlists ? p->nlists : 1) * sizeof(uint64_t));
		if (!bad_e || !kmax) { free(bad_e); free(kmax); ERR("out of host memory"); }
		list_check_t lc = { p, bad_e, kmax };
		jn_par_for(p->nlists, list_check_item, &lc);
		char msg[512] = "";
		int fail_l = -1;
		for (int l = 0; l < p->nlists && fail_l < 0; l++) {
			jn_list_t *L = &p->lists[l];
			if (L->nin > 65535 || L->nout > 65535) {
				snprintf(msg, sizeof msg,
					 "index list %d maps sub-bases of %d x %d states: more than the 65535 of the packed device format",
					 L->id, L->nin, L->nout);
				fail_l = l;
			} else if (bad_e[l] >= 0) {
				const int64_t e = bad_e[l];
				snprintf(msg, sizeof msg,
					 "index list %d entry %lld: in %d / out %d outside the %d x %d sub-bases", L->id, (long long)e,
					 L->triples[3 * e], L->triples[3 * e + 1], L->nin, L->nout);
				fail_l = l;
			}
		}
		for (int i = 0; i < p->ninstr && fail_l < 0; i++) {
			const jn_instr_t *x = &p->instr[i];
			const jn_me_t *M = &p->mes[x->me];
			if (x->kind == JN_KIND_NP) {
				const jn_list_t *Ln = &p->lists[x->ln], *Lp = &p->lists[x->lp];
				const uint64_t kmax_n = kmax[x->ln], kmax_p = kmax[x->lp];
				if (Ln->len && Lp->len && (kmax_n >= M->nd_n || kmax_n + M->nd_n * kmax_p >= (uint64_t)M->len)) {
					snprintf(msg, sizeof msg,
						 "instruction %d: matrix index outside matrix block %d", i, M->id);
					fail_l = 0;
				}
			} else {
				const int l = x->kind == JN_KIND_N ? x->ln : x->lp;
				const jn_list_t *L = &p->lists[l];
				if (L->len && kmax[l] >= (uint64_t)M->len) {
					int64_t e = 0;
					while ((int64_t)((uint32_t)L->triples[3 * e + 2] & 0x7fffffffu) < M->len) e++;
					snprintf(msg, sizeof msg,
						 "index list %d entry %lld: matrix index outside matrix block %d", L->id, (long long)e, M->id);
					fail_l = 0;
				}
			}
		}
		free(bad_e); free(kmax);
		if (fail_l >= 0) ERR("%s", msg);
	}

	/* matrix elements some product actually reads: the compulsory traffic */
	if (me_census(p)) ERR("out of host memory");

	/* CSR views */
	int64_t nrp = 0, nent = 0;
	for (int l = 0; l < p->nlists; l++) {
		jn_list_t *L = &p->lists[l];
		L->csr_out_ptr = nrp; nrp += L->nout + 1;
		L->csr_in_ptr = nrp; nrp += L->nin + 1;
		L->ent_out = nent; nent += L->len;
		L->ent_in = nent; nent += L->len;
		p->list_entries += L->len;
	}
	if (nent > 0xffffffffll) ERR("index lists too long for 32-bit offsets");
	p->n_rowptr = nrp; p->n_ent = nent;
	p->rowptr = malloc((nrp ? nrp : 1) * sizeof(uint32_t));
	p->ent = malloc((nent ? nent : 1) * 2 * sizeof(uint32_t));
	if (!p->rowptr || !p->ent) ERR("out of host memory for list views");
	{
		uint8_t *bad = calloc(p->nlists ? p->nlists : 1, 1);
		if (!bad) ERR("out of host memory for list views");
		csr_job_t cj = { p, bad };
		jn_par_for(p->nlists, csr_list, &cj);
		int any = 0;
		for (int l = 0; l < p->nlists; l++) any |= bad[l];
		free(bad);
		if (any) ERR("out of host memory for list views");
	}
	/* walks: the non-empty destination rows of both views of every list */
	{
		int64_t nw = 0;
		for (int l = 0; l < p->nlists; l++) {
			jn_list_t *L = &p->lists[l];
			for (int32_t r = 0; r < L->nout; r++) nw += p->rowptr[L->csr_out_ptr + r + 1] > p->rowptr[L->csr_out_ptr + r];
			for (int32_t r = 0; r < L->nin; r++) nw += p->rowptr[L->csr_in_ptr + r + 1] > p->rowptr[L->csr_in_ptr + r];
		}
		p->walks = malloc((nw ? nw : 1) * 2 * sizeof(uint32_t));
		if (!p->walks) ERR("out of host memory for walks");
		for (int l = 0; l < p->nlists; l++) {
			jn_list_t *L = &p->lists[l];
			for (int view = 0; view < 2; view++) {
				const int64_t ptr = view ? L->csr_in_ptr : L->csr_out_ptr;
				const int32_t n = view ? L->nin : L->nout;
				if (view) L->walk_in = p->nwalks; else L->walk_out = p->nwalks;
				for (int32_t r = 0; r < n; r++) {
					uint32_t a = p->rowptr[ptr + r], b = p->rowptr[ptr + r + 1];
					if (b == a) continue;
					if (b - a > 65535) ERR("index list %d: %u entries map onto one state, more than 65535", L->id, b - a);
					p->walks[2 * p->nwalks] = a;
					p->walks[2 * p->nwalks + 1] = (b - a) | ((uint32_t)r << 16);
					p->nwalks++;
				}
				if (view) L->nwalk_in = p->nwalks - L->walk_in; else L->nwalk_out = p->nwalks - L->walk_out;
			}
		}
	}

	/* terms: forward on the output block, transpose on the input block */
	p->terms = malloc(2 * (size_t)p->ninstr * sizeof(jn_term_t));
	int *term_dst = malloc(2 * (size_t)p->ninstr * sizeof(int));
	p->term_dst = term_dst;
	for (int i = 0; i < p->ninstr; i++) {
		jn_instr_t *x = &p->instr[i];
		for (int dir = 0; dir < 2; dir++) {
			if (dir == 1 && x->bin == x->bout) break;
			jn_term_t t;
			memset(&t, 0, sizeof t);
			int src = dir ? x->bout : x->bin, dst = dir ? x->bin : x->bout;
			t.kind = x->kind;
			t.nd = (int32_t)p->mes[x->me].nd_n;
			t.src_off = p->blocks[src].offset;
			t.Nn_src = (int32_t)p->blocks[src].Nn;
			t.Nn_dst = (int32_t)p->blocks[dst].Nn;
			if (x->lp >= 0) {
				jn_list_t *L = &p->lists[x->lp];
				t.p_ptr = dir ? L->csr_in_ptr : L->csr_out_ptr;
				t.p_ent = 0;
			}
			if (x->ln >= 0) {
				jn_list_t *L = &p->lists[x->ln];
				t.n_ptr = dir ? L->csr_in_ptr : L->csr_out_ptr;
				t.n_ent = 0;
			}
			t.me_off = p->mes[x->me].offset;
			if (x->ln >= 0) {
				t.n_e0 = p->rowptr[t.n_ptr];
				t.n_e1 = p->rowptr[t.n_ptr + t.Nn_dst];
				const jn_list_t *L = &p->lists[x->ln];
				t.nw0 = dir ? L->walk_in : L->walk_out;
				t.nw1 = t.nw0 + (dir ? L->nwalk_in : L->nwalk_out);
			}
			if (x->lp >= 0) {
				const jn_list_t *L = &p->lists[x->lp];
				t.pw0 = dir ? L->walk_in : L->walk_out;
				t.pw1 = t.pw0 + (dir ? L->nwalk_in : L->nwalk_out);
			}
			t.instr = i;
			t.transpose = dir;
			term_dst[p->nterms] = dst;
			p->terms[p->nterms++] = t;
		}
	}
	/* visits for accounting */
	for (int i = 0; i < p->ninstr; i++) {
		jn_instr_t *x = &p->instr[i];
		double v;
		if (x->kind == JN_KIND_NP) v = (double)p->lists[x->ln].len * (double)p->lists[x->lp].len;
		else if (x->kind == JN_KIND_P) v = (double)p->lists[x->lp].len * (double)p->blocks[x->bin].Nn;
		else v = (double)p->lists[x->ln].len * (double)p->blocks[x->bin].Np;
		p->visits += (x->bin == x->bout) ? v : 2 * v;
	}

	/* block tiles for exact fixed-point accumulation */
	if (build_block_tiles(p, term_dst, target_units, err, errlen)) goto fail;
	free(slot_of_id); free(kind_of_id);
	free(c.l); free(c.m); free(line);
	return 0;
fail:
	if (f) fclose(f);
	free(line);
	free(c.b); free(c.l); free(c.m);
	free(slot_of_id); free(kind_of_id);
	jn_plan_free(p);
	return 1;
}
