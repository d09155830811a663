/*
 * jn_transform3.c — host plan of the three-body J -> M transform (see
 * jn_transform3.h for the per-element form the device evaluates).
 *
 * Reference parts restated here, in the order the plan builds them:
 *   manager shells (e; l, j descending; tz)      src/Neptune/bases/shells.c:8-71
 *   single-particle order (e, l, j, m desc, tz)  src/Neptune/bases/sp_states.c:7-70
 *   ASCII J-scheme input (.cnf / .mat)           src/Neptune/input/read_3nf_ascii_format.c:14-279,
 *                                                src/Neptune/bases/shells.c:170-330,
 *                                                src/Neptune/bases/jjj_coupled_3p.c:361-494
 *   J-scheme matrix of a coupled block           src/Neptune/input/read_3nf_ascii_format.c:332-437,
 *                                                src/Neptune/bases/jjj_coupled_3p.c:571-669
 *   three-particle M-scheme bases from Anicre    src/Neptune/bases/m_scheme_3p_basis.c:385-418, 646-760;
 *                                                src/Mercury/transform_3nf_block_manager/transform_3nf_block_manager.c:496-544
 *   total-M blocks                               src/Neptune/bases/m_scheme_3p_basis.c:420-622;
 *                                                src/Mercury/transformed_block/transformed_block.c:67-80
 *   coupled basis of an M block                  src/Neptune/bases/jjj_coupled_3p.c:17-76, 228-357
 *   J_abc range and coupled blocks               src/Neptune/block_transform/block_transform.c:33-145, 147-356
 *   S = CG(ja jb jab) CG(jab jc jabc) (+-1)      src/Neptune/jjj_transformation/jjj_transformation.c:13-159
 *   connections, ket / bra states and phases     src/Mercury/connection_list/connection_list.c:61-180, 380-552;
 *                                                src/Mercury/transformed_block/transformed_block.c:113-290
 *
 * Where the reference depends on an unspecified order it is pinned here:
 * the two qsort calls it makes on ties are taken as stable (glibc's qsort is
 * a merge sort), and a J-scheme directory must hold one .cnf and one .mat
 * file.  Inputs on which the reference reads out of bounds or through a
 * failed lookup are reported as errors instead: shells of the J-scheme file
 * that the manager's shells lack, indices past the file's states, basis
 * files whose states are not ascending, and blocks that change total M.
 */
#define _GNU_SOURCE        /* qsort_r */
#include "jn_transform3.h"
#include "jn_jt.h"

#include <dirent.h>
#include <errno.h>
#include <pthread.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define TERR(...) do { snprintf(err, errlen, __VA_ARGS__); goto fail; } while (0)
#define MAX_EMAX 7              /* J_abc <= 45 (doubled): within the Clebsch-Gordan routine's range */

typedef struct { void *a; size_t n, cap, es; } vec3_t;

static int vpush(vec3_t *v, const void *e)
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
/* open-addressing hash map: 64-bit key pair -> 64-bit value           */
/* ------------------------------------------------------------------ */
typedef struct { uint64_t k0, k1; uint64_t v; int used; } hslot_t;
typedef struct { hslot_t *s; size_t cap, n; } hmap_t;

static uint64_t mix(uint64_t z)
{
	z += 0x9e3779b97f4a7c15ull;
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

static int hgrow(hmap_t *h)
{
	size_t cap = h->cap ? 2 * h->cap : 1024;
	hslot_t *s = (hslot_t *)calloc(cap, sizeof *s);
	if (!s) return -1;
	for (size_t i = 0; i < h->cap; i++)
		if (h->s[i].used) {
			size_t j = mix(h->s[i].k0 ^ mix(h->s[i].k1)) & (cap - 1);
			while (s[j].used) j = (j + 1) & (cap - 1);
			s[j] = h->s[i];
		}
	free(h->s);
	h->s = s;
	h->cap = cap;
	return 0;
}

/* value slot of (k0, k1), inserted with v = init when absent; NULL when out of memory */
static uint64_t *hget(hmap_t *h, uint64_t k0, uint64_t k1, int insert, uint64_t init)
{
	if (insert && 2 * (h->n + 1) > h->cap && hgrow(h)) return NULL;
	if (!h->cap) return NULL;
	size_t j = mix(k0 ^ mix(k1)) & (h->cap - 1);
	while (h->s[j].used) {
		if (h->s[j].k0 == k0 && h->s[j].k1 == k1) return &h->s[j].v;
		j = (j + 1) & (h->cap - 1);
	}
	if (!insert) return NULL;
	h->s[j].used = 1; h->s[j].k0 = k0; h->s[j].k1 = k1; h->s[j].v = init;
	h->n++;
	return &h->s[j].v;
}

static void hfree(hmap_t *h) { free(h->s); memset(h, 0, sizeof *h); }

/* ------------------------------------------------------------------ */
/* shells and single-particle states                                    */
/* ------------------------------------------------------------------ */
typedef struct { int e, n, l, j, tz; } shell3_t;

/* the manager's shells (new_shells): e ascending, l from e down in steps
 * of 2, j from 2l+1 down, then tz = -1 (proton), +1 (neutron) */
static int gj_shells(int emax, shell3_t *out)
{
	int n = 0;
	for (int e = 0; e <= emax; e++)
		for (int l = e; l >= (e & 1); l -= 2)
			for (int j = 2 * l + 1; j >= abs(2 * l - 1); j -= 2)
				for (int tz = -1; tz <= 1; tz += 2) {
					if (out) { shell3_t s = { e, (e - l) / 2, l, j, tz }; out[n] = s; }
					n++;
				}
	return n;
}

typedef struct { int shell, m, j, tz; } sp3_t;

/* Neptune's sorted single-particle list: orbital k of the Anicre order
 * (e, l, j ascending, m descending) is state 2k (proton) and 2k+1 (neutron) */
static int sp_states(int emax, const shell3_t *sh, int nsh, sp3_t **out)
{
	int n = 0;
	for (int pass = 0; pass < 2; pass++) {
		n = 0;
		for (int e = 0; e <= emax; e++)
			for (int l = e & 1; l <= e; l += 2)
				for (int j = abs(2 * l - 1); j <= 2 * l + 1; j += 2)
					for (int m = j; m >= -j; m -= 2)
						for (int tz = -1; tz <= 1; tz += 2) {
							if (pass) {
								int s = -1;
								for (int q = 0; q < nsh && s < 0; q++)
									if (sh[q].e == e && sh[q].l == l && sh[q].j == j && sh[q].tz == tz) s = q;
								sp3_t v = { s, m, j, tz };
								(*out)[n] = v;
							}
							n++;
						}
		if (!pass && !(*out = (sp3_t *)calloc(n, sizeof(sp3_t)))) return -1;
	}
	return n;
}

/* ------------------------------------------------------------------ */
/* coupled states: (a, b, c, jab, jabc), 8 bits each                   */
/* ------------------------------------------------------------------ */
static uint64_t jkey(int a, int b, int c, int jab, int jabc)
{
	return (uint64_t)a | (uint64_t)b << 8 | (uint64_t)c << 16 | (uint64_t)jab << 24 | (uint64_t)jabc << 32;
}
#define KA(k) ((int)((k) & 255))
#define KB(k) ((int)(((k) >> 8) & 255))
#define KC(k) ((int)(((k) >> 16) & 255))
#define KJAB(k) ((int)(((k) >> 24) & 255))
#define KJABC(k) ((int)(((k) >> 32) & 255))

/* ------------------------------------------------------------------ */
/* the J-scheme directory (the reference's ASCII format)               */
/* ------------------------------------------------------------------ */
typedef struct {
	int nsh;
	shell3_t *sh;           /* file shells */
	int *tr;                /* file shell -> manager shell, -1 when absent */
	int64_t ns;
	uint64_t *key;          /* canonical key of each file state */
	int *phase;             /* -1 when the file orders a and b against the manager's shells */
	int64_t ne;
	int64_t *bra, *ket;
	double *e;
} jfile_t;

static void jfile_free(jfile_t *f)
{
	free(f->sh); free(f->tr); free(f->key); free(f->phase); free(f->bra); free(f->ket); free(f->e);
	memset(f, 0, sizeof *f);
}

static int ends_with(const char *s, const char *t)
{
	size_t a = strlen(s), b = strlen(t);
	return a >= b && !strcmp(s + a - b, t);
}

static int begins_with(const char *s, const char *t) { return !strncmp(s, t, strlen(t)); }

/* getline into a static-sized buffer; returns 0 at end of file */
static int next_line(FILE *f, char *buf, size_t n) { return fgets(buf, (int)n, f) != NULL; }

/* one stretch of the matrix file, parsed on its own thread: "b k e" rows as
 * sscanf(" %ld %ld %lg ") reads them, rows beginning with --- skipped */
typedef struct {
	char *beg, *end;
	int64_t nstates;
	int64_t n, cap;
	int64_t *bra, *ket;
	double *e;
	const char *bad;        /* first bad row, or NULL */
	int why;                /* 1 incomplete row, 2 state out of range, 3 out of memory */
} matchunk_t;

static void *parse_mat_chunk(void *arg)
{
	matchunk_t *c = (matchunk_t *)arg;
	for (char *ln = c->beg; ln < c->end && !c->bad;) {
		char *eol = (char *)memchr(ln, '\n', (size_t)(c->end - ln));
		if (eol) *eol = 0;
		char *next = eol ? eol + 1 : c->end;
		if (!begins_with(ln, "---")) {
			char *q = ln, *r;
			long long v[2];
			double e = 0.0;
			int got = 0;
			v[0] = strtoll(q, &r, 10);
			if (r != q) {
				got = 1; q = r;
				v[1] = strtoll(q, &r, 10);
				if (r != q) {
					got = 2; q = r;
					e = strtod(q, &r);
					if (r != q) got = 3;
				}
			}
			/* nothing numeric is skipped (blank rows included: the reference
			   repeats the previous row for them, which changes nothing) */
			if (got == 1 || got == 2) { c->bad = ln; c->why = 1; break; }
			if (got == 3) {
				if (v[0] < 0 || v[1] < 0 || v[0] >= c->nstates || v[1] >= c->nstates) { c->bad = ln; c->why = 2; break; }
				if (c->n == c->cap) {
					c->cap = c->cap ? 2 * c->cap : 4096;
					int64_t *a = (int64_t *)realloc(c->bra, c->cap * sizeof(int64_t));
					if (a) c->bra = a;
					int64_t *b = (int64_t *)realloc(c->ket, c->cap * sizeof(int64_t));
					if (b) c->ket = b;
					double *d = (double *)realloc(c->e, c->cap * sizeof(double));
					if (d) c->e = d;
					if (!a || !b || !d) { c->bad = ln; c->why = 3; break; }
				}
				c->bra[c->n] = v[0]; c->ket[c->n] = v[1]; c->e[c->n] = e;
				c->n++;
			}
		}
		ln = next;
	}
	return NULL;
}

static int read_jfile(jfile_t *J, const char *dir, const shell3_t *msh, int nmsh, char *err, size_t errlen)
{
	memset(J, 0, sizeof *J);
	char cnf[4096] = "", mat[4096] = "";
	int ncnf = 0, nmat = 0;
	DIR *d = opendir(dir);
	if (!d) { snprintf(err, errlen, "Could not open the J-scheme directory \"%s\". %s", dir, strerror(errno)); return -1; }
	struct dirent *de;
	while ((de = readdir(d))) {
		if (ends_with(de->d_name, ".cnf")) { snprintf(cnf, sizeof cnf, "%s/%s", dir, de->d_name); ncnf++; }
		if (ends_with(de->d_name, ".mat")) { snprintf(mat, sizeof mat, "%s/%s", dir, de->d_name); nmat++; }
	}
	closedir(d);
	if (ncnf != 1 || nmat != 1) {
		snprintf(err, errlen, "%s: the J-scheme directory needs one .cnf and one .mat file (has %d and %d)", dir, ncnf, nmat);
		return -1;
	}
	FILE *f = fopen(cnf, "r");
	if (!f) { snprintf(err, errlen, "Could not open file \"%s\". %s", cnf, strerror(errno)); return -1; }
	char line[1024];
	vec3_t shv = { 0 }, stv = { 0 };
	shv.es = sizeof(shell3_t); stv.es = 5 * sizeof(int);
	int stage = 0;          /* 0: before shells, 1: shells, 2: between, 3: states header, 4: states */
	int rc = -1;
	while (next_line(f, line, sizeof line)) {
		if (!strcmp(line, "\n")) continue;
		if (stage == 0) {
			if (strcmp(line, "---single-particle-states---\n")) { snprintf(err, errlen, "%s: no single-particle block", cnf); goto cnf_out; }
			stage = 1;
			continue;
		}
		if (stage == 1 || stage == 4) {
			if (begins_with(line, "---")) {
				if ((stage == 1 && shv.n == 0) || (stage == 4 && stv.n == 0)) continue;   /* headings before the rows */
				if (stage == 4) break;
				stage = 2;
			} else if (stage == 1) {
				int i, n, l, j, tz;
				if (sscanf(line, "%d %d %d %d %d", &i, &n, &l, &j, &tz) < 5) { snprintf(err, errlen, "wrong line format in \"%s\"", line); goto cnf_out; }
				shell3_t s = { 2 * n + l, n, l, j, tz };
				if (vpush(&shv, &s)) { snprintf(err, errlen, "out of memory"); goto cnf_out; }
				continue;
			} else {
				int i, v[5];
				long a, b, c;
				if (sscanf(line, "%d %ld %ld %ld %d %d", &i, &a, &b, &c, &v[3], &v[4]) < 6) { snprintf(err, errlen, "wrong line format in \"%s\"", line); goto cnf_out; }
				v[0] = (int)a; v[1] = (int)b; v[2] = (int)c;
				if (vpush(&stv, v)) { snprintf(err, errlen, "out of memory"); goto cnf_out; }
				continue;
			}
		}
		if (stage == 2) {
			if (!strcmp(line, "---three-particle-states---\n")) { stage = 3; continue; }
			continue;
		}
		if (stage == 3) {
			if (strcmp(line, "---i---a---b---c---Jab-Jabc---\n")) {
				snprintf(err, errlen, "%s: the three-particle states are not jjj-coupled (%.60s)", cnf, line);
				goto cnf_out;
			}
			stage = 4;
			continue;
		}
	}
	if (stage < 4 || !stv.n) { snprintf(err, errlen, "%s: no three-particle states", cnf); goto cnf_out; }
	rc = 0;
cnf_out:
	fclose(f);
	if (rc) { free(shv.a); free(stv.a); return -1; }
	J->nsh = (int)shv.n;
	J->sh = (shell3_t *)shv.a;
	J->ns = (int64_t)stv.n;
	J->tr = (int *)malloc((J->nsh ? J->nsh : 1) * sizeof(int));
	J->key = (uint64_t *)malloc(J->ns * sizeof(uint64_t));
	J->phase = (int *)malloc(J->ns * sizeof(int));
	if (!J->tr || !J->key || !J->phase) { free(stv.a); snprintf(err, errlen, "out of memory"); return -1; }
	/* matching_shells: the first manager shell of equal (e, l, j, tz) (shells.c:430-458) */
	for (int i = 0; i < J->nsh; i++) {
		J->tr[i] = -1;
		for (int q = 0; q < nmsh && J->tr[i] < 0; q++)
			if (msh[q].e == J->sh[i].e && msh[q].l == J->sh[i].l && msh[q].j == J->sh[i].j && msh[q].tz == J->sh[i].tz)
				J->tr[i] = q;
	}
	const int *sv = (const int *)stv.a;
	for (int64_t i = 0; i < J->ns; i++) {
		const int *v = sv + 5 * i;
		for (int q = 0; q < 3; q++)
			if (v[q] < 0 || v[q] >= J->nsh) {
				snprintf(err, errlen, "%s: state %lld names shell %d of %d", cnf, (long long)i, v[q], J->nsh);
				free(stv.a);
				return -1;
			}
		int a = J->tr[v[0]], b = J->tr[v[1]], c = J->tr[v[2]];
		if (a < 0 || b < 0 || c < 0) {
			free(stv.a);
			snprintf(err, errlen, "%s: state %lld uses a shell beyond the single-particle energy limit", cnf, (long long)i);
			return -1;
		}
		int ph = 1;
		if (a > b) { int t = a; a = b; b = t; ph = -1; }
		if (v[3] < 0 || v[3] > 255 || v[4] < 0 || v[4] > 255) { free(stv.a); snprintf(err, errlen, "%s: state %lld: J out of range", cnf, (long long)i); return -1; }
		J->key[i] = jkey(a, b, c, v[3], v[4]);
		J->phase[i] = ph;
	}
	free(stv.a);
	/* the matrix file: "b k e" rows (read as sscanf(" %ld %ld %lg ") reads
	   them), rows beginning with --- skipped; the file is read whole */
	f = fopen(mat, "rb");
	if (!f) { snprintf(err, errlen, "Could not open file \"%s\". %s", mat, strerror(errno)); return -1; }
	fseek(f, 0, SEEK_END);
	const long bytes = ftell(f);
	fseek(f, 0, SEEK_SET);
	char *text = (char *)malloc((bytes > 0 ? bytes : 0) + 1);
	if (!text || (bytes > 0 && fread(text, 1, bytes, f) != (size_t)bytes)) {
		fclose(f); free(text); snprintf(err, errlen, "%s: read failed", mat); return -1;
	}
	fclose(f);
	text[bytes > 0 ? bytes : 0] = 0;
	/* stretches of whole rows, parsed in parallel and joined in file order */
	int nthr = (int)(bytes / (4l << 20)) + 1;
	if (nthr > 16) nthr = 16;
	matchunk_t ch[16];
	pthread_t th[16];
	memset(ch, 0, sizeof ch);
	char *pos = text, *stop = text + (bytes > 0 ? bytes : 0);
	for (int i = 0; i < nthr; i++) {
		ch[i].beg = pos;
		char *cut = i == nthr - 1 ? stop : text + (bytes / nthr) * (i + 1);
		if (cut < pos) cut = pos;
		while (cut > text && cut < stop && cut[-1] != '\n') cut++;     /* end after a newline */
		ch[i].end = cut;
		ch[i].nstates = J->ns;
		pos = cut;
	}
	int started = 0;
	for (int i = 1; i < nthr; i++)
		if (pthread_create(&th[i], NULL, parse_mat_chunk, &ch[i]) == 0) started |= 1 << i;
	parse_mat_chunk(&ch[0]);
	for (int i = 1; i < nthr; i++) {
		if (started & (1 << i)) pthread_join(th[i], NULL);
		else parse_mat_chunk(&ch[i]);
	}
	rc = 0;
	int64_t n = 0;
	for (int i = 0; i < nthr && !rc; i++) {
		if (ch[i].bad) {
			if (ch[i].why == 1) snprintf(err, errlen, "%s: incomplete row \"%.60s\"", mat, ch[i].bad);
			else if (ch[i].why == 2) snprintf(err, errlen, "%s: row names state %.40s of %lld", mat, ch[i].bad, (long long)J->ns);
			else snprintf(err, errlen, "out of memory");
			rc = -1;
		}
		n += ch[i].n;
	}
	if (!rc) {
		J->bra = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
		J->ket = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
		J->e = (double *)malloc((n ? n : 1) * sizeof(double));
		if (!J->bra || !J->ket || !J->e) { snprintf(err, errlen, "out of memory"); rc = -1; }
	}
	int64_t o = 0;
	for (int i = 0; i < nthr; i++) {
		if (!rc && ch[i].n) {
			memcpy(J->bra + o, ch[i].bra, ch[i].n * sizeof(int64_t));
			memcpy(J->ket + o, ch[i].ket, ch[i].n * sizeof(int64_t));
			memcpy(J->e + o, ch[i].e, ch[i].n * sizeof(double));
			o += ch[i].n;
		}
		free(ch[i].bra); free(ch[i].ket); free(ch[i].e);
	}
	free(text);
	J->ne = rc ? 0 : n;
	return rc;
}

/* ------------------------------------------------------------------ */
/* Anicre basis files                                                   */
/* ------------------------------------------------------------------ */
typedef struct { int sp, k, E; int64_t n; int16_t *s; int *M; } kfile_t;   /* sp: 0 proton, 1 neutron */

typedef struct {
	const char *dir;
	int norb;
	const sp3_t *spst;
	vec3_t files;           /* kfile_t * */
} kcache_t;

static void kcache_free(kcache_t *c)
{
	for (size_t i = 0; i < c->files.n; i++) {
		kfile_t *f = ((kfile_t **)c->files.a)[i];
		free(f->s); free(f->M); free(f);
	}
	free(c->files.a);
	memset(&c->files, 0, sizeof c->files);
}

static const kfile_t *kfile(kcache_t *c, int sp, int k, int E, char *err, size_t errlen)
{
	kfile_t **f = (kfile_t **)c->files.a;
	for (size_t i = 0; i < c->files.n; i++)
		if (f[i]->sp == sp && f[i]->k == k && f[i]->E == E) return f[i];
	char path[4352];
	snprintf(path, sizeof path, "%s/%.*s_inds_index_lists/basis_energy_%d", c->dir, k, sp ? "nnn" : "ppp", E);
	FILE *fp = fopen(path, "rb");
	if (!fp) { snprintf(err, errlen, "Could not open file \"%s\". %s", path, strerror(errno)); return NULL; }
	fseek(fp, 0, SEEK_END);
	long bytes = ftell(fp);
	fseek(fp, 0, SEEK_SET);
	if (bytes < 0 || bytes % (2 * k)) { fclose(fp); snprintf(err, errlen, "%s: size is not a multiple of %d", path, 2 * k); return NULL; }
	kfile_t *nf = (kfile_t *)calloc(1, sizeof *nf);
	if (!nf) { fclose(fp); snprintf(err, errlen, "out of memory"); return NULL; }
	nf->sp = sp; nf->k = k; nf->E = E; nf->n = bytes / (2 * k);
	nf->s = (int16_t *)malloc(bytes ? bytes : 1);
	nf->M = (int *)malloc((nf->n ? nf->n : 1) * sizeof(int));
	if (!nf->s || !nf->M || (bytes && fread(nf->s, 1, bytes, fp) != (size_t)bytes)) {
		fclose(fp); free(nf->s); free(nf->M); free(nf); snprintf(err, errlen, "%s: short read", path); return NULL;
	}
	fclose(fp);
	for (int64_t i = 0; i < nf->n; i++) {
		int M = 0;
		for (int q = 0; q < k; q++) {
			const int o = nf->s[i * k + q];
			if (o < 0 || o >= c->norb) {
				free(nf->s); free(nf->M); free(nf);
				snprintf(err, errlen, "%s: orbital %d outside the %d orbitals of the single-particle energy limit", path, o, c->norb);
				return NULL;
			}
			M += c->spst[2 * o].m;
		}
		nf->M[i] = M;
	}
	if (vpush(&c->files, &nf)) { free(nf->s); free(nf->M); free(nf); snprintf(err, errlen, "out of memory"); return NULL; }
	return nf;
}

/* annihilated states of `ann` x the first run of created states of `cre`
 * with M + dM, in Mercury's order (connection_list.c:448-498) */
static int kconnections(const kfile_t *ann, const kfile_t *cre, int dM, vec3_t *pairs)
{
	for (int64_t i = 0; i < ann->n; i++) {
		const int Mc = ann->M[i] + dM;
		int64_t c = 0;
		while (c < cre->n && cre->M[c] != Mc) c++;
		for (; c < cre->n && cre->M[c] == Mc; c++) {
			int32_t pr[2] = { (int32_t)i, (int32_t)c };
			if (vpush(pairs, pr)) return -1;
		}
	}
	return 0;
}

/* ------------------------------------------------------------------ */
/* three-particle M-scheme bases, one per (Tz, Ep, En)                  */
/* ------------------------------------------------------------------ */
typedef struct {
	int M;
	int64_t start, n;       /* states of the basis */
	int jlo, jhi;           /* find_min_jabc / find_max_jabc (doubled) */
} mblock_t;

typedef struct {
	int tz, Ep, En, parity;
	int64_t n;
	int *st;                /* n x 3 single-particle states as the basis stores them */
	int *M;
	int64_t first;          /* first global state id */
	int nmb;
	mblock_t *mb;
	/* LUT of a two-species basis over (proton file position, neutron file position) */
	const kfile_t *pf, *nf;
	int64_t lut;
	/* coupled states reached, per J_abc slot: sorted keys */
	int nslots;
	uint64_t **skeys;
	int *nskeys;
} basis3_t;

typedef struct {
	const sp3_t *sp;
	const shell3_t *sh;
	int nslots;
	vec3_t bases;           /* basis3_t */
	vec3_t ms;              /* jn_m3state_t */
	vec3_t terms;           /* jn_m3term_t */
	vec3_t lut;             /* int32 */
	hmap_t cg;              /* Clebsch-Gordan cache */
	int64_t coupled;
	double dense_flops;
	int64_t mblocks;
} t3build_t;

static void basis_free(basis3_t *b)
{
	free(b->st); free(b->M); free(b->mb);
	if (b->skeys)
		for (int s = 0; s < b->nslots; s++) free(b->skeys[s]);
	free(b->skeys); free(b->nskeys);
}

static int st_M(const t3build_t *t, const int *s) { return t->sp[s[0]].m + t->sp[s[1]].m + t->sp[s[2]].m; }

static double cg_cached(t3build_t *t, int j1, int j2, int j3, int m1, int m2, int m3)
{
	const uint64_t k = (uint64_t)j1 | (uint64_t)j2 << 8 | (uint64_t)j3 << 16 | (uint64_t)(m1 + 128) << 24 |
			   (uint64_t)(m2 + 128) << 32 | (uint64_t)(m3 + 128) << 40;
	uint64_t *v = hget(&t->cg, k, 0, 0, 0);
	if (v) { double r; memcpy(&r, v, 8); return r; }
	double r = jn_cg(j1, j2, j3, m1, m2, m3);
	uint64_t bits;
	memcpy(&bits, &r, 8);
	v = hget(&t->cg, k, 0, 1, bits);
	return r;
}

/* stable merge sort of 64-bit records by a comparison on a context */
typedef int (*cmp3_fn)(const void *ctx, uint64_t a, uint64_t b);
static void msort64(uint64_t *a, uint64_t *tmp, size_t n, cmp3_fn cmp, const void *ctx)
{
	if (n < 2) return;
	const size_t h = n / 2;
	msort64(a, tmp, h, cmp, ctx);
	msort64(a + h, tmp, n - h, cmp, ctx);
	size_t i = 0, j = h, k = 0;
	while (i < h && j < n) tmp[k++] = cmp(ctx, a[j], a[i]) < 0 ? a[j++] : a[i++];
	while (i < h) tmp[k++] = a[i++];
	while (j < n) tmp[k++] = a[j++];
	memcpy(a, tmp, n * sizeof *a);
}

/* comp_jjj_states (jjj_coupled_3p.c:17-76): J_abc, then J_ab, Tz, parity, energy */
static int cmp_jjj(const void *ctx, uint64_t x, uint64_t y)
{
	const shell3_t *sh = (const shell3_t *)ctx;
	if (KJABC(x) != KJABC(y)) return KJABC(x) - KJABC(y);
	if (KJAB(x) != KJAB(y)) return KJAB(x) - KJAB(y);
	const int tx = sh[KA(x)].tz + sh[KB(x)].tz + sh[KC(x)].tz, ty = sh[KA(y)].tz + sh[KB(y)].tz + sh[KC(y)].tz;
	if (tx != ty) return tx - ty;
	const int px = (sh[KA(x)].l + sh[KB(x)].l + sh[KC(x)].l) & 1, py = (sh[KA(y)].l + sh[KB(y)].l + sh[KC(y)].l) & 1;
	if (px != py) return px - py;
	return (sh[KA(x)].e + sh[KB(x)].e + sh[KC(x)].e) - (sh[KA(y)].e + sh[KB(y)].e + sh[KC(y)].e);
}

/* compare_m_scheme_3p_states_m: total M only */
static int cmp_M(const void *ctx, uint64_t x, uint64_t y)
{
	const int *M = (const int *)ctx;
	return M[x] - M[y];
}

static void sort3(int *s, int *phase)
{
	int p = 1, t;
	if (s[0] > s[1]) { t = s[0]; s[0] = s[1]; s[1] = t; p = -p; }
	if (s[1] > s[2]) { t = s[1]; s[1] = s[2]; s[2] = t; p = -p; }
	if (s[0] > s[1]) { t = s[0]; s[0] = s[1]; s[1] = t; p = -p; }
	if (phase) *phase = p;
}

/* the coupled basis of one M block (new_jjj_basis_m_scheme), sorted; *out malloc'ed */
static int mblock_coupled(const t3build_t *t, const int *st, int64_t n, uint64_t **out, int64_t *nout)
{
	vec3_t keys = { 0 };
	keys.es = sizeof(uint64_t);
	hmap_t seen = { 0 };
	const sp3_t *sp = t->sp;
	const shell3_t *sh = t->sh;
	for (int64_t i = 0; i < n; i++) {
		int c0[3] = { st[3 * i], st[3 * i + 1], st[3 * i + 2] };
		/* sort_on_shells: three conditional swaps on the shell index */
#define SH(x) (sp[x].shell)
		int tmp;
		if (SH(c0[0]) > SH(c0[1])) { tmp = c0[0]; c0[0] = c0[1]; c0[1] = tmp; }
		if (SH(c0[1]) > SH(c0[2])) { tmp = c0[1]; c0[1] = c0[2]; c0[2] = tmp; }
		if (SH(c0[0]) > SH(c0[1])) { tmp = c0[0]; c0[0] = c0[1]; c0[1] = tmp; }
		int cands[3][3], num;
		const int sa = SH(c0[0]), sb = SH(c0[1]), sc = SH(c0[2]);
		for (int q = 0; q < 3; q++) memcpy(cands[q], c0, sizeof c0);
		if (sa == sb && sb == sc) {
			/* (a b c), (a c b), (c a b) */
			tmp = cands[1][1]; cands[1][1] = cands[1][2]; cands[1][2] = tmp;
			tmp = cands[2][2]; cands[2][2] = cands[2][1]; cands[2][1] = cands[2][0]; cands[2][0] = tmp;
			num = 3;
		} else if (sa == sb && sb < sc) {
			/* (a c b), (b c a) */
			tmp = cands[0][1]; cands[0][1] = cands[0][2]; cands[0][2] = tmp;
			tmp = cands[1][2]; cands[1][2] = cands[1][0]; cands[1][0] = cands[1][1]; cands[1][1] = tmp;
			num = 2;
		} else if (sa < sb && sb == sc) {
			/* (a b c), (a c b) */
			tmp = cands[1][1]; cands[1][1] = cands[1][2]; cands[1][2] = tmp;
			num = 2;
		} else {
			num = 1;
		}
		for (int q = 0; q < num; q++) {
			const int a = SH(cands[q][0]), b = SH(cands[q][1]), c = SH(cands[q][2]);
			const int mab = sp[cands[q][0]].m + sp[cands[q][1]].m, mabc = mab + sp[cands[q][2]].m;
			const int ja = sh[a].j, jb = sh[b].j, jc = sh[c].j;
			int jab0 = abs(ja - jb);
			if (abs(mab) > jab0) jab0 = abs(mab);
			const int step = a == b ? 4 : 2;
			for (int jab = jab0; jab <= ja + jb; jab += step) {
				int jabc0 = abs(jab - jc);
				if (abs(mabc) > jabc0) jabc0 = abs(mabc);
				for (int jabc = jabc0; jabc <= jab + jc; jabc += 2) {
					const uint64_t k = jkey(a, b, c, jab, jabc);
					uint64_t *v = hget(&seen, k, 0, 1, 0);
					if (!v) { hfree(&seen); free(keys.a); return -1; }
					if (*v) continue;
					*v = 1;
					if (vpush(&keys, &k)) { hfree(&seen); free(keys.a); return -1; }
				}
			}
		}
#undef SH
	}
	hfree(&seen);
	uint64_t *tmpb = (uint64_t *)malloc((keys.n ? keys.n : 1) * sizeof(uint64_t));
	if (!tmpb) { free(keys.a); return -1; }
	msort64((uint64_t *)keys.a, tmpb, keys.n, cmp_jjj, sh);
	free(tmpb);
	*out = keys.a ? (uint64_t *)keys.a : (uint64_t *)malloc(sizeof(uint64_t));
	*nout = (int64_t)keys.n;
	return 0;
}

static int cmp_u64(const void *x, const void *y)
{
	const uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
	return a < b ? -1 : a > b;
}

static int64_t find_key(const uint64_t *k, int64_t n, uint64_t v)
{
	int64_t lo = 0, hi = n;
	while (lo < hi) {
		int64_t mid = (lo + hi) / 2;
		if (k[mid] < v) lo = mid + 1; else hi = mid;
	}
	return lo < n && k[lo] == v ? lo : -1;
}

/* sorted shell triple of a coupled key: the index of its permutation class */
static uint64_t shell_class(int a, int b, int c)
{
	int s[3] = { a, b, c };
	sort3(s, NULL);
	return (uint64_t)s[0] | (uint64_t)s[1] << 8 | (uint64_t)s[2] << 16;
}

/* S of coupled state k and M-scheme state st (new_jjj_transformation,
 * jjj_transformation.c:51-121): the first permutation of the state whose
 * shells match k in order gives CG(ja jb jab; ma mb) CG(jab jc jabc; mab mc)
 * times its sign; 0 when |M| > jabc or no permutation matches */
static double s_coef(t3build_t *t, uint64_t k, const int *st)
{
	const sp3_t *sp = t->sp;
	const shell3_t *sh = t->sh;
	const int a = KA(k), b = KB(k), c = KC(k), jab = KJAB(k), jabc = KJABC(k);
	int m[3] = { st[0], st[1], st[2] };
	if (abs(sp[m[0]].m + sp[m[1]].m + sp[m[2]].m) > jabc) return 0.0;
	for (int p = 0; p < 6; p++) {
		if (sp[m[0]].shell == a && sp[m[1]].shell == b && sp[m[2]].shell == c) {
			const int ma = sp[m[0]].m, mb = sp[m[1]].m, mc = sp[m[2]].m;
			const double cg1 = cg_cached(t, sh[a].j, sh[b].j, jab, ma, mb, ma + mb);
			const double cg2 = cg_cached(t, jab, sh[c].j, jabc, ma + mb, mc, ma + mb + mc);
			const double r = cg1 * cg2 * ((p & 1) ? -1.0 : 1.0);
			return 0.0 + r;
		}
		int tmp;
		if (p & 1) { tmp = m[0]; m[0] = m[1]; m[1] = tmp; }
		else { tmp = m[1]; m[1] = m[2]; m[2] = tmp; }
	}
	return 0.0;
}

/* one basis: states, M blocks, coupled states per slot, expansion terms */
static int build_basis(t3build_t *t, kcache_t *kc, int tz, int Ep, int En, char *err, size_t errlen)
{
	basis3_t *B0 = (basis3_t *)t->bases.a;
	for (size_t i = 0; i < t->bases.n; i++)
		if (B0[i].tz == tz && B0[i].Ep == Ep && B0[i].En == En) return (int)i;
	basis3_t b;
	memset(&b, 0, sizeof b);
	b.tz = tz; b.Ep = Ep; b.En = En;
	b.lut = -1;
	b.nslots = t->nslots;
	const int nn = (tz + 3) / 2, np = 3 - nn;
	if (np == 3 || nn == 3) {
		/* read_single_particle_type_file: the file's states in file order */
		const kfile_t *f = kfile(kc, nn == 3, 3, nn == 3 ? En : Ep, err, errlen);
		if (!f) return -1;
		b.n = f->n;
		b.st = (int *)malloc((b.n ? b.n : 1) * 3 * sizeof(int));
		if (!b.st) { snprintf(err, errlen, "out of memory"); return -1; }
		for (int64_t i = 0; i < b.n; i++) {
			for (int q = 0; q < 3; q++) b.st[3 * i + q] = 2 * f->s[3 * i + q] + (nn == 3);
			if (!(b.st[3 * i] < b.st[3 * i + 1] && b.st[3 * i + 1] < b.st[3 * i + 2])) {
				snprintf(err, errlen, "basis file of %s energy %d: state %lld is not in ascending order", nn == 3 ? "nnn" : "ppp",
					 nn == 3 ? En : Ep, (long long)i);
				free(b.st);
				return -1;
			}
		}
		b.pf = nn == 3 ? NULL : f;
		b.nf = nn == 3 ? f : NULL;
	} else {
		/* read_two_particle_type_files: protons major, neutrons minor, each
		   state sorted, then a stable sort by total M */
		const kfile_t *pf = kfile(kc, 0, np, Ep, err, errlen);
		const kfile_t *nf = pf ? kfile(kc, 1, nn, En, err, errlen) : NULL;
		if (!nf) return -1;
		b.pf = pf; b.nf = nf;
		b.n = pf->n * nf->n;
		int *raw = (int *)malloc((b.n ? b.n : 1) * 3 * sizeof(int));
		int *Mraw = (int *)malloc((b.n ? b.n : 1) * sizeof(int));
		uint64_t *ord = (uint64_t *)malloc((b.n ? b.n : 1) * sizeof(uint64_t));
		uint64_t *tmp = (uint64_t *)malloc((b.n ? b.n : 1) * sizeof(uint64_t));
		b.st = (int *)malloc((b.n ? b.n : 1) * 3 * sizeof(int));
		int32_t *lpos = (int32_t *)malloc((b.n ? b.n : 1) * sizeof(int32_t));
		if (!raw || !Mraw || !ord || !tmp || !b.st || !lpos) {
			free(raw); free(Mraw); free(ord); free(tmp); free(b.st); free(lpos);
			snprintf(err, errlen, "out of memory");
			return -1;
		}
		for (int64_t pi = 0; pi < pf->n; pi++)
			for (int64_t ni = 0; ni < nf->n; ni++) {
				const int64_t i = pi * nf->n + ni;
				int s[3], q = 0;
				for (int r = 0; r < np; r++) s[q++] = 2 * pf->s[pi * np + r];
				for (int r = 0; r < nn; r++) s[q++] = 2 * nf->s[ni * nn + r] + 1;
				sort3(s, NULL);
				memcpy(raw + 3 * i, s, sizeof s);
				Mraw[i] = st_M(t, s);
				ord[i] = (uint64_t)i;
			}
		msort64(ord, tmp, (size_t)b.n, cmp_M, Mraw);
		for (int64_t i = 0; i < b.n; i++) {
			memcpy(b.st + 3 * i, raw + 3 * ord[i], 3 * sizeof(int));
			lpos[ord[i]] = (int32_t)i;
		}
		/* LUT: connection order (neutrons, then protons) sorted, with its sign */
		b.lut = (int64_t)t->lut.n;
		for (int64_t pi = 0; pi < pf->n; pi++)
			for (int64_t ni = 0; ni < nf->n; ni++) {
				int s[3], q = 0, ph;
				for (int r = 0; r < nn; r++) s[q++] = 2 * nf->s[ni * nn + r] + 1;
				for (int r = 0; r < np; r++) s[q++] = 2 * pf->s[pi * np + r];
				sort3(s, &ph);
				const int32_t pos = lpos[pi * nf->n + ni];
				const int32_t v = ph > 0 ? pos : -pos - 1;     /* made global below */
				if (vpush(&t->lut, &v)) { snprintf(err, errlen, "out of memory"); return -1; }
			}
		free(raw); free(Mraw); free(ord); free(tmp); free(lpos);
	}
	b.M = (int *)malloc((b.n ? b.n : 1) * sizeof(int));
	if (!b.M) { snprintf(err, errlen, "out of memory"); return -1; }
	for (int64_t i = 0; i < b.n; i++) b.M[i] = st_M(t, b.st + 3 * i);
	b.first = (int64_t)t->ms.n;
	if (b.lut >= 0) {
		int32_t *L = (int32_t *)t->lut.a + b.lut;
		for (int64_t i = 0; i < b.n; i++) L[i] = L[i] >= 0 ? (int32_t)(b.first + L[i]) : (int32_t)(-(b.first + (-L[i] - 1)) - 1);
	}
	if (b.n) {
		b.parity = (Ep + En) & 1;
		/* total-M blocks: [M of the first state, M of the last state] in steps of 2,
		   each the run of its states (generate_block) */
		vec3_t mbv = { 0 };
		mbv.es = sizeof(mblock_t);
		for (int M = b.M[0]; M <= b.M[b.n - 1]; M += 2) {
			mblock_t m = { M, 0, 0, -1, -1 };
			int64_t i = 0;
			while (i < b.n && b.M[i] != M) i++;
			m.start = i;
			while (i < b.n && b.M[i] == M) i++;
			m.n = i - m.start;
			for (int64_t q = m.start; q < m.start + m.n; q++) {
				const int *s = b.st + 3 * q;
				const int ja = t->sh[t->sp[s[0]].shell].j, jb = t->sh[t->sp[s[1]].shell].j, jc = t->sh[t->sp[s[2]].shell].j;
				int lo = abs(abs(ja - jb) - jc);
				if (abs(M) > lo) lo = abs(M);
				if (m.jlo < 0 || lo < m.jlo) m.jlo = lo;
				if (ja + jb + jc > m.jhi) m.jhi = ja + jb + jc;
			}
			if (vpush(&mbv, &m)) { free(mbv.a); snprintf(err, errlen, "out of memory"); return -1; }
		}
		b.nmb = (int)mbv.n;
		b.mb = (mblock_t *)mbv.a;
	}
	/* the states' slots in the global arrays */
	for (int64_t i = 0; i < b.n; i++) {
		jn_m3state_t z = { 0, 0, 0, 0 };
		if (vpush(&t->ms, &z)) { snprintf(err, errlen, "out of memory"); return -1; }
	}
	/* per M block: coupled basis, then each state's terms */
	b.skeys = (uint64_t **)calloc(t->nslots, sizeof(uint64_t *));
	b.nskeys = (int *)calloc(t->nslots, sizeof(int));
	vec3_t slot_keys[64];
	memset(slot_keys, 0, sizeof slot_keys);
	for (int s = 0; s < t->nslots; s++) slot_keys[s].es = sizeof(uint64_t);
	vec3_t pend = { 0 };    /* terms with their coupled key; v is resolved when the slot lists are final */
	pend.es = sizeof(jn_m3term_t) + sizeof(uint64_t);
	int64_t term0 = (int64_t)t->terms.n;
	for (int q = 0; q < b.nmb; q++) {
		const mblock_t *m = &b.mb[q];
		if (!m->n) continue;
		t->mblocks++;
		uint64_t *keys = NULL;
		int64_t nk = 0;
		if (mblock_coupled(t, b.st + 3 * m->start, m->n, &keys, &nk)) { snprintf(err, errlen, "out of memory"); return -1; }
		t->coupled += nk;
		for (int64_t i = 0; i < nk; i++) {
			const int s = (KJABC(keys[i]) - 1) / 2;
			if (s >= t->nslots || !(KJABC(keys[i]) & 1)) {
				snprintf(err, errlen, "J_abc %d out of range", KJABC(keys[i]));
				free(keys);
				return -1;
			}
			if (vpush(&slot_keys[s], &keys[i])) { free(keys); snprintf(err, errlen, "out of memory"); return -1; }
		}
		/* candidates per shell class, in basis order */
		hmap_t cls = { 0 };
		int64_t *next = (int64_t *)malloc((nk ? nk : 1) * sizeof(int64_t));
		for (int64_t i = nk - 1; i >= 0; i--) {
			uint64_t *head = hget(&cls, shell_class(KA(keys[i]), KB(keys[i]), KC(keys[i])), 0, 1, (uint64_t)-1);
			next[i] = (int64_t)*head;
			*head = (uint64_t)i;
		}
		for (int64_t i = m->start; i < m->start + m->n; i++) {
			const int *s = b.st + 3 * i;
			jn_m3state_t *ms = (jn_m3state_t *)t->ms.a + b.first + i;
			ms->ent = (int32_t)(term0 + (int64_t)pend.n);
			ms->jlo = (int8_t)((m->jlo - 1) / 2);
			ms->jhi = (int8_t)((m->jhi - 1) / 2);
			const uint64_t *head = hget(&cls, shell_class(t->sp[s[0]].shell, t->sp[s[1]].shell, t->sp[s[2]].shell), 0, 0, 0);
			int cnt = 0;
			for (int64_t a = head ? (int64_t)*head : -1; a >= 0; a = next[a]) {
				const double S = s_coef(t, keys[a], s);
				if (!(fabs(S) > 1e-10)) continue;
				unsigned char rec[sizeof(jn_m3term_t) + sizeof(uint64_t)];
				jn_m3term_t tm = { S, 0, (KJABC(keys[a]) - 1) / 2 };
				memcpy(rec, &tm, sizeof tm);
				memcpy(rec + sizeof tm, &keys[a], sizeof(uint64_t));
				if (vpush(&pend, rec)) { free(next); hfree(&cls); free(keys); snprintf(err, errlen, "out of memory"); return -1; }
				cnt++;
			}
			if (cnt > 32767) { free(next); hfree(&cls); free(keys); snprintf(err, errlen, "too many coupled terms for one state"); return -1; }
			ms->nent = (int16_t)cnt;
		}
		free(next);
		hfree(&cls);
		free(keys);
	}
	/* slot key lists: sorted, unique */
	for (int s = 0; s < t->nslots; s++) {
		uint64_t *k = (uint64_t *)slot_keys[s].a;
		size_t n = slot_keys[s].n, u = 0;
		if (n) qsort(k, n, sizeof *k, cmp_u64);
		for (size_t i = 0; i < n; i++)
			if (!u || k[i] != k[u - 1]) k[u++] = k[i];
		b.skeys[s] = k;
		b.nskeys[s] = (int)u;
	}
	/* terms with their V index */
	for (size_t i = 0; i < pend.n; i++) {
		const unsigned char *rec = (const unsigned char *)pend.a + i * pend.es;
		jn_m3term_t tm;
		uint64_t k;
		memcpy(&tm, rec, sizeof tm);
		memcpy(&k, rec + sizeof tm, sizeof k);
		tm.v = (int32_t)find_key(b.skeys[tm.slot], b.nskeys[tm.slot], k);
		if (vpush(&t->terms, &tm)) { free(pend.a); snprintf(err, errlen, "out of memory"); return -1; }
	}
	free(pend.a);
	if (vpush(&t->bases, &b)) { snprintf(err, errlen, "out of memory"); return -1; }
	return (int)t->bases.n - 1;
}

void jn_t3plan_free(jn_t3plan_t *p)
{
	if (!p) return;
	free(p->info); free(p->tb); free(p->tb_info); free(p->ms); free(p->term); free(p->voff); free(p->vld); free(p->V);
	free(p->vrows); free(p->elem_pair); free(p->pair_seg); free(p->seg);
	free(p->conn_ket); free(p->conn_bra); free(p->conn_sign); free(p->pc); free(p->nc); free(p->lut);
	memset(p, 0, sizeof *p);
}

int jn_t3plan_build(jn_t3plan_t *p, const char *comb, const char *lists_dir, int Z, int N, int emax,
		    const char *jscheme_dir, char *err, size_t errlen)
{
	memset(p, 0, sizeof *p);
	t3build_t t;
	memset(&t, 0, sizeof t);
	kcache_t kc;
	memset(&kc, 0, sizeof kc);
	jfile_t J;
	memset(&J, 0, sizeof J);
	uint64_t *fkeys = NULL;                 /* the file's canonical coupled states, sorted */
	int64_t nfk = 0, nch = 0, *chsize = NULL, *choff = NULL;
	int32_t *fch = NULL, *floc = NULL, *fkid = NULL;
	double *vnd = NULL, *vdg = NULL;        /* V per channel: as read, and with the mirror of diagonal blocks */
	shell3_t *sh = NULL;
	sp3_t *sp = NULL;
	vec3_t tb = { 0 }, tbi = { 0 }, c0 = { 0 }, pcv = { 0 }, ncv = { 0 }, pairs = { 0 }, ebv = { 0 }, Vv = { 0 };
	tb.es = sizeof(jn_t3block_t); tbi.es = sizeof(int); c0.es = 3 * sizeof(int32_t); pcv.es = sizeof(jn_p3conn_t);
	ncv.es = sizeof(jn_nconn_t); pairs.es = 2 * sizeof(int32_t); ebv.es = 2 * sizeof(int); Vv.es = sizeof(double);
	t.bases.es = sizeof(basis3_t); t.ms.es = sizeof(jn_m3state_t); t.terms.es = sizeof(jn_m3term_t); t.lut.es = sizeof(int32_t);

	if (Z < 0 || N < 0 || Z + N < 3) TERR("the three-body transform needs at least three particles (Z=%d N=%d)", Z, N);
	if (emax < 0 || emax > MAX_EMAX) TERR("single-particle energy %d out of range (0..%d)", emax, MAX_EMAX);
	p->Z = Z; p->N = N; p->emax = emax;
	const int nsh = gj_shells(emax, NULL);
	sh = (shell3_t *)malloc(nsh * sizeof *sh);
	if (!sh) TERR("out of memory");
	gj_shells(emax, sh);
	const int nsp = sp_states(emax, sh, nsh, &sp);
	if (nsp < 0) TERR("out of memory");
	t.sp = sp; t.sh = sh;
	t.nslots = (3 * (2 * emax + 1) + 1) / 2 + 1;
	p->nslots = t.nslots;
	kc.dir = lists_dir; kc.norb = nsp / 2; kc.spst = sp; kc.files.es = sizeof(kfile_t *);

	if (read_jfile(&J, jscheme_dir, sh, nsh, err, errlen)) goto fail;
	p->file_states = J.ns;
	p->file_elements = J.ne;
	/* V over the file's canonical coupled states, both ways the reference
	   fills a block (read_3nf_ascii_format.c:410-425): rows b, columns k,
	   the last row wins; diagonal blocks also write the mirror.  A cut pairs
	   states of one (Jabc, Tz, parity) channel only, so V is held densely per
	   channel; rows across channels are never read. */
	fkeys = (uint64_t *)malloc((J.ns ? J.ns : 1) * sizeof(uint64_t));
	if (!fkeys) TERR("out of memory");
	memcpy(fkeys, J.key, J.ns * sizeof(uint64_t));
	qsort(fkeys, J.ns, sizeof(uint64_t), cmp_u64);
	for (int64_t i = 0; i < J.ns; i++)
		if (!nfk || fkeys[i] != fkeys[nfk - 1]) fkeys[nfk++] = fkeys[i];
	fch = (int32_t *)malloc((nfk ? nfk : 1) * sizeof(int32_t));
	floc = (int32_t *)malloc((nfk ? nfk : 1) * sizeof(int32_t));
	{
		/* channels in key order: (jabc, tz, parity) of the manager's shells */
		hmap_t chm = { 0 };
		vec3_t chn = { 0 };
		chn.es = sizeof(int64_t);
		for (int64_t i = 0; i < nfk && fch && floc; i++) {
			const uint64_t k = fkeys[i];
			const int tz = sh[KA(k)].tz + sh[KB(k)].tz + sh[KC(k)].tz, par = (sh[KA(k)].l + sh[KB(k)].l + sh[KC(k)].l) & 1;
			uint64_t *c = hget(&chm, (uint64_t)KJABC(k) * 64 + (uint64_t)(tz + 8) * 2 + par, 0, 1, (uint64_t)-1);
			if (!c) { hfree(&chm); free(chn.a); TERR("out of memory"); }
			if (*c == (uint64_t)-1) {
				int64_t z = 0;
				*c = chn.n;
				if (vpush(&chn, &z)) { hfree(&chm); free(chn.a); TERR("out of memory"); }
			}
			fch[i] = (int32_t)*c;
			floc[i] = (int32_t)((int64_t *)chn.a)[*c]++;
		}
		hfree(&chm);
		if (!fch || !floc) { free(chn.a); TERR("out of memory"); }
		nch = (int64_t)chn.n;
		chsize = (int64_t *)chn.a;
		choff = (int64_t *)malloc((nch + 1) * sizeof(int64_t));
		if (!choff) TERR("out of memory");
		choff[0] = 0;
		for (int64_t c = 0; c < nch; c++) choff[c + 1] = choff[c] + chsize[c] * chsize[c];
		vnd = (double *)calloc(choff[nch] ? choff[nch] : 1, sizeof(double));
		vdg = (double *)calloc(choff[nch] ? choff[nch] : 1, sizeof(double));
		fkid = (int32_t *)malloc((J.ns ? J.ns : 1) * sizeof(int32_t));
		if (!vnd || !vdg || !fkid) TERR("out of memory");
		for (int64_t i = 0; i < J.ns; i++) fkid[i] = (int32_t)find_key(fkeys, nfk, J.key[i]);
	}
	for (int64_t i = 0; i < J.ne; i++) {
		const int32_t kb = fkid[J.bra[i]], kk = fkid[J.ket[i]];
		if (fch[kb] != fch[kk]) continue;
		const double v = J.e[i] * (J.phase[J.bra[i]] * J.phase[J.ket[i]]);
		const int64_t o = choff[fch[kb]], n = chsize[fch[kb]];
		vnd[o + floc[kb] * n + floc[kk]] = v;
		vdg[o + floc[kb] * n + floc[kk]] = v;
		vdg[o + floc[kk] * n + floc[kb]] = v;
	}

	if (jn_read_me_blocks(comb, &p->info, &p->nblocks, err, errlen)) goto fail;
	int64_t nelem = 0;
	for (int i = 0; i < p->nblocks; i++) {
		const jn_meblock_info_t *b = &p->info[i];
		if (b->np + b->nn != 3) continue;
		jn_t3block_t d;
		memset(&d, 0, sizeof d);
		d.out = nelem;
		const int tz = b->nn - b->np;
		const int kEp = b->dp, kEn = b->dn, bEp = b->dp + b->dEp, bEn = b->dn + b->dEn;
		const int kb = build_basis(&t, &kc, tz, b->np ? kEp : 0, b->nn ? kEn : 0, err, errlen);
		if (kb < 0) goto fail;
		const int bb = build_basis(&t, &kc, tz, b->np ? bEp : 0, b->nn ? bEn : 0, err, errlen);
		if (bb < 0) goto fail;
		const basis3_t *KB = &((basis3_t *)t.bases.a)[kb], *BB = &((basis3_t *)t.bases.a)[bb];
		if (b->dMp + b->dMn != 0) TERR("matrix block %d changes total M by %d", b->id, b->dMp + b->dMn);
		int eb = -1;
		for (size_t q = 0; q < ebv.n && eb < 0; q++)
			if (((int *)ebv.a)[2 * q] == kb && ((int *)ebv.a)[2 * q + 1] == bb) eb = (int)q;
		if (eb < 0) {
			int pr[2] = { kb, bb };
			if (vpush(&ebv, pr)) TERR("out of memory");
			eb = (int)ebv.n - 1;
		}
		d.eb = eb;
		if (b->np == 3 || b->nn == 3) {
			const int sp_ = b->nn == 3;
			const int depth = sp_ ? b->dn : b->dp, dE = sp_ ? b->dEn : b->dEp, dM = sp_ ? b->dMn : b->dMp;
			const kfile_t *ann = kfile(&kc, sp_, 3, depth, err, errlen);
			const kfile_t *cre = ann ? kfile(&kc, sp_, 3, depth + dE, err, errlen) : NULL;
			if (!cre) goto fail;
			pairs.n = 0;
			if (kconnections(ann, cre, dM, &pairs)) TERR("out of memory");
			const uint64_t want = sp_ ? b->Nn : b->Np;
			if ((uint64_t)pairs.n != want)
				TERR("matrix block %d should have %llu connections but has %zu", b->id, (unsigned long long)want, pairs.n);
			d.conn = (int32_t)c0.n;
			for (size_t q = 0; q < pairs.n; q++) {
				const int32_t *pr = (const int32_t *)pairs.a + 2 * q;
				int32_t e[3] = { (int32_t)(KB->first + pr[0]), (int32_t)(BB->first + pr[1]), 1 };
				if (vpush(&c0, e)) TERR("out of memory");
			}
			d.kind = 0;
			d.count = (int64_t)pairs.n;
		} else {
			/* protons x neutrons, protons major (connection_list.c:108-147) */
			const kfile_t *pa = kfile(&kc, 0, b->np, b->dp, err, errlen);
			const kfile_t *pcr = pa ? kfile(&kc, 0, b->np, b->dp + b->dEp, err, errlen) : NULL;
			const kfile_t *na = pcr ? kfile(&kc, 1, b->nn, b->dn, err, errlen) : NULL;
			const kfile_t *ncr = na ? kfile(&kc, 1, b->nn, b->dn + b->dEn, err, errlen) : NULL;
			if (!ncr) goto fail;
			pairs.n = 0;
			if (kconnections(pa, pcr, b->dMp, &pairs)) TERR("out of memory");
			const int64_t npc = (int64_t)pairs.n;
			d.conn = (int32_t)pcv.n;
			for (size_t q = 0; q < pairs.n; q++) {
				const int32_t *pr = (const int32_t *)pairs.a + 2 * q;
				jn_p3conn_t c = { pr[0], pr[1], (int32_t)KB->lut, (int32_t)BB->lut, (int32_t)KB->nf->n, (int32_t)BB->nf->n };
				if (vpush(&pcv, &c)) TERR("out of memory");
			}
			pairs.n = 0;
			if (kconnections(na, ncr, b->dMn, &pairs)) TERR("out of memory");
			const int64_t nnc = (int64_t)pairs.n;
			d.nconn = (int32_t)ncv.n;
			for (size_t q = 0; q < pairs.n; q++) {
				const int32_t *pr = (const int32_t *)pairs.a + 2 * q;
				jn_nconn_t c = { pr[0], pr[1] };
				if (vpush(&ncv, &c)) TERR("out of memory");
			}
			if ((uint64_t)npc != b->Np || (uint64_t)nnc != b->Nn)
				TERR("matrix block %d should have %llu x %llu connections but has %lld x %lld", b->id,
				     (unsigned long long)b->Np, (unsigned long long)b->Nn, (long long)npc, (long long)nnc);
			d.kind = 1;
			d.nn = (int32_t)nnc;
			d.count = npc * nnc;
		}
		nelem += d.count;
		if (vpush(&tb, &d) || vpush(&tbi, &i)) TERR("out of memory");
	}
	if (pcv.n > 0x7fffffff || ncv.n > 0x7fffffff || c0.n > 0x7fffffff || t.ms.n > 0x7fffffff || t.terms.n > 0x7fffffff)
		TERR("too many connections or states");

	/* V per (energy block, slot): rows are the bra basis' coupled states,
	   columns the ket basis'; zero when the bases' parities differ */
	p->neb = (int)ebv.n;
	p->voff = (int64_t *)malloc((p->neb ? p->neb : 1) * t.nslots * sizeof(int64_t));
	p->vld = (int32_t *)malloc((p->neb ? p->neb : 1) * t.nslots * sizeof(int32_t));
	p->vrows = (int32_t *)malloc((p->neb ? p->neb : 1) * t.nslots * sizeof(int32_t));
	if (!p->voff || !p->vld || !p->vrows) TERR("out of memory");
	for (int e = 0; e < p->neb; e++) {
		const basis3_t *K = &((basis3_t *)t.bases.a)[((int *)ebv.a)[2 * e]];
		const basis3_t *B = &((basis3_t *)t.bases.a)[((int *)ebv.a)[2 * e + 1]];
		const int diag = K == B;
		for (int s = 0; s < t.nslots; s++) {
			p->voff[e * t.nslots + s] = -1;
			p->vld[e * t.nslots + s] = 0;
			p->vrows[e * t.nslots + s] = 0;
			if (K->parity != B->parity || !K->nskeys[s] || !B->nskeys[s]) continue;
			p->voff[e * t.nslots + s] = (int64_t)Vv.n;
			p->vld[e * t.nslots + s] = K->nskeys[s];
			p->vrows[e * t.nslots + s] = B->nskeys[s];
			const double *vt = diag ? vdg : vnd;
			int64_t *cid = (int64_t *)malloc((size_t)K->nskeys[s] * sizeof(int64_t));
			if (!cid) TERR("out of memory");
			for (int c = 0; c < K->nskeys[s]; c++) cid[c] = find_key(fkeys, nfk, K->skeys[s][c]);
			for (int r = 0; r < B->nskeys[s]; r++) {
				const int64_t rk = find_key(fkeys, nfk, B->skeys[s][r]);
				for (int c = 0; c < K->nskeys[s]; c++) {
					double x = 0.0;
					const int64_t ck = cid[c];
					if (rk >= 0 && ck >= 0 && fch[rk] == fch[ck])
						x = vt[choff[fch[rk]] + (int64_t)floc[rk] * chsize[fch[rk]] + floc[ck]];
					if (vpush(&Vv, &x)) { free(cid); TERR("out of memory"); }
				}
			}
			free(cid);
		}
		/* flops of the reference's dense D_M per M block and J_abc */
		for (int q = 0; q < K->nmb; q++) {
			const mblock_t *mk = &K->mb[q];
			const mblock_t *mbr = NULL;
			for (int r = 0; r < B->nmb; r++)
				if (B->mb[r].M == mk->M) mbr = &B->mb[r];
			if (!mbr || !mk->n || !mbr->n) continue;
			for (int s = 0; s < t.nslots; s++) {
				const double nk = K->nskeys[s], nb = B->nskeys[s];
				t.dense_flops += 2.0 * (nb * nk * (double)mk->n + nb * (double)mbr->n * (double)mk->n);
			}
		}
	}
	p->n3 = (int)tb.n;
	p->tb = (jn_t3block_t *)tb.a; tb.a = NULL;
	p->tb_info = (int *)tbi.a; tbi.a = NULL;
	p->nelem = nelem;
	p->nms = (int64_t)t.ms.n;
	p->ms = (jn_m3state_t *)t.ms.a; t.ms.a = NULL;
	p->nterm = (int64_t)t.terms.n;
	p->term = (jn_m3term_t *)t.terms.a; t.terms.a = NULL;
	p->nv = (int64_t)Vv.n;
	p->V = (double *)Vv.a; Vv.a = NULL;
	p->nconn0 = (int64_t)c0.n;
	p->conn_ket = (int32_t *)malloc((c0.n ? c0.n : 1) * sizeof(int32_t));
	p->conn_bra = (int32_t *)malloc((c0.n ? c0.n : 1) * sizeof(int32_t));
	p->conn_sign = (int32_t *)malloc((c0.n ? c0.n : 1) * sizeof(int32_t));
	if (!p->conn_ket || !p->conn_bra || !p->conn_sign) TERR("out of memory");
	for (size_t q = 0; q < c0.n; q++) {
		const int32_t *e = (const int32_t *)c0.a + 3 * q;
		p->conn_ket[q] = e[0]; p->conn_bra[q] = e[1]; p->conn_sign[q] = e[2];
	}
	p->npc = (int64_t)pcv.n; p->pc = (jn_p3conn_t *)pcv.a; pcv.a = NULL;
	p->nnc = (int64_t)ncv.n; p->nc = (jn_nconn_t *)ncv.a; ncv.a = NULL;
	p->nlut = (int64_t)t.lut.n; p->lut = (int32_t *)t.lut.a; t.lut.a = NULL;
	p->coupled_states = t.coupled;
	p->mblocks = t.mblocks;
	p->dense_flops = t.dense_flops;
	for (size_t i = 0; i < t.bases.n; i++) basis_free(&((basis3_t *)t.bases.a)[i]);
	free(t.bases.a); hfree(&t.cg);
	free(c0.a); free(pairs.a); free(ebv.a); free(sh); free(sp);
	free(fkeys); free(fch); free(floc); free(fkid); free(chsize); free(choff); free(vnd); free(vdg);
	jfile_free(&J);
	kcache_free(&kc);
	return 0;
fail:
	for (size_t i = 0; i < t.bases.n; i++) basis_free(&((basis3_t *)t.bases.a)[i]);
	free(t.bases.a); free(t.ms.a); free(t.terms.a); free(t.lut.a); hfree(&t.cg);
	free(tb.a); free(tbi.a); free(c0.a); free(pcv.a); free(ncv.a); free(pairs.a); free(ebv.a); free(Vv.a);
	free(sh); free(sp);
	free(fkeys); free(fch); free(floc); free(fkid); free(chsize); free(choff); free(vnd); free(vdg);
	jfile_free(&J);
	kcache_free(&kc);
	jn_t3plan_free(p);
	return -1;
}

/* ket state, bra state and sign of element i of three-body block blk */
static void t3_element_states(const jn_t3plan_t *p, int blk, int64_t i, int32_t *ket, int32_t *bra)
{
	const jn_t3block_t *b = &p->tb[blk];
	if (b->kind == 0) {
		*ket = p->conn_ket[b->conn + i];
		*bra = p->conn_bra[b->conn + i];
		return;
	}
	const int64_t kp = i / b->nn, kn = i - kp * b->nn;
	const jn_p3conn_t *c = &p->pc[b->conn + kp];
	const jn_nconn_t *n = &p->nc[b->nconn + kn];
	int32_t k = p->lut[c->ket_lut + (int64_t)c->p_ann * c->ket_nn + n->n_ann];
	int32_t r = p->lut[c->bra_lut + (int64_t)c->p_cre * c->bra_nn + n->n_cre];
	*ket = k < 0 ? -k - 1 : k;
	*bra = r < 0 ? -r - 1 : r;
}

static int cmp_block_eb(const void *a, const void *b, void *plan)
{
	const jn_t3plan_t *p = (const jn_t3plan_t *)plan;
	const int x = *(const int *)a, y = *(const int *)b;
	const int ex = p->tb[x].eb, ey = p->tb[y].eb;
	if (ex != ey) return ex < ey ? -1 : 1;
	return x - y;
}

/* Every element's inner sums sum_r S_ket,r V[v][v_r] depend on its energy
 * block, its ket state, the slot and the bra's row v only: they are computed
 * once per (energy block, ket) pair and slot, for every row (the reference
 * forms the same products as V S_ket, block_transform.c:147-356). */
int jn_t3plan_shared(jn_t3plan_t *p, char *err, size_t errlen)
{
	free(p->elem_pair); free(p->pair_seg); free(p->seg);
	p->elem_pair = NULL; p->pair_seg = NULL; p->seg = NULL;
	p->npairs = p->nseg = p->nT = 0;
	int32_t *stamp = (int32_t *)malloc((p->nms ? p->nms : 1) * sizeof(int32_t));
	int32_t *pid = (int32_t *)malloc((p->nms ? p->nms : 1) * sizeof(int32_t));
	int *order = (int *)malloc((p->n3 ? p->n3 : 1) * sizeof(int));
	int64_t pcap = 1024, npairs = 0;
	int32_t *pairs = (int32_t *)malloc(pcap * 2 * sizeof(int32_t));
	p->elem_pair = (int32_t *)malloc((p->nelem ? p->nelem : 1) * sizeof(int32_t));
	if (!stamp || !pid || !order || !pairs || !p->elem_pair) goto oom;
	for (int64_t i = 0; i < p->nms; i++) stamp[i] = -1;
	for (int b = 0; b < p->n3; b++) order[b] = b;
	qsort_r(order, (size_t)p->n3, sizeof(int), cmp_block_eb, p);
	/* pairs in order of first use, blocks grouped by energy block */
	for (int ob = 0; ob < p->n3; ob++) {
		const int blk = order[ob];
		const jn_t3block_t *b = &p->tb[blk];
		for (int64_t i = 0; i < b->count; i++) {
			int32_t ket, bra;
			t3_element_states(p, blk, i, &ket, &bra);
			if (ket < 0 || ket >= p->nms) { snprintf(err, errlen, "element state out of range"); goto fail; }
			if (stamp[ket] != b->eb) {
				stamp[ket] = b->eb;
				if (npairs == pcap) {
					pcap *= 2;
					int32_t *q = (int32_t *)realloc(pairs, pcap * 2 * sizeof(int32_t));
					if (!q) goto oom;
					pairs = q;
				}
				if (npairs >= 0x7fffffff) { snprintf(err, errlen, "too many (energy block, ket) pairs"); goto fail; }
				pairs[2 * npairs] = b->eb;
				pairs[2 * npairs + 1] = ket;
				pid[ket] = (int32_t)npairs++;
			}
			p->elem_pair[b->out + i] = pid[ket];
		}
	}
	/* segments: the ket's slots in term order, T laid out pair by pair */
	p->pair_seg = (int64_t *)malloc((size_t)(npairs + 1) * sizeof(int64_t));
	int64_t scap = npairs * 4 + 16, nseg = 0, nT = 0;
	p->seg = (jn_t3seg_t *)malloc((size_t)scap * sizeof(jn_t3seg_t));
	if (!p->pair_seg || !p->seg) goto oom;
	for (int64_t k = 0; k < npairs; k++) {
		const int eb = pairs[2 * k];
		const jn_m3state_t *K = &p->ms[pairs[2 * k + 1]];
		p->pair_seg[k] = nseg;
		for (int r = K->ent; r < K->ent + K->nent;) {
			const int slot = p->term[r].slot;
			int r1 = r;
			while (r1 < K->ent + K->nent && p->term[r1].slot == slot) r1++;
			if (nseg == scap) {
				scap *= 2;
				jn_t3seg_t *q = (jn_t3seg_t *)realloc(p->seg, (size_t)scap * sizeof(jn_t3seg_t));
				if (!q) goto oom;
				p->seg = q;
			}
			jn_t3seg_t *sg = &p->seg[nseg++];
			const int64_t off = p->voff[(int64_t)eb * p->nslots + slot];
			sg->term0 = r;
			sg->nterm = (int16_t)(r1 - r);
			sg->slot = (int16_t)slot;
			sg->eb = eb;
			sg->rows = off >= 0 ? p->vrows[(int64_t)eb * p->nslots + slot] : 0;
			sg->toff = off >= 0 ? nT : -1;
			nT += sg->rows;
			r = r1;
		}
	}
	p->pair_seg[npairs] = nseg;
	p->npairs = npairs;
	p->nseg = nseg;
	p->nT = nT;
	free(stamp); free(pid); free(order); free(pairs);
	return 0;
oom:
	snprintf(err, errlen, "out of memory");
fail:
	free(stamp); free(pid); free(order); free(pairs);
	free(p->elem_pair); free(p->pair_seg); free(p->seg);
	p->elem_pair = NULL; p->pair_seg = NULL; p->seg = NULL;
	return -1;
}
