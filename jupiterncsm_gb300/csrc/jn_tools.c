/*
 * jn_tools.c — host-side drop-ins for the reference's file tools around the
 * product: Anicre index-list conversion (Aurora), evaluation-order
 * scheduling (Mars) and operator sums (Vulcan).  They read the combination
 * table the way src/Utilities/combination_table/combination_table.c:473-640
 * does and write the reference's file formats unchanged.
 */
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "../../include/jncsm.h"

/* the library's failure recorder (jn_matvec.cu) */
jn_status jn_fail(jn_status s, const char *fmt, ...);

typedef struct {
	char type[8];
	int Ebra, Mbra, Eket, Mket, depth;
	long id;
} tl_list;

typedef struct {
	char type[8];           /* neutron part then proton part, e.g. "nnp", "p" */
	unsigned long long nn, np;      /* neutron and proton combinations */
	long id;
} tl_me;

typedef struct {
	int nparticles;
	unsigned long long mults;
	long in, out, l1, l2, me;       /* l2 = 0: single list */
	long row;               /* position in comb.txt */
} tl_calc;

typedef struct {
	tl_list *l; long nl;
	tl_me *m; long nm;
	tl_calc *c; long nc;
} tl_table;

static void table_free(tl_table *t)
{
	free(t->l); free(t->m); free(t->c);
	memset(t, 0, sizeof *t);
}

static int words(char *s, char **w, int maxw)
{
	int n = 0;
	char *save = NULL;
	for (char *tok = strtok_r(s, " \t\r\n", &save); tok && n < maxw; tok = strtok_r(NULL, " \t\r\n", &save)) w[n++] = tok;
	return n;
}

/* "63=" -> 63 */
static long id_of(const char *s) { return strtol(s, NULL, 10); }

#define GROW(arr, n, cap) do { if ((n) == (cap)) { (cap) = (cap) ? 2 * (cap) : 256; (arr) = realloc((arr), (cap) * sizeof *(arr)); } } while (0)

static jn_status read_table(const char *path, tl_table *t)
{
	memset(t, 0, sizeof *t);
	FILE *f = fopen(path, "r");
	if (!f) return jn_fail(JN_ERR_IO, "Could not open \"%s\". %s", path, strerror(errno));
	char *line = NULL, *w[40];
	size_t cap = 0;
	long cl = 0, cm = 0, cc = 0, row = 0;
	int section = 0;        /* 2 conn lists, 3 cross, 4 same, 5 calc blocks */
	jn_status st = JN_OK;
	while (!st && getline(&line, &cap, f) >= 0) {
		row++;
		if (strstr(line, "***")) {
			section = strstr(line, "Conn lists") ? 2 : strstr(line, "Matrix-elements V (cross p-n)") ? 3 :
				  strstr(line, "Matrix-elements V (same p/n)") ? 4 : strstr(line, "Calc blocks") ? 5 : 0;
			continue;
		}
		char *calc = strstr(line, "CALCBLOCK:");
		if (calc) {
			/* "<word> <mults> # CALCBLOCK:<n>: in, out, l1[, l2], me" (calculation_blocks.c:31-84) */
			tl_calc c = { 0 };
			c.row = row;
			char *p = calc;
			while (p > line && (p[-1] == ' ' || p[-1] == '\t')) p--;
			while (p > line && p[-1] != ' ' && p[-1] != '\t') p--;     /* the '#' */
			while (p > line && (p[-1] == ' ' || p[-1] == '\t')) p--;
			while (p > line && p[-1] != ' ' && p[-1] != '\t') p--;     /* the count */
			if (sscanf(p, "%llu", &c.mults) != 1 ||
			    (sscanf(calc, "CALCBLOCK:%d: %ld, %ld, %ld, %ld, %ld", &c.nparticles, &c.in, &c.out, &c.l1, &c.l2, &c.me) != 6 &&
			     (c.l2 = 0, sscanf(calc, "CALCBLOCK:%d: %ld, %ld, %ld, %ld", &c.nparticles, &c.in, &c.out, &c.l1, &c.me) != 5))) {
				st = jn_fail(JN_ERR_FORMAT, "CALCBLOCK \"%s\" is not formatted correctly", calc);
				break;
			}
			GROW(t->c, t->nc, cc);
			t->c[t->nc++] = c;
			continue;
		}
		if (!strstr(line, "ARRAY:")) continue;
		int n = words(line, w, 40);
		if (section == 2 && n >= 10) {
			GROW(t->l, t->nl, cl);
			tl_list *l = &t->l[t->nl++];
			snprintf(l->type, sizeof l->type, "%s", w[0]);
			l->Ebra = atoi(w[1]); l->Mbra = atoi(w[2]); l->Eket = atoi(w[3]); l->Mket = atoi(w[4]);
			l->depth = atoi(w[5]);
			l->id = id_of(w[9]);
		} else if (section == 3 && n >= 14) {
			GROW(t->m, t->nm, cm);
			tl_me *m = &t->m[t->nm++];
			snprintf(m->type, sizeof m->type, "%s%s", w[4], w[0]);
			m->np = strtoull(w[8], NULL, 10);
			m->nn = strtoull(w[9], NULL, 10);
			m->id = id_of(w[13]);
		} else if (section == 4 && n >= 9) {
			GROW(t->m, t->nm, cm);
			tl_me *m = &t->m[t->nm++];
			snprintf(m->type, sizeof m->type, "%s", w[0]);
			const unsigned long long comb = strtoull(w[4], NULL, 10);
			m->np = w[0][0] == 'p' ? comb : 0;
			m->nn = w[0][0] == 'p' ? 0 : comb;
			m->id = id_of(w[8]);
		} else if (section >= 2 && section <= 4) {
			st = jn_fail(JN_ERR_FORMAT, "malformed row %ld of %s", row, path);
		}
	}
	free(line);
	fclose(f);
	if (st) table_free(t);
	return st;
}

/* ------------------------------------------------------------------ */
/* Aurora                                                              */
/* ------------------------------------------------------------------ */
static jn_status read_anicre_list(const char *path, int human_readable, int32_t **out, size_t *n)
{
	*out = NULL;
	*n = 0;
	FILE *f = fopen(path, "r");
	if (!f) return jn_fail(JN_ERR_IO, "Could not open file %s. %s", path, strerror(errno));
	jn_status st = JN_OK;
	if (!human_readable) {
		fseek(f, 0, SEEK_END);
		const long bytes = ftell(f);
		fseek(f, 0, SEEK_SET);
		if (bytes < 0 || bytes % 12) {
			st = jn_fail(JN_ERR_FORMAT, "The file %s does not include index triples", path);
		} else {
			*n = (size_t)bytes / 12;
			*out = malloc(bytes ? (size_t)bytes : 1);
			if (*n && fread(*out, 12, *n, f) != *n) st = jn_fail(JN_ERR_IO, "Could not read %ld bytes from file %s", bytes, path);
		}
	} else {
		/* rows "in out <sign>k" (src/Aurora/index_list/index_list.c:21-66); the sign goes to bit 31 of k */
		size_t cap = 0;
		char *line = NULL;
		size_t lcap = 0, r = 0;
		while (getline(&line, &lcap, f) >= 0) {
			r++;
			int i, j, k;
			char sign;
			if (sscanf(line, "%d %d %c%d", &i, &j, &sign, &k) != 4 || k < 0) {
				st = jn_fail(JN_ERR_FORMAT, "Could not parse row %zu in file %s", r, path);
				break;
			}
			if (*n == cap) { cap = cap ? 2 * cap : 1024; *out = realloc(*out, cap * 12); }
			(*out)[3 * *n] = i;
			(*out)[3 * *n + 1] = j;
			(*out)[3 * *n + 2] = (int32_t)((uint32_t)k | (sign == '-' ? 0x80000000u : 0u));
			(*n)++;
		}
		free(line);
	}
	fclose(f);
	if (st) { free(*out); *out = NULL; *n = 0; }
	return st;
}

jn_status jn_aurora(const char *comb, const char *anicre_dir, const char *output_dir, int Z, int N, int human_readable,
		    int skip_three_body, int *converted)
{
	(void)Z; (void)N;       /* the reference reads them for the table; the list rows do not depend on them */
	if (!comb || !anicre_dir || !output_dir) return jn_fail(JN_ERR_INVALID, "null argument");
	tl_table t;
	jn_status st = read_table(comb, &t);
	if (st) return st;
	mkdir(output_dir, 0755);
	int done = 0;
	for (long q = 0; q < t.nl && !st; q++) {
		const tl_list *L = &t.l[q];
		if (skip_three_body && strlen(L->type) == 3) continue;
		char path[8192];
		snprintf(path, sizeof path, "%s/%s_inds_index_lists/index_list_E_in%d_E_out%d_M_in%d_M_out%d_dE%d_dM%d_depth%d",
			 anicre_dir, L->type, L->Ebra, L->Eket, L->Mbra, L->Mket, L->Eket - L->Ebra, L->Mket - L->Mbra, L->depth);
		int32_t *tri;
		size_t n;
		struct stat sb;
		/* as aurora.x: a list Anicre did not write is reported and skipped */
		if (stat(path, &sb) != 0) {
			fprintf(stderr, "Could not open file %s. %s\n", path, strerror(errno));
			continue;
		}
		if ((st = read_anicre_list(path, human_readable, &tri, &n))) break;
		snprintf(path, sizeof path, "%s/index_list_%ld", output_dir, L->id);
		FILE *f = fopen(path, "wb");
		if (!f) st = jn_fail(JN_ERR_IO, "Could not open file %s. %s", path, strerror(errno));
		else {
			if (n && fwrite(tri, 12, n, f) != n) st = jn_fail(JN_ERR_IO, "Could not write indices to file %s", path);
			fclose(f);
		}
		free(tri);
		done++;
	}
	table_free(&t);
	if (converted) *converted = done;
	return st;
}

/* ------------------------------------------------------------------ */
/* Mars                                                                */
/* ------------------------------------------------------------------ */
static int cmp_calc(const void *a, const void *b)
{
	const tl_calc *x = a, *y = b;
	if (x->out != y->out) return x->out < y->out ? -1 : 1;
	if (x->in != y->in) return x->in < y->in ? -1 : 1;
	if (x->mults != y->mults) return x->mults > y->mults ? -1 : 1;
	return x->row < y->row ? -1 : x->row > y->row;
}

jn_status jn_mars(const char *comb, int Z, int N, const char *output_file, int two_body_only, int *num_rows)
{
	(void)Z; (void)N;
	if (!comb || !output_file) return jn_fail(JN_ERR_INVALID, "null argument");
	tl_table t;
	jn_status st = read_table(comb, &t);
	if (st) return st;
	/* one-body blocks are zero and skipped; two-body only keeps two-particle blocks (mars.c:92-170) */
	long n = 0;
	for (long q = 0; q < t.nc; q++)
		if (t.c[q].nparticles == 2 || (!two_body_only && t.c[q].nparticles == 3)) t.c[n++] = t.c[q];
	/* the order of the panel engine's schedule: by output block, then input block, largest first */
	qsort(t.c, n, sizeof *t.c, cmp_calc);
	FILE *f = fopen(output_file, "w");
	if (!f) st = jn_fail(JN_ERR_IO, "Could not open %s. %s", output_file, strerror(errno));
	for (long q = 0; q < n && !st; q++) {
		const tl_calc *c = &t.c[q];
		if (c->l2) fprintf(f, "BLOCK: %ld %ld %ld %ld %ld\n", c->in, c->out, c->l1, c->l2, c->me);
		else fprintf(f, "BLOCK: %ld %ld %ld %ld\n", c->in, c->out, c->l1, c->me);
	}
	if (f && fclose(f) != 0 && !st) st = jn_fail(JN_ERR_IO, "Could not write %s", output_file);
	table_free(&t);
	if (num_rows) *num_rows = (int)n;
	return st;
}

/* ------------------------------------------------------------------ */
/* Vulcan                                                              */
/* ------------------------------------------------------------------ */
jn_status jn_vulcan(const char *comb, int Z, int N, int num_operators, const char *const *operator_dirs,
		    const double *coefficients, const char *output_dir)
{
	(void)Z; (void)N;
	if (!comb || !output_dir || num_operators < 0 || (num_operators && (!operator_dirs || !coefficients)))
		return jn_fail(JN_ERR_INVALID, "null argument");
	tl_table t;
	jn_status st = read_table(comb, &t);
	if (st) return st;
	mkdir(output_dir, 0755);
	size_t maxlen = 1;
	for (long q = 0; q < t.nm; q++) {
		const tl_me *m = &t.m[q];
		const size_t len = m->nn && m->np ? m->nn * m->np : m->nn + m->np;
		if (len > maxlen) maxlen = len;
	}
	double *acc = malloc(maxlen * sizeof(double)), *in = malloc(maxlen * sizeof(double));
	if (!acc || !in) st = jn_fail(JN_ERR_NOMEM, "out of host memory for blocks of %zu elements", maxlen);
	for (long q = 0; q < t.nm && !st; q++) {
		const tl_me *m = &t.m[q];
		/* get_matrix_block_length (src/Utilities/matrix_block_setting/matrix_block_setting.c:3-23) */
		const size_t len = m->nn && m->np ? m->nn * m->np : m->nn + m->np;
		memset(acc, 0, len * sizeof(double));
		char path[8192];
		for (int i = 0; i < num_operators && !st; i++) {
			snprintf(path, sizeof path, "%s/%ld_matrix_elements", operator_dirs[i], m->id);
			FILE *f = fopen(path, "rb");
			if (!f) continue;       /* an absent block is zero (vulcan.c:153-176) */
			if (fseek(f, 2 * (long)sizeof(uint64_t), SEEK_SET) || fread(in, sizeof(double), len, f) != len)
				st = jn_fail(JN_ERR_IO, "Could not read block %ld from operator %s", m->id, operator_dirs[i]);
			fclose(f);
			const double c = coefficients[i];
			for (size_t j = 0; j < len && !st; j++) acc[j] += c * in[j];
		}
		if (st) break;
		snprintf(path, sizeof path, "%s/%ld_matrix_elements", output_dir, m->id);
		FILE *f = fopen(path, "wb");
		if (!f) { st = jn_fail(JN_ERR_IO, "Could not open %s. %s", path, strerror(errno)); break; }
		const uint64_t hdr[2] = { m->nn, m->np };
		if (fwrite(hdr, sizeof(uint64_t), 2, f) != 2 || fwrite(acc, sizeof(double), len, f) != len)
			st = jn_fail(JN_ERR_IO, "Could not write matrix block %ld to %s", m->id, output_dir);
		fclose(f);
	}
	free(acc); free(in);
	table_free(&t);
	return st;
}
