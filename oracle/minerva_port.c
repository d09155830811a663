/*
 * minerva_port.c — TEST INFRASTRUCTURE ONLY (the oracle; never a product path).
 *
 * A plain, single-threaded C restatement of the reference's index-list block
 * matrix-vector product, used by tests/ as the checker for the CUDA path and
 * pinned against the compiled reference (oracle/_ref, ref_harness.c).  It
 * reads the same files and applies the instructions strictly in evaluation
 * order, so its summation order is fixed.
 *
 * Followed reference code (paths relative to the reference src/ tree):
 *   comb.txt ARRAYMP / Conn-lists rows   Utilities/combination_table/combination_table.c:419-522
 *   evaluation-order rows                Minerva/evaluation_order/evaluation_order.c:175-243
 *   index_list_<id> records              Minerva/index_list/index_list.c:69-97
 *   <id>_matrix_elements                 Minerva/matrix_block/matrix_block.c:22-62
 *   sign bit / index mask                Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:7-18
 *   n / p / np kernels (diagonal)        matrix_vector_multiplication.c:20-210
 *   off-diagonal kernels (+ transpose)   matrix_vector_multiplication.c:212-462
 *   diagonal vs off-diagonal dispatch    Minerva/scheduler/scheduler.c:194-246
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <time.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int32_t in, out, mi; } triple_t;

typedef struct {
	int kind;                 /* 1 neutron, 2 proton, 3 neutron-proton */
	long bin, bout, ln, lp, me;
} instr_t;

typedef struct {
	long nids;
	long *np, *nn;            /* basis block dims by id (0 if not a block) */
	long nblocks;
	size_t *offset;           /* vector offset by block id */
	char *ltype;              /* 'n' / 'p' by list id */
	triple_t **lists; size_t *llen;
	double **mes; size_t *me_nd;   /* neutron matrix dimension */
	instr_t *ins; long nins;
	size_t dim;
} port_t;

static int words(char *s, char **w, int maxw)
{
	int n = 0;
	while (*s && n < maxw) {
		while (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r') s++;
		if (!*s) break;
		w[n++] = s;
		while (*s && *s != ' ' && *s != '\t' && *s != '\n' && *s != '\r') s++;
		if (*s) *s++ = 0;
	}
	return n;
}

static long idval(const char *s) { return strtol(s, NULL, 10); } /* "12=" -> 12 */

static void grow(port_t *p, long id)
{
	if (id < p->nids) return;
	long n = id + 1024;
	p->np = realloc(p->np, n * sizeof(long)); p->nn = realloc(p->nn, n * sizeof(long));
	p->ltype = realloc(p->ltype, n);
	p->offset = realloc(p->offset, n * sizeof(size_t));
	for (long i = p->nids; i < n; i++) { p->np[i] = p->nn[i] = 0; p->ltype[i] = 0; p->offset[i] = 0; }
	p->nids = n;
}

void port_close(void *h);

void *port_open(const char *comb, const char *order, const char *lists_dir, const char *me_dir)
{
	port_t *p = calloc(1, sizeof *p);
	FILE *f = fopen(comb, "r");
	if (!f) { free(p); return NULL; }
	char line[4096], *w[32];
	int section = 0;
	while (fgets(line, sizeof line, f)) {
		if (strstr(line, "***")) {
			section = strstr(line, "mp-states") ? 1 : strstr(line, "Conn lists") ? 2 :
				  strstr(line, "Matrix-elements") ? 3 : 0;
			continue;
		}
		if (section == 3 && strstr(line, "ARRAY:")) {
			/* matrix-element ids share the id space: make room for them */
			char *a = strstr(line, "ARRAY:") + 6;
			grow(p, strtol(a, NULL, 10));
			continue;
		}
		if (section == 1 && strstr(line, "ARRAYMP:")) {
			int n = words(line, w, 32);
			if (n < 10) continue;
			long id = idval(w[9]);
			grow(p, id);
			p->np[id] = atol(w[4]); p->nn[id] = atol(w[5]);
			p->nblocks++;
		} else if (section == 2 && strstr(line, "ARRAY:")) {
			int n = words(line, w, 32);
			if (n < 10) continue;
			long id = idval(w[9]);
			grow(p, id);
			p->ltype[id] = w[0][0];
		}
	}
	fclose(f);
	size_t off = 0;
	for (long b = 1; b <= p->nblocks; b++) { p->offset[b] = off; off += (size_t)(p->np[b] * p->nn[b]); }
	p->dim = off;
	p->lists = calloc(p->nids, sizeof *p->lists); p->llen = calloc(p->nids, sizeof(size_t));
	p->mes = calloc(p->nids, sizeof *p->mes); p->me_nd = calloc(p->nids, sizeof(size_t));
	f = fopen(order, "r");
	if (!f) { port_close(p); return NULL; }
	long cap = 0;
	while (fgets(line, sizeof line, f)) {
		char *b = strstr(line, "BLOCK:");
		if (!b || strstr(line, "UNLOAD_")) continue;
		int n = words(b, w, 32);
		instr_t x = { 0, atol(w[1]), atol(w[2]), -1, -1, 0 };
		if (n == 6) {
			long l1 = atol(w[3]), l2 = atol(w[4]);
			x.me = atol(w[5]);
			x.kind = 3;
			if (p->ltype[l1] == 'n') { x.ln = l1; x.lp = l2; } else { x.ln = l2; x.lp = l1; }
		} else {
			long l = atol(w[3]);
			x.me = atol(w[4]);
			if (p->ltype[l] == 'n') { x.kind = 1; x.ln = l; } else { x.kind = 2; x.lp = l; }
		}
		if (p->nins == cap) { cap = cap ? 2 * cap : 256; p->ins = realloc(p->ins, cap * sizeof(instr_t)); }
		p->ins[p->nins++] = x;
	}
	fclose(f);
	char path[4096];
	for (long i = 0; i < p->nins; i++) {
		long ids[2] = { p->ins[i].ln, p->ins[i].lp };
		for (int q = 0; q < 2; q++) {
			long id = ids[q];
			if (id < 0 || p->lists[id]) continue;
			snprintf(path, sizeof path, "%s/index_list_%ld", lists_dir, id);
			FILE *g = fopen(path, "rb");
			if (!g) { port_close(p); return NULL; }
			fseek(g, 0, SEEK_END); long nb = ftell(g); fseek(g, 0, SEEK_SET);
			p->llen[id] = (size_t)nb / 12;
			p->lists[id] = malloc(nb ? (size_t)nb : 1);
			if (fread(p->lists[id], 12, p->llen[id], g) != p->llen[id]) { fclose(g); port_close(p); return NULL; }
			fclose(g);
		}
		long me = p->ins[i].me;
		if (p->mes[me]) continue;
		snprintf(path, sizeof path, "%s/%ld_matrix_elements", me_dir, me);
		FILE *g = fopen(path, "rb");
		if (!g) { port_close(p); return NULL; }
		size_t hdr[2];
		if (fread(hdr, sizeof(size_t), 2, g) != 2) { fclose(g); port_close(p); return NULL; }
		size_t len = hdr[0] == 0 ? hdr[1] : hdr[1] == 0 ? hdr[0] : hdr[0] * hdr[1];
		p->me_nd[me] = hdr[0];
		p->mes[me] = malloc(len ? len * sizeof(double) : 1);
		if (fread(p->mes[me], sizeof(double), len, g) != len) { fclose(g); port_close(p); return NULL; }
		fclose(g);
	}
	return p;
}

size_t port_dimension(void *h) { return ((port_t *)h)->dim; }
long port_num_instructions(void *h) { return ((port_t *)h)->nins; }

static inline int sgn(int32_t mi) { return (mi & (int32_t)0x80000000) ? -1 : 1; }
static inline size_t idx(int32_t mi) { return (size_t)(mi & 0x7FFFFFFF); }

static void apply_instr(const port_t *p, const instr_t *I, const double *x, double *y);

/* y += H x, instructions applied in evaluation-order sequence */
void port_matvec(void *h, const double *x, double *y)
{
	port_t *p = h;
	for (long i = 0; i < p->nins; i++) apply_instr(p, &p->ins[i], x, y);
}

/*
 * y += H x with the reference's parallel scheme: an OpenMP task farm over
 * the instructions (Minerva/scheduler/scheduler.c:97-137, lock-guarded
 * fetch evaluation_order.c:138-161) writing into one output replica per
 * thread, reduced at the end (Minerva/vector_block/vector_block.c:49-66,
 * 145-155).  Returns the wall time of the parallel region in seconds.
 */
double port_matvec_omp(void *h, const double *x, double *y, int nthreads)
{
	port_t *p = h;
	if (nthreads > 0) omp_set_num_threads(nthreads);
	int T = omp_get_max_threads();
	double *rep = calloc((size_t)T * p->dim + 1, sizeof(double));
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	long next = 0;
#pragma omp parallel
	{
		double *mine = rep + (size_t)omp_get_thread_num() * p->dim;
		for (;;) {
			long i;
#pragma omp atomic capture
			i = next++;
			if (i >= p->nins) break;
			apply_instr(p, &p->ins[i], x, mine);
		}
#pragma omp barrier
#pragma omp for schedule(static)
		for (long e = 0; e < (long)p->dim; e++) {
			double s = 0.0;
			for (int t = 0; t < omp_get_num_threads(); t++) s += rep[(size_t)t * p->dim + e];
			y[e] += s;
		}
	}
	clock_gettime(CLOCK_MONOTONIC, &t1);
	free(rep);
	return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

static void apply_instr(const port_t *p, const instr_t *I, const double *x, double *y)
{
	{
		const int diag = I->bin == I->bout;
		const long Np_i = p->np[I->bin], Nn_i = p->nn[I->bin], Nn_o = p->nn[I->bout];
		const double *xi = x + p->offset[I->bin], *xo = x + p->offset[I->bout];
		double *yo = y + p->offset[I->bout], *yi = y + p->offset[I->bin];
		const double *M = p->mes[I->me];
		if (I->kind == 1) {
			const triple_t *L = p->lists[I->ln];
			for (size_t e = 0; e < p->llen[I->ln]; e++) {
				double m = M[idx(L[e].mi)];
				if (fabs(m) < 1e-12) continue;
				double sm = sgn(L[e].mi) * m;
				for (long q = 0; q < Np_i; q++) {
					size_t oi = (size_t)L[e].out + (size_t)Nn_o * q, ii = (size_t)L[e].in + (size_t)Nn_i * q;
					yo[oi] += sm * xi[ii];
					if (!diag) yi[ii] += sm * xo[oi];
				}
			}
		} else if (I->kind == 2) {
			const triple_t *L = p->lists[I->lp];
			for (size_t e = 0; e < p->llen[I->lp]; e++) {
				double m = M[idx(L[e].mi)];
				if (fabs(m) < 1e-12) continue;
				double sm = sgn(L[e].mi) * m;
				for (long n = 0; n < Nn_i; n++) {
					size_t oi = (size_t)Nn_i * L[e].out + n, ii = (size_t)Nn_i * L[e].in + n;
					yo[oi] += sm * xi[ii];
					if (!diag) yi[ii] += sm * xo[oi];
				}
			}
		} else {
			const triple_t *Ln = p->lists[I->ln], *Lp = p->lists[I->lp];
			const size_t nd = p->me_nd[I->me];
			for (size_t a = 0; a < p->llen[I->ln]; a++)
				for (size_t b = 0; b < p->llen[I->lp]; b++) {
					size_t ii = (size_t)Ln[a].in + (size_t)Nn_i * Lp[b].in;
					size_t oi = (size_t)Ln[a].out + (size_t)Nn_o * Lp[b].out;
					double sm = (double)(sgn(Ln[a].mi) * sgn(Lp[b].mi)) * M[idx(Ln[a].mi) + nd * idx(Lp[b].mi)];
					yo[oi] += sm * xi[ii];
					if (!diag) yi[ii] += sm * xo[oi];
				}
		}
	}
}

void port_close(void *h)
{
	port_t *p = h;
	if (!p) return;
	for (long i = 0; i < p->nids; i++) {
		if (p->lists && p->lists[i]) free(p->lists[i]);
		if (p->mes && p->mes[i]) free(p->mes[i]);
	}
	free(p->lists); free(p->llen); free(p->mes); free(p->me_nd);
	free(p->np); free(p->nn); free(p->ltype); free(p->offset); free(p->ins);
	free(p);
}
