/*
 * jn_mercury — drop-in for mercury_J_scheme_to_internal.x
 * (src/Mercury/programs/mercury_J_scheme_to_internal.c:65-398): same
 * command line (src/Mercury/arguments/arguments.c:88-199), same output
 * files (<output>/<id>_matrix_elements), computed on the GPU.
 *
 *   jn_mercury <combination file> <index list base directory> <output path>
 *              [--num-protons n] [--num-neutrons n] [--single-particle-energy e]
 *              [--two-particle-energy e] [--exclude-kinetic-energy] [--no-2nf]
 *              [--finished-blocks-file path] [--max-loaded-memory m]
 *              [--single-block] [--block-id n] [--LEC-CE x] ... [--LEC-C4 x]
 *              <interaction path 2nf> [interaction path 3nf]
 *
 * As the reference does:
 *  - one-body blocks are written as zeros; two-body blocks come from the
 *    Antoine file, or are zeros with --no-2nf, whose only interaction path
 *    is then the three-body one;
 *  - three-body blocks come from the J-scheme directory (the ASCII format:
 *    one .cnf, one .mat), grouped in energy blocks in the combination
 *    table's sorted order (combination_table.c:642-676, 760-770); energy
 *    blocks listed in the finished-blocks file (size_t indices, default
 *    ./finished_blocks) are skipped and every block written is appended;
 *  - --LEC-* and --max-loaded-memory act on the HDF5 format only, and
 *    --single-block / --block-id are read but unused, so all are accepted
 *    and have no effect.
 * The HDF5 J-scheme format needs a library this build does not have; a path
 * that is not a directory is reported as such.
 */
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include "../../include/jncsm.h"
#include "jn_transform.h"

static int is_int(const char *s)
{
	if (!s || !*s) return 0;
	if (*s == '-' || *s == '+') s++;
	for (; *s; s++) if (*s < '0' || *s > '9') return 0;
	return 1;
}

static void usage(const char *p)
{
	printf("Usage: %s <combination file path> <index list base directory> <output path> "
	       "[--num-protons <integer>] [--num-neutrons <integer>] [--single-particle-energy <integer>] "
	       "[--two-particle-energy <integer>] [--max-loaded-memory <integer>] [--single-block] "
	       "[--block-id <integer>] [--finished-blocks-file <filepath>] [--no-2nf] [--LEC-CE <float>] "
	       "[--LEC-CD <float>] [--LEC-C1 <float>] [--LEC-C3 <float>] [--LEC-C4 <float>] "
	       "<interaction path 2nf> [interaction path 3nf]\n", p);
}

static int write_zero_block(const char *dir, const jn_meblock_info_t *b)
{
	char path[8192];
	snprintf(path, sizeof path, "%s/%d_matrix_elements", dir, b->id);
	FILE *f = fopen(path, "wb");
	if (!f) { fprintf(stderr, "Could not open file %s for writing\n", path); return -1; }
	size_t hdr[2] = { (size_t)b->Nn, (size_t)b->Np };
	const size_t n = b->np && b->nn ? (size_t)(b->Np * b->Nn) : (size_t)(b->np ? b->Np : b->Nn);
	int bad = fwrite(hdr, sizeof(size_t), 2, f) != 2;
	double z[1024] = { 0 };
	for (size_t done = 0; !bad && done < n; done += 1024) {
		const size_t k = n - done < 1024 ? n - done : 1024;
		bad = fwrite(z, sizeof(double), k, f) != k;
	}
	if (fclose(f) || bad) { fprintf(stderr, "Could not write %s\n", path); return -1; }
	return 0;
}

static int write_elements(const char *dir, const jn_meblock_info_t *b, const double *x, size_t n)
{
	char path[8192];
	snprintf(path, sizeof path, "%s/%d_matrix_elements", dir, b->id);
	FILE *f = fopen(path, "wb");
	if (!f) { fprintf(stderr, "Could not open file %s for writing\n", path); return -1; }
	size_t hdr[2] = { (size_t)b->Nn, (size_t)b->Np };
	int bad = fwrite(hdr, sizeof(size_t), 2, f) != 2 || (n && fwrite(x, sizeof(double), n, f) != n);
	if (fclose(f) || bad) { fprintf(stderr, "Could not write %s\n", path); return -1; }
	return 0;
}

/* compare_matrix_block_settings (combination_table.c:725-757) on three-body rows */
static const jn_meblock_info_t *g_rows;
static int cmp_rows(const void *x, const void *y)
{
	const jn_meblock_info_t *a = &g_rows[*(const int *)x], *b = &g_rows[*(const int *)y];
	int d;
	if ((d = a->nn - b->nn)) return d;
	if ((d = b->dp - a->dp)) return d;
	if ((d = a->dEp - b->dEp)) return d;
	if ((d = b->dn - a->dn)) return d;
	if ((d = a->dEn - b->dEn)) return d;
	if ((d = a->dMp - b->dMp)) return d;
	if ((d = a->dMn - b->dMn)) return d;
	return *(const int *)x - *(const int *)y;      /* stable */
}

static int same_energy_block(const jn_meblock_info_t *a, const jn_meblock_info_t *b)
{
	return a->dp == b->dp && a->dEp == b->dEp && a->dn == b->dn && a->dEn == b->dEn && a->np == b->np && a->nn == b->nn;
}

static int three_body(const char *comb, const char *lists, const char *out, int Z, int N, int e1, const char *v3,
		      const char *finished_path, const jn_meblock_info_t *rows, int nrows)
{
	struct stat sb;
	if (stat(v3, &sb) || !S_ISDIR(sb.st_mode)) {
		fprintf(stderr, "%s: not a J-scheme directory (the HDF5 format is not part of this build)\n", v3);
		return -1;
	}
	jn_transform3 *t = NULL;
	if (jn_transform3_open(comb, lists, Z, N, e1, v3, &t) != JN_OK || jn_transform3_run(t, NULL) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		jn_transform3_close(t);
		return -1;
	}
	/* energy blocks in the reference's order */
	int *ord = (int *)malloc((nrows ? nrows : 1) * sizeof(int)), n3 = 0;
	for (int i = 0; i < nrows; i++)
		if (rows[i].np + rows[i].nn == 3) ord[n3++] = i;
	g_rows = rows;
	qsort(ord, n3, sizeof(int), cmp_rows);
	/* finished energy blocks (load_finished_blocks, mercury_J_scheme_to_internal.c:414-437) */
	size_t nfin = 0, *fin = NULL;
	FILE *f = fopen(finished_path, "rb");
	if (f) {
		fseek(f, 0, SEEK_END);
		nfin = (size_t)ftell(f) / sizeof(size_t);
		fseek(f, 0, SEEK_SET);
		fin = (size_t *)malloc((nfin ? nfin : 1) * sizeof(size_t));
		if (fread(fin, sizeof(size_t), nfin, f) != nfin) nfin = 0;
		fclose(f);
	}
	FILE *done = fopen(finished_path, "ab");
	if (!done) fprintf(stderr, "Could not open %s: %s\n", finished_path, strerror(errno));
	int rc = 0;
	double *buf = NULL;
	size_t cap = 0, eb = 0;
	for (int i = 0; i < n3 && !rc; eb++) {
		int j = i + 1;
		while (j < n3 && same_energy_block(&rows[ord[i]], &rows[ord[j]])) j++;
		int skip = 0;
		for (size_t q = 0; q < nfin && !skip; q++) skip = fin[q] == eb;
		if (!skip) {
			printf("Launching block %zu\n", eb);
			for (int q = i; q < j && !rc; q++) {
				const jn_meblock_info_t *b = &rows[ord[q]];
				size_t n = 0;
				if (jn_transform3_elements(t, b->id, NULL, 0, &n) != JN_OK) { rc = -1; break; }
				if (n > cap) { free(buf); cap = n; buf = (double *)malloc(cap * sizeof(double)); }
				if (jn_transform3_elements(t, b->id, buf, cap, &n) != JN_OK) { rc = -1; break; }
				rc = write_elements(out, b, buf, n);
			}
			if (!rc && done) {
				fwrite(&eb, sizeof(size_t), 1, done);
				fflush(done);
			}
			printf("Finished block %zu\n", eb);
		}
		i = j;
	}
	if (rc && !*jn_last_error()) fprintf(stderr, "three-body blocks failed\n");
	else if (rc) fprintf(stderr, "%s\n", jn_last_error());
	if (done) fclose(done);
	free(buf); free(fin); free(ord);
	jn_transform3_close(t);
	return rc;
}

int main(int argc, char **argv)
{
	if (argc < 4) { usage(argv[0]); return 0; }
	const char *comb = argv[1], *lists = argv[2], *out = argv[3], *v2 = NULL, *v3 = NULL;
	const char *finished = "finished_blocks";
	int Z = 0, N = 0, e1 = 0, e2 = 0, kinetic = 1, no2nf = 0, extra = 0;
	for (int i = 4; i < argc; i++) {
		const char *a = argv[i];
#define INTARG(name, var)                                                                        \
	if (!strcmp(a, name)) {                                                                  \
		if (i + 1 >= argc || !is_int(argv[i + 1])) {                                     \
			fprintf(stderr, name " takes integer values only\n");                    \
			return 1;                                                                \
		}                                                                                \
		var = atoi(argv[++i]);                                                           \
		continue;                                                                        \
	}
		int unused = 0;
		INTARG("--num-protons", Z);
		INTARG("--num-neutrons", N);
		INTARG("--single-particle-energy", e1);
		INTARG("--two-particle-energy", e2);
		INTARG("--block-id", unused);
#undef INTARG
		if (!strcmp(a, "--max-loaded-memory") || !strncmp(a, "--LEC-", 6)) {
			if (i + 1 >= argc) { fprintf(stderr, "%s takes a value\n", a); return 1; }
			i++;
			continue;
		}
		if (!strcmp(a, "--finished-blocks-file")) {
			if (i + 1 >= argc) { fprintf(stderr, "%s takes a value\n", a); return 1; }
			finished = argv[++i];
			continue;
		}
		if (!strcmp(a, "--exclude-kinetic-energy")) { kinetic = 0; continue; }
		if (!strcmp(a, "--no-2nf")) { no2nf = 1; continue; }
		if (!strcmp(a, "--single-block")) continue;
		if (!v2) v2 = a;
		else if (!v3) v3 = a;
		else extra = 1;
		(void)unused;
	}
	if (!v2 || extra) { usage(argv[0]); return 0; }
	if (no2nf) v3 = v2;
	printf("Mercury starts:\n");
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	jn_meblock_info_t *rows = NULL;
	int nrows = 0;
	char err[1024];
	if (jn_read_me_blocks(comb, &rows, &nrows, err, sizeof err)) { fprintf(stderr, "%s\n", err); return 1; }
	mkdir(out, 0755);
	if (!no2nf) {
		if (jn_transform_2nf(comb, lists, out, Z, N, e1, e2, v2, kinetic) != JN_OK) {
			fprintf(stderr, "%s\n", jn_last_error());
			free(rows);
			return 1;
		}
	} else {
		/* one-body and two-body blocks as zeros (generate_2nf_zero_matrix_blocks) */
		for (int i = 0; i < nrows; i++)
			if (rows[i].np + rows[i].nn <= 2 && write_zero_block(out, &rows[i])) { free(rows); return 1; }
	}
	if (v3 && three_body(comb, lists, out, Z, N, e1, v3, finished, rows, nrows)) { free(rows); return 1; }
	free(rows);
	clock_gettime(CLOCK_MONOTONIC, &t1);
	printf("Mercury ends after %lg µs\n", (t1.tv_sec - t0.tv_sec) * 1e6 + (t1.tv_nsec - t0.tv_nsec) * 1e-3);
	return 0;
}
