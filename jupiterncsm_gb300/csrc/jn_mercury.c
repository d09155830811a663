/*
 * jn_mercury — drop-in for the two-body part of mercury_J_scheme_to_internal.x
 * (src/Mercury/programs/mercury_J_scheme_to_internal.c:65-202): same
 * command line (src/Mercury/arguments/arguments.c:88-160), same output
 * files (<output>/<id>_matrix_elements), computed on the GPU.
 *
 *   jn_mercury <combination file> <index list base directory> <output path>
 *              [--num-protons n] [--num-neutrons n] [--single-particle-energy e]
 *              [--two-particle-energy e] [--exclude-kinetic-energy]
 *              <interaction path 2nf>
 *
 * The three-body path of the reference (an HDF5 J-scheme reader and the
 * JJJ transform) is not part of this build: a second interaction path or
 * --no-2nf is rejected with a message.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/jncsm.h"

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
	       "[--two-particle-energy <integer>] [--exclude-kinetic-energy] <interaction path 2nf>\n", p);
}

int main(int argc, char **argv)
{
	if (argc < 5) { usage(argv[0]); return 0; }
	const char *comb = argv[1], *lists = argv[2], *out = argv[3], *v2 = NULL;
	int Z = 0, N = 0, e1 = 0, e2 = 0, kinetic = 1;
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
		INTARG("--num-protons", Z);
		INTARG("--num-neutrons", N);
		INTARG("--single-particle-energy", e1);
		INTARG("--two-particle-energy", e2);
#undef INTARG
		if (!strcmp(a, "--exclude-kinetic-energy")) { kinetic = 0; continue; }
		if (!strcmp(a, "--no-2nf") || (v2 && a[0] != '-')) {
			fprintf(stderr, "%s: the three-body transform is not part of this build\n", argv[0]);
			return 1;
		}
		if (a[0] == '-') { fprintf(stderr, "%s: unknown option %s\n", argv[0], a); return 1; }
		v2 = a;
	}
	if (!v2) { usage(argv[0]); return 0; }
	printf("Mercury starts:\n");
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	jn_status s = jn_transform_2nf(comb, lists, out, Z, N, e1, e2, v2, kinetic);
	if (s != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return 1;
	}
	clock_gettime(CLOCK_MONOTONIC, &t1);
	printf("Mercury ends after %lg µs\n", (t1.tv_sec - t0.tv_sec) * 1e6 + (t1.tv_nsec - t0.tv_nsec) * 1e-3);
	return 0;
}
