/*
 * jn_bacchus — drop-in for the reference's bacchus.x on one GB300.
 *
 * Same command line (src/Bacchus/settings/settings.c:27-65:
 * [--settings-file <file>.conf] [--max-memory-load <size>] [--help]), same
 * run file, same results channel: the final eigensystem block on stdout in
 * print_eigensystem's format (src/Bacchus/eigensystem/eigensystem.c:99-113)
 * and eigenvectors 1..target_eigenvector+1 written as
 * <eigenvector_directory>/eigenvector_<i>/vec_<block>
 * (src/Bacchus/programs/bacchus.c:68-87).  The Krylov vectors stay in GPU
 * memory, so krylow_vector_directory is not written.
 *
 * By default the solver follows the reference's algorithm (start vector e_0,
 * partial reorthogonalisation, convergence of the lowest Ritz value); the
 * optional run-file group `gpu { reorthogonalize = "full"; }` selects full
 * reorthogonalisation with a residual-bound test on gpu.num_eigenvalues.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/jncsm.h"

static double now_us(void)
{
	struct timespec t;
	clock_gettime(CLOCK_REALTIME, &t);
	return t.tv_sec * 1e6 + t.tv_nsec * 1e-3;
}

static int ends_with(const char *s, const char *suffix)
{
	size_t a = strlen(s), b = strlen(suffix);
	return a >= b && strcmp(s + a - b, suffix) == 0;
}

int main(int argc, char **argv)
{
	const char *conf = "bacchus.conf";
	double t0 = now_us();
	printf("Bacchus starts:\n");
	for (int i = 1; i < argc; i++) {
		if (!strcmp(argv[i], "--settings-file") && i + 1 < argc) {
			conf = argv[++i];
			if (!ends_with(conf, ".conf")) {
				fprintf(stderr, "\"%s\" is not a settings file, the filename must end in .conf\n", conf);
				return EXIT_FAILURE;
			}
		} else if (!strcmp(argv[i], "--max-memory-load") && i + 1 < argc) {
			i++; /* everything is resident in GPU memory: accepted and ignored */
		} else if (!strcmp(argv[i], "--help") || !strcmp(argv[i], "-h")) {
			printf("Usage: %s [--settings-file <file>.conf] [--max-memory-load <size>]\n", argv[0]);
			return EXIT_FAILURE;
		} else {
			fprintf(stderr, "Unknown argument \"%s\"\n", argv[i]);
			return EXIT_FAILURE;
		}
	}
	jn_run_settings rs;
	if (jn_read_settings(conf, &rs) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	jn_ctx *ctx = NULL;
	if (jn_open(conf, &ctx) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	if (rs.gpu_precision == 32 && jn_set_precision(ctx, 32) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	jn_lanczos_options o;
	memset(&o, 0, sizeof o);
	o.max_iterations = rs.max_num_lanczos_iterations;
	o.num_eigenvalues = rs.gpu_num_eigenvalues;
	if (o.num_eigenvalues < rs.target_eigenvector + 1) o.num_eigenvalues = rs.target_eigenvector + 1;
	o.tolerance = rs.convergence_tolerance;
	o.mode = rs.gpu_full_reorthogonalization ? JN_LANCZOS_FULL : JN_LANCZOS_REFERENCE;
	o.check_every = 1;
	o.verbose = 0;
	o.criterion = rs.converge_eigenvectors ? JN_CONVERGE_EIGENVECTORS : JN_CONVERGE_EIGENVALUES;
	printf("Diagonalzation start:\n");
	double td = now_us();
	jn_lanczos_result r;
	jn_status st = jn_lanczos(ctx, &o, &r);
	if (st != JN_OK && st != JN_ERR_NOT_CONVERGED) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	printf("Diagonalization end after %lg \xc2\xb5s\n", now_us() - td);
	double *ritz = malloc((r.num_ritz_values + 1) * sizeof(double));
	int n = 0;
	if (jn_lanczos_ritz_values(ctx, ritz, r.num_ritz_values, &n) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	jn_print_eigensystem(ritz, n);
	if (jn_lanczos_save_eigenvectors(ctx, rs.eigenvector_directory, rs.target_eigenvector + 1) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	free(ritz);
	jn_close(ctx);
	printf("Bacchus ends after %lg \xc2\xb5s\n", now_us() - t0);
	return EXIT_SUCCESS;
}
