/*
 * ref_bacchus.c — TEST INFRASTRUCTURE ONLY (the oracle; never a product path).
 *
 * The reference's Bacchus eigensolver, compiled unchanged from its own
 * sources by oracle/Makefile into oracle/_ref/ref_bacchus, driven through
 * its own API exactly as its main program does
 * (src/Bacchus/programs/bacchus.c:23-102): combination table, evaluation
 * order, the file-backed generative matrix (the Minerva scheduler),
 * new_lanczos_environment / diagonalize / get_eigensystem, the eigensystem
 * block on stdout and the eigenvector directories.  Two things stand in for
 * what this image lacks: the run file's values come from the command line
 * instead of the libconfig-based reader (src/Bacchus/settings/settings.c),
 * and LAPACK's dsteqr_/dsyev_ are scipy's bundled OpenBLAS build of the
 * same routines (renamed at compile time).
 *
 * Usage: ref_bacchus comb order lists_dir me_dir Z N krylov_dir
 *                    max_iterations tolerance criterion eigenvector_dir target
 * criterion: 0 converge the lowest eigenvalue, 1 its eigenvector
 * (src/Bacchus/lanczos/lanczos.h:11-16).  The last line printed is
 * "ref_bacchus: <dimension of the final eigensystem>".
 */
#include <combination_table/combination_table.h>
#include <evaluation_order/evaluation_order.h>
#include <lanczos/lanczos.h>
#include <matrix/matrix.h>
#include <eigensystem/eigensystem.h>
#include <vector/vector.h>

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char **argv)
{
	if (argc != 13) {
		fprintf(stderr, "usage: %s comb order lists_dir me_dir Z N krylov_dir max_iterations tolerance criterion "
				"eigenvector_dir target\n", argv[0]);
		return EXIT_FAILURE;
	}
	const size_t Z = strtoul(argv[5], NULL, 10), N = strtoul(argv[6], NULL, 10);
	combination_table_t table = new_combination_table(argv[1], Z, N);
	evaluation_order_t order = read_evaluation_order(argv[2], table);
	lanczos_settings_t ls = {
		.dimension = get_full_dimension(table),
		.vector_settings = setup_vector_settings(table),
		.krylow_vectors_directory_name = strdup(argv[7]),
		.max_num_iterations = strtoul(argv[8], NULL, 10),
		.eigenvalue_tolerance = strtod(argv[9], NULL),
		.convergence_critera = atoi(argv[10]) ? converge_eigenvectors : converge_eigenvalues,
		.target_eigenvalue = 0,
		.matrix = new_generative_matrix(order, table, argv[3], argv[4], (size_t)64e9),
	};
	lanczos_environment_t env = new_lanczos_environment(ls);
	diagonalize(env);
	eigensystem_t es = get_eigensystem(env);
	print_eigensystem(es);
	const char *eigvec_dir = argv[11];
	const size_t target = strtoul(argv[12], NULL, 10);
	for (size_t i = 0; i <= target; i++) {
		vector_settings_t vs = ls.vector_settings;
		vs.directory_name = calloc(strlen(eigvec_dir) + 256, 1);
		sprintf(vs.directory_name, "%s/eigenvector_%lu", eigvec_dir, (unsigned long)(i + 1));
		vector_t v = new_zero_vector(vs);
		get_eigenvector(v, es, i);
		save_vector(v);
		free_vector(v);
		free(vs.directory_name);
	}
	printf("ref_bacchus: %lu\n", (unsigned long)get_num_eigenvalues(es));
	free_eigensystem(es);
	free_lanczos_environment(env);
	free_matrix(ls.matrix);
	free_evaluation_order(order);
	free_combination_table(table);
	free(ls.krylow_vectors_directory_name);
	return EXIT_SUCCESS;
}
