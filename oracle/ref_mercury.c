/*
 * oracle/ref_mercury.c — test infrastructure only.
 *
 * Drives the reference's own J->M two-body transform, compiled unchanged
 * from src/Mercury, src/Neptune and src/Utilities, through its API, as the
 * reference program does in generate_1nf_matrix_blocks and
 * generate_2nf_matrix_blocks (src/Mercury/programs/mercury_J_scheme_to_internal.c:108-202):
 * zero one-body blocks, then every two-body block of the combination
 * table, decoupling a new (energies, Tz) block only when the settings
 * change (transform_block_settings.c:4-38).  Writes <id>_matrix_elements
 * files into the output directory and prints the wall time in seconds.
 *
 * usage: ref_mercury <comb.txt> <index list dir> <output dir> <Z> <N>
 *                    <single-particle energy> <two-particle energy> <antoine file> [exclude-kinetic]
 */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include <combination_table/combination_table.h>
#include <connection_list/connection_list.h>
#include <input/read_2nf_antoine_format.h>
#include <mercury_matrix_block/mercury_matrix_block.h>
#include <single_particle_basis/single_particle_basis.h>
#include <transform_2nf_block_manager/transform_2nf_block_manager.h>
#include <transform_block_settings/transform_block_settings.h>

/* The 3NF reader and the interaction tables need HDF5, which is absent;
 * nothing on the two-body path calls these. */
void *get_matrix(void *data_file, void *m_basis, void *n_basis)
{
	(void)data_file; (void)m_basis; (void)n_basis;
	fprintf(stderr, "ref_mercury: the 3NF reader is not built\n");
	exit(3);
}
double get_matrix_element(interaction_t interaction, int *bra_state, int *ket_state, size_t num_particles, int E1,
			  int E2, int Tz, int M)
{
	(void)interaction; (void)bra_state; (void)ket_state; (void)num_particles; (void)E1; (void)E2; (void)Tz; (void)M;
	fprintf(stderr, "ref_mercury: interaction tables are not built\n");
	exit(3);
}

int main(int argc, char **argv)
{
	if (argc < 9) {
		fprintf(stderr, "usage: %s comb index_list_dir out Z N e1 e2 antoine [exclude-kinetic]\n", argv[0]);
		return 2;
	}
	const char *comb = argv[1], *lists = argv[2], *out = argv[3];
	int Z = atoi(argv[4]), N = atoi(argv[5]), e1 = atoi(argv[6]), e2 = atoi(argv[7]);
	const char *antoine = argv[8];
	int kinetic = !(argc > 9 && atoi(argv[9]));
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	combination_table_t table = new_combination_table(comb, Z, N);
	single_particle_basis_t sp = new_antoine_single_particle_basis(e1);
	while (has_next_1nf_block(table)) {
		matrix_block_setting_t b = next_1nf_block_iterator(table);
		connection_list_t c = new_connection_list(lists, sp, b);
		mercury_matrix_block_t m = new_zero_mercury_matrix_block(c);
		save_mercury_matrix_block(m, out);
		free_mercury_matrix_block(m);
		free_connection_list(c);
	}
	antoine_2nf_file_t data = open_antoine_2nf_file(antoine, Z + N, e1, e2, kinetic);
	transform_2nf_block_manager_t manager = new_transform_2nf_block_manager(data, lists, lists, e1);
	transform_block_settings_t done = { INT_MAX };
	size_t nblocks = 0;
	while (has_next_2nf_block(table)) {
		matrix_block_setting_t b = next_2nf_block_iterator(table);
		transform_block_settings_t cur = setup_transform_block(b);
		if (compare_transform_block_settings(&done, &cur) != 0) {
			decouple_transform_2nf_block(manager, cur);
			done = cur;
		}
		mercury_matrix_block_t m = get_transform_2nf_matrix_block(manager, b);
		save_mercury_matrix_block(m, out);
		free_mercury_matrix_block(m);
		nblocks++;
	}
	free_transform_2nf_block_manager(manager);
	free_antoine_2nf_file(data);
	free_single_particle_basis(sp);
	free_combination_table(table);
	clock_gettime(CLOCK_MONOTONIC, &t1);
	printf("blocks %zu seconds %.6f\n", nblocks, (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
	return 0;
}
