/*
 * oracle/ref_mercury3.c — test infrastructure only.
 *
 * Drives the reference's own J->M three-body transform, compiled unchanged
 * from src/Mercury, src/Neptune and src/Utilities, through its API, as
 * generate_3nf_matrix_blocks_parallel does
 * (src/Mercury/programs/mercury_J_scheme_to_internal.c:306-398), one energy
 * block after another: get_transformed_block decouples every total-M block
 * of the energy block, get_3nf_mercury_matrix reads each matrix block's
 * elements, save_mercury_matrix_block writes <id>_matrix_elements.
 *
 * The J-scheme input is the reference's ASCII format, opened with its own
 * open_ascii_data (src/Neptune/input/read_3nf_ascii_format.c:197-279).  The
 * format dispatcher read_3nf_file.c cannot be compiled here (it includes the
 * HDF5 reader, and hdf5.h is absent), so its ASCII branches are restated:
 * open_data_file's ASCII case, get_matrix -> get_matrix_ascii, and
 * is_subset_of_basis -> 1 (src/Neptune/input/read_3nf_file.c:12-44, 81-122).
 *
 * usage: ref_mercury3 <comb.txt> <index list dir> <output dir> <Z> <N>
 *                     <single-particle energy> <J-scheme directory>
 * prints the wall time of the transform in seconds.
 */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include <combination_table/combination_table.h>
#include <input/read_3nf_ascii_format.h>
#include <input/read_3nf_file.h>
#include <matrix_energy_block/matrix_energy_block.h>
#include <mercury_matrix_block/mercury_matrix_block.h>
#include <transform_3nf_block_manager/transform_3nf_block_manager.h>
#include <transformed_block/transformed_block.h>

Dens_Matrix *get_matrix(Data_File *data_file, void *m_basis, void *n_basis)
{
	if (data_file->signature != ASCII) {
		fprintf(stderr, "ref_mercury3: only the ASCII format is built\n");
		exit(3);
	}
	return get_matrix_ascii((ASCII_Data *)data_file->data_pointer, m_basis, n_basis);
}

int is_subset_of_basis(JJJ_Basis *j_scheme, Data_File *data_file)
{
	(void)j_scheme; (void)data_file;
	return 1;
}

/* the interaction tables need HDF5; nothing on this path calls them */
double get_matrix_element(interaction_t interaction, int *bra_state, int *ket_state, size_t num_particles, int E1, int E2,
			  int Tz, int M)
{
	(void)interaction; (void)bra_state; (void)ket_state; (void)num_particles; (void)E1; (void)E2; (void)Tz; (void)M;
	fprintf(stderr, "ref_mercury3: interaction tables are not built\n");
	exit(3);
}

int main(int argc, char **argv)
{
	if (argc < 8) {
		fprintf(stderr, "usage: %s comb index_list_dir out Z N e_single jscheme_dir\n", argv[0]);
		return 2;
	}
	const char *comb = argv[1], *lists = argv[2], *out = argv[3];
	int Z = atoi(argv[4]), N = atoi(argv[5]), e1 = atoi(argv[6]);
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	ASCII_Data *ascii = open_ascii_data(argv[7]);
	if (!ascii) {
		fprintf(stderr, "ref_mercury3: could not open %s\n", argv[7]);
		return 1;
	}
	Data_File data = { ASCII, ascii, 0 };
	combination_table_t table = new_combination_table(comb, Z, N);
	transform_3nf_block_manager_t manager = new_transform_3nf_block_manager(&data, lists, e1);
	size_t nblocks = 0;
	while (has_next_3nf_matrix_energy_block(table)) {
		matrix_energy_block_t eb = next_3nf_matrix_energy_block(table);
		transformed_block_t tb = get_transformed_block(manager, eb);
		while (has_next_energy_matrix_block(eb)) {
			matrix_block_setting_t s = next_energy_matrix_block(eb);
			mercury_matrix_block_t m = get_3nf_mercury_matrix(tb, s);
			save_mercury_matrix_block(m, out);
			free_mercury_matrix_block(m);
			nblocks++;
		}
		free_transformed_block(tb);
		free_matrix_energy_block(eb);
	}
	free_transform_3nf_block_manager(manager);
	free_combination_table(table);
	clock_gettime(CLOCK_MONOTONIC, &t1);
	fprintf(stderr, "ref_mercury3: %zu three-body blocks\n", nblocks);
	printf("%.6f\n", (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
	return 0;
}
