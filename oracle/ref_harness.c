/*
 * ref_harness.c — TEST INFRASTRUCTURE ONLY (the oracle; never a product path).
 *
 * Drives the reference JupiterNCSM code, compiled unchanged from its own
 * sources by oracle/Makefile into oracle/_ref/libref_minerva.so, through the
 * reference's own API:
 *
 *   ref_matvec_files   the shipped path: run_matrix_vector_multiplication
 *                      (src/Minerva/scheduler/scheduler.c:80-145) with the
 *                      Minerva memory manager re-reading every file.
 *   ref_mem_*          the reference kernels without file I/O: all index
 *                      lists, matrix-element blocks and vector blocks are
 *                      loaded once with the reference loaders, then each call
 *                      runs the reference multiplication_* kernels
 *                      (src/Minerva/matrix_vector_multiplication/
 *                      matrix_vector_multiplication.c:20-462) over the
 *                      evaluation order with the same OpenMP task farm and
 *                      per-thread output replicas as the shipped scheduler
 *                      (scheduler.c:97-137, vector_block.c:49-66, 145-155).
 *
 * Used by tests/ as the parity reference and by bench.py's CPU-baseline leg.
 */
#include <combination_table/combination_table.h>
#include <evaluation_order/evaluation_order.h>
#include <index_list/index_list.h>
#include <matrix_block/matrix_block.h>
#include <matrix_vector_multiplication/matrix_vector_multiplication.h>
#include <scheduler/scheduler.h>
#include <vector_block/vector_block.h>
#include <global_constants/global_constants.h>

#include <fcntl.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

static int quiet_begin(void)
{
	fflush(stdout);
	int saved = dup(1);
	int devnull = open("/dev/null", O_WRONLY);
	if (devnull >= 0) { dup2(devnull, 1); close(devnull); }
	return saved;
}

static void quiet_end(int saved)
{
	fflush(stdout);
	if (saved >= 0) { dup2(saved, 1); close(saved); }
}

/* y files in out_dir are read, accumulated into and rewritten, as Bacchus
 * expects (vector_block.c:49-99). */
int ref_matvec_files(const char *comb, const char *order, const char *lists_dir, const char *me_dir,
		     const char *in_dir, const char *out_dir, int Z, int N, double max_memory_bytes, int nthreads)
{
	if (nthreads > 0) omp_set_num_threads(nthreads);
	int saved = quiet_begin();
	combination_table_t table = new_combination_table(comb, (size_t)Z, (size_t)N);
	evaluation_order_t eo = read_evaluation_order(order, table);
	scheduler_t s = new_scheduler(eo, table, lists_dir, me_dir, (size_t)max_memory_bytes);
	run_matrix_vector_multiplication(out_dir, in_dir, s);
	free_scheduler(s);
	free_evaluation_order(eo);
	free_combination_table(table);
	quiet_end(saved);
	return 0;
}

/* ------------------------------------------------------------------ */
typedef struct {
	combination_table_t table;
	evaluation_order_t eo;
	size_t ninstr;
	evaluation_instruction_t *instr;
	size_t nids;
	index_list_t *lists;          /* by id */
	matrix_block_t *mes;          /* by id */
	size_t nblocks;
	size_t *block_offset;         /* by block id */
	size_t *block_len;
	vector_block_t *in;           /* by id */
	vector_block_t *out;          /* by id, one replica per thread */
	int nthreads;
	double **replica;             /* [thread * (nblocks+1) + id] */
	size_t dim;
} ref_mem_t;

void *ref_mem_open(const char *comb, const char *order, const char *lists_dir, const char *me_dir,
		   const char *zero_vec_dir, int Z, int N, int nthreads)
{
	if (nthreads > 0) omp_set_num_threads(nthreads);
	int saved = quiet_begin();
	ref_mem_t *c = calloc(1, sizeof *c);
	c->table = new_combination_table(comb, (size_t)Z, (size_t)N);
	c->eo = read_evaluation_order(order, c->table);
	c->ninstr = get_num_instructions(c->eo);
	c->instr = calloc(c->ninstr, sizeof *c->instr);
	evaluation_order_iterator_t it = get_evaluation_order_iterator(c->eo);
	for (size_t i = 0; has_next_instruction(it); i++) c->instr[i] = next_instruction(it);
	free_evaluation_order_iterator(it);
	c->nids = get_num_arrays(c->table) + 1;
	c->lists = calloc(c->nids, sizeof *c->lists);
	c->mes = calloc(c->nids, sizeof *c->mes);
	for (size_t i = 0; i < c->ninstr; i++) {
		evaluation_instruction_t *x = &c->instr[i];
		if (x->type == unload || x->type == unknown) continue;
		if (x->neutron_index != no_index && !c->lists[x->neutron_index])
			c->lists[x->neutron_index] = new_index_list_from_id(lists_dir, x->neutron_index);
		if (x->proton_index != no_index && !c->lists[x->proton_index])
			c->lists[x->proton_index] = new_index_list_from_id(lists_dir, x->proton_index);
		if (!c->mes[x->matrix_element_file])
			c->mes[x->matrix_element_file] = new_matrix_block(x->matrix_element_file, me_dir);
	}
	c->nblocks = get_num_basis_blocks(c->table);
	c->block_offset = calloc(c->nblocks + 1, sizeof(size_t));
	c->block_len = calloc(c->nblocks + 1, sizeof(size_t));
	c->in = calloc(c->nblocks + 1, sizeof *c->in);
	c->out = calloc(c->nblocks + 1, sizeof *c->out);
	size_t off = 0;
	for (size_t b = 1; b <= c->nblocks; b++) {
		basis_block_t bb = get_basis_block(c->table, b);
		c->block_offset[b] = off;
		c->block_len[b] = bb.num_proton_states * bb.num_neutron_states;
		off += c->block_len[b];
		c->in[b] = new_vector_block(zero_vec_dir, bb);
	}
	c->dim = off;
#pragma omp parallel
	{
#pragma omp single
		{
			c->nthreads = omp_get_num_threads();
			c->replica = calloc((size_t)c->nthreads * (c->nblocks + 1), sizeof(double *));
			for (size_t b = 1; b <= c->nblocks; b++)
				c->out[b] = new_output_vector_block(zero_vec_dir, get_basis_block(c->table, b));
		}
		int t = omp_get_thread_num();
		for (size_t b = 1; b <= c->nblocks; b++)
			c->replica[(size_t)t * (c->nblocks + 1) + b] = get_vector_block_elements(c->out[b]);
	}
	quiet_end(saved);
	return c;
}

static void run_instr(ref_mem_t *c, const evaluation_instruction_t *x)
{
	size_t bi = x->vector_block_in, bo = x->vector_block_out;
	matrix_block_t me = c->mes[x->matrix_element_file];
	if (bi == bo) {
		/* scheduler.c:264-345 */
		if (x->type == neutron_block)
			multiplication_neutrons(c->out[bo], c->in[bi], me, c->lists[x->neutron_index]);
		else if (x->type == proton_block)
			multiplication_protons(c->out[bo], c->in[bi], me, c->lists[x->proton_index]);
		else
			multiplication_neutrons_protons(c->out[bo], c->in[bi], me, c->lists[x->neutron_index],
							c->lists[x->proton_index]);
	} else {
		/* scheduler.c:347-418: left = (in x_in -> out y_out), right = transpose */
		if (x->type == neutron_block)
			multiplication_neutrons_off_diag(c->out[bo], c->out[bi], c->in[bi], c->in[bo], me,
							 c->lists[x->neutron_index]);
		else if (x->type == proton_block)
			multiplication_protons_off_diag(c->out[bo], c->out[bi], c->in[bi], c->in[bo], me,
							c->lists[x->proton_index]);
		else
			multiplication_neutrons_protons_off_diag(c->out[bo], c->out[bi], c->in[bi], c->in[bo], me,
								 c->lists[x->neutron_index],
								 c->lists[x->proton_index]);
	}
}

/* y = y + H x over the whole vector (block-concatenated layout). Returns the
 * wall time of the kernel region in seconds (copy-in/out excluded). */
double ref_mem_matvec(void *handle, const double *x, double *y)
{
	ref_mem_t *c = handle;
	for (size_t b = 1; b <= c->nblocks; b++)
		memcpy(get_vector_block_elements(c->in[b]), x + c->block_offset[b], c->block_len[b] * sizeof(double));
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	size_t next = 0;
#pragma omp parallel
	{
		int t = omp_get_thread_num();
		for (size_t b = 1; b <= c->nblocks; b++)
			memset(c->replica[(size_t)t * (c->nblocks + 1) + b], 0, c->block_len[b] * sizeof(double));
#pragma omp barrier
		for (;;) {
			size_t i;
#pragma omp atomic capture
			i = next++;
			if (i >= c->ninstr) break;
			const evaluation_instruction_t *x = &c->instr[i];
			if (x->type == unload || x->type == unknown) continue;
			run_instr(c, x);
		}
	}
	clock_gettime(CLOCK_MONOTONIC, &t1);
	for (size_t b = 1; b <= c->nblocks; b++)
		for (int t = 0; t < c->nthreads; t++) {
			const double *r = c->replica[(size_t)t * (c->nblocks + 1) + b];
			double *yo = y + c->block_offset[b];
			for (size_t e = 0; e < c->block_len[b]; e++) yo[e] += r[e];
		}
	return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

size_t ref_mem_dimension(void *handle) { return ((ref_mem_t *)handle)->dim; }
int ref_mem_threads(void *handle) { return ((ref_mem_t *)handle)->nthreads; }

void ref_mem_close(void *handle)
{
	ref_mem_t *c = handle;
	if (!c) return;
	for (size_t i = 0; i < c->nids; i++) {
		if (c->lists[i]) free_index_list(c->lists[i]);
		if (c->mes[i]) free_matrix_block(c->mes[i]);
	}
	for (size_t b = 1; b <= c->nblocks; b++) { free_vector_block(c->in[b]); free_vector_block(c->out[b]); }
	free(c->lists); free(c->mes); free(c->in); free(c->out); free(c->replica);
	free(c->block_offset); free(c->block_len); free(c->instr);
	free_evaluation_order(c->eo);
	free_combination_table(c->table);
	free(c);
}
