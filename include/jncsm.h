/*
 * jncsm.h — C ABI of libjncsm_gpu.so, the GB300 (sm_103a) implementation of
 * JupiterNCSM's hot path: the index-list block matrix-vector product that
 * Bacchus' Lanczos solver applies every iteration, and the Lanczos solve
 * around it.
 *
 * Every call returns a jn_status and never exits the process; the message of
 * the last failure on the calling thread is jn_last_error().  Buffers are
 * caller-owned.  A context is used by one host thread at a time.
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the reference's src/ tree).
 */
#ifndef JNCSM_H
#define JNCSM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
	JN_OK = 0,
	JN_ERR_INVALID = 1,     /* bad argument */
	JN_ERR_IO = 2,          /* a file could not be opened / read / written */
	JN_ERR_FORMAT = 3,      /* malformed or inconsistent input files */
	JN_ERR_CUDA = 4,        /* CUDA runtime error or no usable GPU */
	JN_ERR_NOMEM = 5,       /* host or device allocation failed */
	JN_ERR_NOT_CONVERGED = 6,
	JN_ERR_TIMEOUT = 7      /* a bounded device-side wait gave up */
} jn_status;

typedef struct jn_ctx jn_ctx;

/* Message of the last failure of a jn_* call on this thread. */
const char *jn_last_error(void);

/* Library version string. */
const char *jn_version(void);

/*
 * Open a Hamiltonian described by a Bacchus run file: reads the combination
 * table, evaluation order, every index list and every matrix-element block
 * once, validates all indices, and uploads them to the current CUDA device.
 * Replaces parse_settings + new_combination_table + read_evaluation_order +
 * new_generative_matrix (Bacchus/settings/settings.c:27-214,
 * Utilities/combination_table/combination_table.c:83-137,
 * Minerva/evaluation_order/evaluation_order.c:43-112,
 * Bacchus/matrix/matrix.c:52-66).
 */
jn_status jn_open(const char *bacchus_conf, jn_ctx **ctx);

/* The same from explicit paths (Z protons, N neutrons). */
jn_status jn_open_files(const char *combination_table_file, const char *evaluation_order_file,
			const char *index_lists_base_directory, const char *matrix_file_base_directory,
			int num_protons, int num_neutrons, jn_ctx **ctx);

void jn_close(jn_ctx *ctx);

/* Full M-scheme dimension D = sum_b Np_b * Nn_b
 * (Utilities/combination_table/combination_table.c:139-147). */
size_t jn_dimension(const jn_ctx *ctx);

/* Number of basis blocks; block b (0-based) has id, offset into the full
 * vector and length Np*Nn. */
int jn_num_blocks(const jn_ctx *ctx);
jn_status jn_block_info(const jn_ctx *ctx, int b, int *id, size_t *offset, size_t *length);

/*
 * y += H x with FP64 vectors in HOST memory (copied in and out inside the
 * call).  Replaces run_matrix_vector_multiplication
 * (Minerva/scheduler/scheduler.c:80-145), whose output blocks are also
 * accumulated into (Minerva/vector_block/vector_block.c:49-99).
 * Deterministic: the same inputs give bit-identical y.
 */
jn_status jn_matvec(jn_ctx *ctx, const double *x, double *y);

/* y += H x (accumulate = 1) or y = H x (accumulate = 0) on DEVICE pointers,
 * enqueued on `stream` (a cudaStream_t, NULL for the context's stream). */
jn_status jn_matvec_device(jn_ctx *ctx, const double *d_x, double *d_y, int accumulate, void *stream);

/*
 * File-level drop-in for run_matrix_vector_multiplication(out_dir, in_dir, ...):
 * reads in_dir/vec_<id> and out_dir/vec_<id>, adds H x to the latter and
 * writes it back (Minerva/vector_block/vector_block.c:28-99, 136-155).
 */
jn_status jn_matvec_files(jn_ctx *ctx, const char *output_vector_directory, const char *input_vector_directory);

/* y (+)= H x on device pointers, on the context's stream, with CUDA events
 * around each of the two kernels of the product; waits for completion and
 * returns their durations in milliseconds (ms[0] the gather-multiply kernel,
 * ms[1] the ordered reduction).  Used for roofline accounting. */
jn_status jn_matvec_profile(jn_ctx *ctx, const double *d_x, double *d_y, int accumulate, float ms[2]);

/* Synchronise the context's stream. */
jn_status jn_synchronize(jn_ctx *ctx);

/* Plan statistics.  algorithmic_bytes is the compulsory traffic of one
 * product: every index list once in the reference's 12-byte record format,
 * every matrix element some list pair indexes (8 bytes), x read and y
 * written (16 bytes per basis state).  multiply_adds counts both directions
 * of off-diagonal instructions. */
typedef struct {
	size_t dimension;
	int num_blocks;
	int num_instructions;
	size_t list_entries;
	size_t me_elements;
	size_t me_referenced;
	double multiply_adds;
	double algorithmic_bytes;
	int num_work_units;
	int num_tiles;
} jn_plan_stats;
jn_status jn_get_plan_stats(const jn_ctx *ctx, jn_plan_stats *stats);

/* The same statistics from the files alone, on the host (no GPU needed):
 * parses and validates the problem exactly as jn_open_files does. */
jn_status jn_inspect_files(const char *combination_table_file, const char *evaluation_order_file,
			   const char *index_lists_base_directory, const char *matrix_file_base_directory,
			   int num_protons, int num_neutrons, jn_plan_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
