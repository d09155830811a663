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
 * The host plans are built on all cores (at most 32 threads; the
 * environment variable JN_HOST_THREADS caps them), and the results do not
 * depend on the number of threads.
 * Replaces parse_settings + new_combination_table + read_evaluation_order +
 * new_generative_matrix (Bacchus/settings/settings.c:27-214,
 * Utilities/combination_table/combination_table.c:83-137,
 * Minerva/evaluation_order/evaluation_order.c:43-112,
 * Bacchus/matrix/matrix.c:52-66).
 */
jn_status jn_open(const char *bacchus_conf, jn_ctx **ctx);

/* The Bacchus run file (libconfig syntax) as the reference reads it
 * (Bacchus/settings/settings.c:79-211), plus an optional `gpu` group that the
 * reference ignores: gpu.num_eigenvalues, gpu.precision ("fp64"/"fp32"),
 * gpu.reorthogonalize ("full"/"partial"). */
typedef struct {
	char combination_table_file[4096];
	char evaluation_order_file[4096];
	char index_lists_base_directory[4096];
	char matrix_file_base_directory[4096];
	int num_protons, num_neutrons;
	char krylow_vector_directory[4096];
	int max_num_lanczos_iterations;
	double convergence_tolerance;
	int target_eigenvector;
	int converge_eigenvectors;
	char eigenvector_directory[4096];
	int gpu_num_eigenvalues;
	int gpu_precision;              /* 64 or 32 */
	int gpu_full_reorthogonalization;
} jn_run_settings;
jn_status jn_read_settings(const char *bacchus_conf, jn_run_settings *settings);

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
 * Range: every product but engine 2's at precision 64 sums in 64-bit fixed
 * point, with x bounded in FP32.  It is exact to FP64 level while
 * max|x| < 2^127 and abs_bound * max|x| lies in [2^-47, 2^121), where
 * abs_bound bounds |H| row sums (a normalised vector, as in Lanczos, is
 * always inside).  Outside that range this call returns JN_ERR_INVALID
 * instead of a wrong result; x = 0 is always accepted.
 */
jn_status jn_matvec(jn_ctx *ctx, const double *x, double *y);

/* y += H x (accumulate = 1) or y = H x (accumulate = 0) on DEVICE pointers,
 * enqueued on `stream` (a cudaStream_t, NULL for the context's stream).
 * The caller keeps x inside jn_matvec's range: it is not checked here,
 * which would take a synchronisation. */
jn_status jn_matvec_device(jn_ctx *ctx, const double *d_x, double *d_y, int accumulate, void *stream);

/*
 * File-level drop-in for run_matrix_vector_multiplication(out_dir, in_dir, ...):
 * reads in_dir/vec_<id> and out_dir/vec_<id>, adds H x to the latter and
 * writes it back (Minerva/vector_block/vector_block.c:28-99, 136-155).
 */
jn_status jn_matvec_files(jn_ctx *ctx, const char *output_vector_directory, const char *input_vector_directory);

/*
 * y += H x (accumulate = 1) or y = H x (accumulate = 0) on DEVICE pointers,
 * for callers that must not allocate device memory: a solver that has sized
 * its Krylov basis to the memory it was granted, an application under a
 * fixed device-memory budget, or a loop that cannot take the synchronisation
 * an allocation may bring.  It always runs the block-tile engine (3) at the
 * context's precision, whatever jn_set_engine chose: its result equals
 * jn_matvec_device's bit for bit when engine 3 is the context's engine, and
 * agrees with the other engines to rounding (about 1e-15 of max|y| at
 * precision 64, FP32 level at 32).  Precision 32 needs jn_set_precision(ctx,
 * 32) first (it builds the FP32 matrix elements this entry point reads).
 * Its scratch is a fixed array inside the library that every GPU loading
 * the library holds until exit, so it serves dimensions up to
 * JN_NOALLOC_MAX_DIM and rejects larger ones.  All calls share that array:
 * calls whose kernels overlap on the GPU race, so serialise them.  The first
 * call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and caches it for the life of the process; make
 * that first call before any stream capture.  The cached address does not
 * survive cudaDeviceReset: do not call this entry point on a device after
 * resetting it.  A basis with a sub-basis wider than a block-tile row (more
 * than 8 191 neutron states in one block) has no block-tile engine: this
 * entry point, engine 3 and the batched solvers then return JN_ERR_INVALID
 * with the reason, while jn_open, the walk engine and jn_lanczos work.  No
 * counterpart in the reference, which has no device memory.
 */
#define JN_NOALLOC_MAX_DIM 262144
jn_status jn_matvec_device_noalloc(jn_ctx *ctx, const double *d_x, double *d_y, int accumulate, void *stream);

/* y (+)= H x on device pointers, on the context's stream, with CUDA events
 * around the gather-multiply kernel; waits for completion and returns
 * durations in milliseconds: ms[0] the gather-multiply kernel alone, ms[1]
 * everything else of the product (clearing, x preparation, the final
 * conversion into y).  Used for roofline accounting. */
jn_status jn_matvec_profile(jn_ctx *ctx, const double *d_x, double *d_y, int accumulate, float ms[2]);

/* Arithmetic of the products of this context: 64 (default) computes every
 * multiply-add in FP64; 32 uses FP32 copies of the matrix elements and of x,
 * sums each term in FP32 and combines the terms with error-free (TwoSum)
 * compensation; x and y stay FP64 at the interface.  Matrix elements of
 * single-species blocks below 1e-12 in magnitude are stored as zero in the
 * FP32 copy, which is the reference's skip (matrix_vector_multiplication.c:52-53). */
jn_status jn_set_precision(jn_ctx *ctx, int precision);

/* Product engine: 4 — panels: every instruction's referenced matrix
 * elements, signs applied, stored densely and streamed once, with the
 * blocks of y a CTA touches accumulated in shared memory as exact 64-bit
 * fixed-point integers; 5 — walks: each instruction's longer list walked by
 * destination in lane chunks, the other list's rows grouped by connection
 * index, each row summed in registers over a chunk and rounded once into
 * the lane's shared-memory slot (the walk plan is built on the first
 * product); 3 — shared-memory block tiles with exact 64-bit fixed-point
 * sums; 2 — one warp per 32-element piece, FP64 sums in fixed term order
 * (its plan is built and uploaded here, the first time it is selected).
 * Defaults: engine 5 at precision 64 (its exact-integer arithmetic); at
 * precision 32, engine 4 when the dimension is at most 26 624, else 5.
 * jn_set_engine fixes one engine for both precisions.  Engines 3, 4 and 5
 * give bit-identical results whatever the execution order. */
jn_status jn_set_engine(jn_ctx *ctx, int engine);

/* Arithmetic of the walk engine's precision-64 products: 0 (default) —
 * exact integers: matrix elements and x as 52-bit fixed-point integers
 * (scaled to max|M| and max|x|) split into 28 + 24 bits, three 32 x 32 ->
 * 64-bit integer multiply-adds per contribution, every sum exact and each
 * row's sum rounded once to the nearest output unit; 1 — FP64 fused
 * multiply-adds (bound by GB300's narrow FP64 pipe).  Both are within
 * 1e-13 of FP64 products relative to max|y|.  This extends the solver seam
 * (no reference counterpart: the reference computes in FP64 only). */
jn_status jn_set_walk_arithmetic(jn_ctx *ctx, int fp64_fma);

/* The walk engine's plan (built here if it was not yet):
 * out[0] warp tasks, out[1] pieces, out[2] row groups, out[3] multiply-adds
 * including chunk padding, out[4] including idle lanes, out[5] length of the
 * walk element array (the matrix elements plus the transposed copies of the
 * blocks that proton walks read), out[6] persistent CTAs at the current
 * arithmetic.  No reference counterpart (plan statistics). */
jn_status jn_walk_stats(jn_ctx *ctx, double out[7]);

/*
 * Autotuner.  Times candidate schedules of the product on the context's own
 * problem and precision: for the panel engine, rows per lane per warp task
 * (8 ... 128) x persistent CTAs per SM; the walk and block-tile engines
 * are one candidate each (with tune_engine, every engine is timed; without,
 * only the context's own).  The fastest (median of `trials` CUDA-event timings of
 * the product kernel, each after a write of twice the L2 size, so that the
 * product's data streams from HBM) is installed.  The panel schedule is
 * tuned at both precisions (when the FP64 kernel fits): `tuning` reports the
 * context's own, and jn_set_precision installs the other's when the
 * precision changes.  jn_set_panel_schedule sets one schedule for both.  The panel engine's
 * schedule never changes a result bit (each contribution is rounded on its
 * own); switching engines changes results at the 1e-15 level, so
 * tune_engine = 0 keeps them bit-identical to the untuned context.  No
 * counterpart in the reference, whose evaluation order comes from Mars
 * (src/Mars/programs/mars.c:92-170).
 */
typedef struct {
	int engine;             /* 4 panels, 5 walks, 3 block tiles */
	int rows_per_lane;      /* panel tasks: rows a lane walks */
	int ctas_per_sm;        /* panel kernels: persistent CTAs per SM */
	float ms;               /* product-kernel time of the choice */
	int candidates;         /* schedules timed */
} jn_tuning;
jn_status jn_autotune(jn_ctx *ctx, int trials, int tune_engine, jn_tuning *tuning);

/* Install a panel schedule directly (rows per lane, CTAs per SM). */
jn_status jn_set_panel_schedule(jn_ctx *ctx, int rows_per_lane, int ctas_per_sm);

/* The engine the next product of this context runs at its current
 * precision (the panel engine falls back to block tiles where its
 * accumulator does not fit), or -1 for a NULL context. */
int jn_active_engine(const jn_ctx *ctx);

/* Synchronise the context's stream. */
jn_status jn_synchronize(jn_ctx *ctx);

/* Plan statistics.  algorithmic_bytes is the compulsory traffic of one
 * product: every index list once in the reference's 12-byte record format,
 * every matrix element some list pair indexes (8 bytes), x read and y
 * written (16 bytes per basis state).  multiply_adds counts both directions
 * of off-diagonal instructions.  num_work_units and num_tiles describe
 * engine 2's plan, which a context builds when jn_set_engine(ctx, 2) first
 * selects it: jn_get_plan_stats reports 0 for both before that. */
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

/* ------------------------------------------------------------------ */
/* Lanczos (Bacchus/lanczos/lanczos.c)                                 */
/* ------------------------------------------------------------------ */
#define JN_MAX_REPORTED 64

typedef enum {
	/* full reorthogonalisation; converged when min(r, r^2/gap) < tolerance
	 * for each of the num_eigenvalues lowest Ritz values */
	JN_LANCZOS_FULL = 0,
	/* the reference's algorithm: start e_0, reorthogonalise v_{k+1} against
	 * v_0..v_{k-3} only, converged when the lowest Ritz value moves by less
	 * than tolerance (lanczos.c:60-253) */
	JN_LANCZOS_REFERENCE = 1
} jn_lanczos_mode;

typedef struct {
	int max_iterations;            /* lanczos.max_num_lanczos_iterations */
	int num_eigenvalues;           /* lowest eigenpairs wanted (<= JN_MAX_REPORTED) */
	double tolerance;              /* lanczos.convergence_tolerance (MeV) */
	int mode;                      /* jn_lanczos_mode */
	int check_every;               /* convergence test interval (1 = every step) */
	const double *start_vector;    /* host, length D; NULL = e_0 as the reference */
	int verbose;                   /* per-iteration lines on stdout */
	int criterion;                 /* JN_LANCZOS_REFERENCE: jn_convergence_criterion (lanczos.converge_eigenvectors) */
} jn_lanczos_options;

/* What JN_LANCZOS_REFERENCE compares between consecutive steps
 * (Bacchus/lanczos/lanczos.h:11-16, lanczos.c:199-235): the lowest Ritz
 * value, or the lowest eigenvector of the tridiagonal matrix (sign chosen so
 * that its first component is not negative; the previous step's vector, one
 * component shorter, counts as zero there), converged when the change is
 * below the tolerance (lanczos.c:276-287). */
typedef enum {
	JN_CONVERGE_EIGENVALUES = 0,
	JN_CONVERGE_EIGENVECTORS = 1
} jn_convergence_criterion;

typedef struct {
	int iterations;                /* Krylov dimension reached */
	int converged;
	int num_ritz_values;           /* = iterations */
	int num_eigenvalues;           /* entries filled below */
	double eigenvalues[JN_MAX_REPORTED];    /* Rayleigh quotients of the Ritz vectors (FP64 products) */
	double ritz_values[JN_MAX_REPORTED];    /* eigenvalues of the tridiagonal matrix */
	double residual_norms[JN_MAX_REPORTED]; /* |H x - rq x| / |x| */
	double iteration_seconds;      /* host time of the Lanczos steps and their convergence checks */
	double refinement_seconds;     /* host time of the Ritz vectors and their FP64-grade products */
} jn_lanczos_result;

/* Run Lanczos on the context's Hamiltonian.  Replaces new_lanczos_environment
 * + diagonalize (Bacchus/lanczos/lanczos.c:37-253).  The Krylov basis stays
 * on the device.  Returns JN_ERR_NOT_CONVERGED (results still filled) when
 * JN_LANCZOS_FULL stops at max_iterations.  The Krylov vectors are
 * normalised (max|x| between D^-1/2 and 1), so the products stay inside
 * jn_matvec's range whenever the matrix elements' row-sum bound lies in
 * [2^-47 D^1/2, 2^121): any Hamiltonian in MeV.  The same holds for the
 * batched solvers. */
jn_status jn_lanczos(jn_ctx *ctx, const jn_lanczos_options *options, jn_lanczos_result *result);

/* All Ritz values of the last solve in ascending order, as get_eigensystem +
 * print_eigensystem report them (lanczos.c:255-265, eigensystem.c:99-113). */
jn_status jn_lanczos_ritz_values(jn_ctx *ctx, double *out, int capacity, int *count);

/* Ritz vector i (0 = lowest) of the last solve, full length D, host memory
 * (get_eigenvector, Bacchus/eigensystem/eigensystem.c:86-97). */
jn_status jn_lanczos_eigenvector(jn_ctx *ctx, int i, double *host_out);

/* Write Ritz vectors 0..count-1 as <directory>/eigenvector_<i+1>/vec_<b>
 * (Bacchus/programs/bacchus.c:68-87). */
jn_status jn_lanczos_save_eigenvectors(jn_ctx *ctx, const char *directory, int count);

/* Print the eigensystem block exactly as print_eigensystem does
 * (Bacchus/eigensystem/eigensystem.c:99-113) for the given values. */
void jn_print_eigensystem(const double *eigenvalues, int count);

/* ------------------------------------------------------------------ */
/* Other matrix elements on the same lists: H(c) = H0 + sum_i c_i H_i   */
/* ------------------------------------------------------------------ */
/* Number of matrix elements of the context (all blocks, plan layout). */
size_t jn_me_count(const jn_ctx *ctx);

/* Read the <id>_matrix_elements files of another directory (same
 * combination table, e.g. another operator H_i) into out, jn_me_count
 * values in the context's layout (host only).  The reference reads its
 * blocks with new_matrix_block (Minerva/matrix_block/matrix_block.c:22-62). */
jn_status jn_read_matrix_elements(const jn_ctx *ctx, const char *matrix_file_base_directory, double *out);

/* Replace the context's matrix elements (host array in the same layout);
 * the lists, the plan and the vectors stay.  No counterpart in the
 * reference, which reads its matrix elements from disk for every product. */
jn_status jn_set_matrix_elements(jn_ctx *ctx, const double *matrix_elements);

/*
 * Batched Lanczos: num_instances Hamiltonians on the context's lists, each
 * with its own matrix elements, solved together (one launch per kernel for
 * all instances, one captured CUDA graph per Lanczos step).  Each instance
 * runs the single solve's full mode: full reorthogonalisation, converged
 * when min(r, r^2/gap) < tolerance for each of the num_eigenvalues lowest
 * Ritz values (Bacchus/lanczos/lanczos.c:74-253 is the single-instance
 * algorithm it extends).  precision 32: FP32 matrix elements and vectors in
 * the products (exact fixed-point sums), FP64 everywhere else; the results
 * are refined by FP64 products of the lowest num_eigenvalues + refine_extra
 * Ritz vectors and an FP64 Rayleigh-Ritz solve.  No counterpart in the
 * reference.
 */
typedef struct {
	int num_instances;
	const double *const *matrix_elements;   /* host, num_instances arrays of jn_me_count values */
	const double *const *start_vectors;     /* host, NULL or num_instances vectors (NULL entries: default) */
	int max_iterations;
	int num_eigenvalues;                    /* <= JN_MAX_REPORTED */
	double tolerance;                       /* MeV */
	int precision;                          /* 32 or 64 */
	int check_every;                        /* convergence test interval in steps (default 10) */
	int use_graph;                          /* replay one captured graph per step */
	int refine_extra;                       /* extra Ritz vectors in the refinement (default 4) */
	int num_eigenvectors;                   /* refined eigenvectors returned per instance (<= num_eigenvalues) */
	double *const *eigenvectors;            /* host, num_instances outputs of num_eigenvectors x D (NULL entries skip) */
} jn_batch_options;

typedef struct {
	int iterations;
	int converged;
	int num_eigenvalues;
	double eigenvalues[JN_MAX_REPORTED];    /* refined, FP64 Rayleigh-Ritz */
	double ritz_values[JN_MAX_REPORTED];    /* of the solve's own (FP32 or FP64) operator */
	double residual_norms[JN_MAX_REPORTED]; /* |H x - e x| / |x| of the refined vectors, FP64 H */
} jn_batch_result;

jn_status jn_lanczos_batch(jn_ctx *ctx, const jn_batch_options *options, jn_batch_result *results);

/*
 * Batched Lanczos over several bases in one solve: options[b] gives basis
 * b's instances (num_instances, matrix_elements, start_vectors,
 * eigenvectors; the solver options must be the same for every basis) and
 * results[b] receives them.  Every step is one captured graph for all
 * instances of all bases: one persistent walk-engine launch computes every
 * instance's product (the instances' walk plans concatenated into one task
 * list, each instance with its own matrix elements), then one launch per
 * vector kernel.  Products in FP32 (precision 32) or FP64 multiply-adds
 * (precision 64), exact fixed-point sums; refinement in FP64.  The contexts
 * must be on one device; the solve runs on ctxs[0]'s stream.  No counterpart
 * in the reference: Vulcan (src/Vulcan/programs/vulcan.c:114-141) writes one
 * H(c) = sum_i c_i H_i to disk, and each H(c) is then a Bacchus run of its
 * own.
 */
jn_status jn_lanczos_batch_bases(jn_ctx *const *ctxs, int num_bases, const jn_batch_options *options,
				 jn_batch_result *const *results);

/* ------------------------------------------------------------------ */
/* J-scheme -> M-scheme two-body transform (Mercury)                   */
/* ------------------------------------------------------------------ */
typedef struct jn_transform jn_transform;

typedef struct {
	int num_two_body_blocks;
	int num_one_body_blocks;        /* written as zeros, as the reference does */
	size_t num_elements;            /* two-body matrix elements computed per run */
	size_t num_pair_states;         /* M-scheme pair states with their (J, T) expansion */
	size_t num_configurations;      /* rows of the interaction file */
	double dense_flops;             /* flops of the reference's dense S^T V S decoupling, for comparison */
	double algorithmic_bytes;       /* compulsory device traffic of one run */
	double plan_seconds;            /* host planning time of jn_transform_open */
} jn_transform_stats;

/*
 * Plan the transform of a J-scheme two-body interaction in the Antoine
 * format (src/Neptune/input/read_2nf_antoine_format.c:70-111) into the
 * M-scheme matrix-element blocks that the combination table lists, and
 * upload the plan to the current CUDA device.  Arguments are those of
 * mercury_J_scheme_to_internal.x (src/Mercury/arguments/arguments.c:88-160):
 * the combination table, the index-list base directory holding
 * <p|n|pp|nn>_inds_index_lists/basis_energy_<E>, Z, N, the single- and
 * two-particle energy limits, the interaction file, and whether the kinetic
 * column is added (the reference's default; --exclude-kinetic-energy turns
 * it off).  Replaces new_transform_2nf_block_manager + open_antoine_2nf_file
 * (src/Mercury/transform_2nf_block_manager/transform_2nf_block_manager.c:89-111).
 */
jn_status jn_transform_open(const char *combination_table_file, const char *index_list_dir, int num_protons,
			    int num_neutrons, int single_particle_energy, int two_particle_energy,
			    const char *antoine_file, int include_kinetic_energy, jn_transform **transform);

/* Enqueue the computation of every two-body block (one kernel) on `stream`
 * (NULL: the transform's stream).  Replaces decouple_transform_2nf_block +
 * get_transform_2nf_matrix_block over all blocks
 * (transform_2nf_block_manager.c:113-268, compute_jt_block in
 * src/Neptune/block_transform/block_transform.c:358-415). */
jn_status jn_transform_run(jn_transform *transform, void *stream);

/* One run on the transform's stream timed with CUDA events (milliseconds). */
jn_status jn_transform_profile(jn_transform *transform, float *ms);

/* Elements of matrix-element block `block_id` from the last run (count only
 * when host_out is NULL). */
jn_status jn_transform_elements(jn_transform *transform, int block_id, double *host_out, size_t capacity,
				size_t *count);

/* Run and write <output_dir>/<id>_matrix_elements for every one- and
 * two-body block (save_mercury_matrix_block,
 * src/Mercury/mercury_matrix_block/mercury_matrix_block.c:106-179). */
jn_status jn_transform_write(jn_transform *transform, const char *output_dir);

jn_status jn_transform_get_stats(const jn_transform *transform, jn_transform_stats *stats);
void jn_transform_close(jn_transform *transform);

/* open + write + close: the two-body part of mercury_J_scheme_to_internal.x
 * (src/Mercury/programs/mercury_J_scheme_to_internal.c:65-202). */
jn_status jn_transform_2nf(const char *combination_table_file, const char *index_list_dir, const char *output_dir,
			   int num_protons, int num_neutrons, int single_particle_energy, int two_particle_energy,
			   const char *antoine_file, int include_kinetic_energy);

/* ------------------------------------------------------------------ */
/* J-scheme -> M-scheme three-body transform (Mercury, three-body part) */
/* ------------------------------------------------------------------ */
typedef struct jn_transform3 jn_transform3;

typedef struct {
	int num_three_body_blocks;
	size_t num_elements;            /* three-body matrix elements computed per run */
	size_t num_states;              /* M-scheme three-particle states with their coupled expansions */
	size_t num_terms;               /* expansion terms over all states */
	size_t num_coupled_states;      /* coupled states over all total-M blocks */
	size_t num_m_blocks;            /* total-M blocks over all bases */
	size_t file_states;             /* coupled states of the J-scheme file */
	size_t file_elements;           /* rows of its matrix file */
	size_t v_entries;               /* J-scheme matrix entries held on the device */
	double dense_flops;             /* flops of the reference's dense S^T V S decoupling, for comparison */
	double algorithmic_bytes;       /* compulsory device traffic of one run */
	double plan_seconds;            /* host planning time of jn_transform3_open */
} jn_transform3_stats;

/*
 * Plan the transform of a jjj-coupled three-body interaction into the
 * M-scheme three-body blocks that the combination table lists, and upload
 * the plan to the current CUDA device.  The interaction is a directory in
 * the reference's ASCII format: one .cnf file (single-particle shells, then
 * jjj-coupled three-particle states) and one .mat file ("bra ket element"
 * rows over those states) (src/Neptune/input/read_3nf_ascii_format.c:14-279).
 * The index-list base directory holds <ppp|pp|p|nnn|nn|n>_inds_index_lists/
 * basis_energy_<E>; single_particle_energy is the shell limit of the
 * manager (src/Mercury/arguments/arguments.c:88-160).  Replaces
 * new_transform_3nf_block_manager + open_data_file
 * (src/Mercury/transform_3nf_block_manager/transform_3nf_block_manager.c:109-124,
 * src/Neptune/input/read_3nf_file.c:12-44).
 */
jn_status jn_transform3_open(const char *combination_table_file, const char *index_list_dir, int num_protons,
			     int num_neutrons, int single_particle_energy, const char *jscheme_dir,
			     jn_transform3 **transform);

/* Enqueue the computation of every three-body block (one kernel) on
 * `stream` (NULL: the transform's stream).  Replaces get_transformed_block
 * + get_3nf_mercury_matrix over all blocks
 * (transform_3nf_block_manager.c:233-284, src/Mercury/transformed_block/transformed_block.c:113-147,
 * compute_jjj_block in src/Neptune/block_transform/block_transform.c:147-356). */
jn_status jn_transform3_run(jn_transform3 *transform, void *stream);

/* One run on the transform's stream timed with CUDA events (milliseconds). */
jn_status jn_transform3_profile(jn_transform3 *transform, float *ms);

/* Elements of three-body block `block_id` from the last run (count only
 * when host_out is NULL). */
jn_status jn_transform3_elements(jn_transform3 *transform, int block_id, double *host_out, size_t capacity,
				 size_t *count);

/* Run and write <output_dir>/<id>_matrix_elements for every three-body block. */
jn_status jn_transform3_write(jn_transform3 *transform, const char *output_dir);

jn_status jn_transform3_get_stats(const jn_transform3 *transform, jn_transform3_stats *stats);
void jn_transform3_close(jn_transform3 *transform);

/* One call: plan, run and write every three-body block (the three-body part
 * of mercury_J_scheme_to_internal.x,
 * src/Mercury/programs/mercury_J_scheme_to_internal.c:306-398). */
jn_status jn_transform_3nf(const char *combination_table_file, const char *index_list_dir, const char *output_dir,
			   int num_protons, int num_neutrons, int single_particle_energy, const char *jscheme_dir);

/* <j1 m1 j2 m2 | j3 m3> with all arguments doubled, as clebsch_gordan
 * defines it (src/Neptune/clebsch_gordan/clebsch_gordan.c:31-42); host only. */
double jn_clebsch_gordan(int j1, int j2, int j3, int m1, int m2, int m3);

/* ------------------------------------------------------------------ */
/* Learned warm start: an MLP from couplings c to a Lanczos start vector */
/* ------------------------------------------------------------------ */
/*
 * A two-hidden-layer perceptron in FP32, trained and evaluated by the
 * library's own CUDA kernels: x (num_inputs) -> gelu(W1 x + b1) (hidden) ->
 * gelu(W2 h1 + b2) (hidden) -> W3 h2 + b3 (num_outputs), with
 * gelu(a) = a (1 + erf(a / sqrt 2)) / 2.  Loss over n samples:
 * sum_s |y_s - t_s|^2 / (2 n).  Parameters are one flat array
 * [W1 (hidden x num_inputs), b1, W2 (hidden x hidden), b2,
 * W3 (num_outputs x hidden), b3], row-major, output index first.  Gradients
 * are summed over samples in sample order, so results repeat bit for bit.
 * Adam (beta1 0.9, beta2 0.999, eps 1e-8) updates the parameters.  Samples
 * are row-major: x is n x num_inputs, t and y are n x num_outputs.  No
 * counterpart in the reference; the reduced-basis idea is that of Ceres
 * (src/Ceres/programs/ceres.c:17-80), which projects operators onto
 * vectors that earlier solves produced.
 */
typedef struct jn_mlp jn_mlp;

jn_status jn_mlp_create(int num_inputs, int hidden, int num_outputs, uint64_t seed, jn_mlp **mlp);
void jn_mlp_destroy(jn_mlp *mlp);
size_t jn_mlp_num_params(const jn_mlp *mlp);
jn_status jn_mlp_get_params(const jn_mlp *mlp, float *params);
jn_status jn_mlp_set_params(jn_mlp *mlp, const float *params);
/* loss and its gradient (num_params values) of the current parameters */
jn_status jn_mlp_loss_and_gradient(jn_mlp *mlp, const float *x, const float *t, int n, float *loss, float *grad);
/* `steps` full-batch Adam steps; final_loss = the loss after the last step */
jn_status jn_mlp_train(jn_mlp *mlp, const float *x, const float *t, int n, int steps, float learning_rate,
		       float *final_loss);
jn_status jn_mlp_predict(jn_mlp *mlp, const float *x, int n, float *y);

/*
 * The warm start for jn_lanczos_batch.  Fitting takes solutions that the
 * solver produced for sample couplings c_s: for each sample its
 * num_vectors lowest eigenvectors.  The target of sample s is the
 * projection of the solver's default start vector r onto them,
 * u_s = sum_e v_e (v_e . r) / |.|, which does not depend on the signs of the
 * v_e and varies smoothly with c.  The reduced basis is the leading
 * basis_size left singular vectors of [u_1 .. u_S] (from the S x S Gram
 * matrix, computed on the GPU).  The MLP learns the coordinates of u_s in
 * that basis from c_s.  A start vector for new couplings is the expansion of
 * the predicted coordinates (a GPU kernel), normalised, plus noise * r / |r|
 * so that no eigenvector can be missing from the Krylov space.  Cold-start
 * Lanczos (start vector r) stays the judge: the warm start only changes
 * where the iteration begins.
 */
typedef struct jn_warm_start jn_warm_start;

typedef struct {
	int hidden;             /* hidden width (default 128) */
	int basis_size;         /* reduced-basis size = MLP outputs (default 32, <= num_samples) */
	int train_steps;        /* full-batch Adam steps (default 3000) */
	float learning_rate;    /* default 1e-3 */
	uint64_t seed;          /* MLP initialisation */
	double noise;           /* weight of r in every start vector (default 0.01) */
} jn_warm_start_options;

/* couplings: num_samples x num_couplings (host, row-major); eigenvectors:
 * num_samples host arrays of num_vectors x dim values (the
 * jn_batch_options.eigenvectors layout).  num_samples <= 2048. */
jn_status jn_warm_start_fit(const jn_warm_start_options *options, int64_t dim, int num_couplings, int num_samples,
			    const double *couplings, int num_vectors, const double *const *eigenvectors,
			    jn_warm_start **warm_start, float *final_loss);
/* n start vectors (host arrays of dim values) for couplings (n x num_couplings) */
jn_status jn_warm_start_vectors(jn_warm_start *warm_start, int n, const double *couplings,
				double *const *start_vectors);
/* the basis_size reduced-basis vectors (basis_size x dim, host) */
jn_status jn_warm_start_basis(const jn_warm_start *warm_start, double *basis);
int jn_warm_start_basis_size(const jn_warm_start *warm_start);
void jn_warm_start_destroy(jn_warm_start *warm_start);

/* The solver's default start vector (what jn_lanczos_batch uses when
 * start_vectors is NULL), dim values, host. */
void jn_default_start_vector(int64_t dim, double *out);

/* ------------------------------------------------------------------ */
/* Subspace matrices of training vectors (Ceres)                        */
/* ------------------------------------------------------------------ */
/* norm[i][j] = <v_i|v_j> and op[i][j] = <v_j|H v_i> for j >= i, mirrored
 * (src/Ceres/norm_matrix/norm_matrix.c:4-28,
 * src/Ceres/subspace_operator/subspace_operator.c:7-61), with H the
 * context's operator at its precision and engine.  vectors: n host arrays of
 * jn_dimension values; norm, op: n x n row-major host outputs (either may be
 * NULL).  The products and dot products run on the GPU. */
jn_status jn_subspace_matrices(jn_ctx *ctx, int n, const double *const *vectors, double *norm, double *op);

/* The same from training-vector directories (<dir>/vec_<block id>, as
 * Bacchus writes them), written as .npy files in the reference's layout
 * (src/Ceres/numpy_matrix/numpy_matrix.c:7-35); either path may be NULL.
 * One call per operator: the reference's ceres.x loops over operators. */
jn_status jn_ceres_files(jn_ctx *ctx, int n, const char *const *vector_dirs, const char *norm_matrix_path,
			 const char *subspace_operator_path);

/* ------------------------------------------------------------------ */
/* File tools around the product (host only, no GPU needed)            */
/* ------------------------------------------------------------------ */
/* Aurora: convert the Anicre index lists under anicre_dir,
 * <type>_inds_index_lists/index_list_E_in<Eb>_E_out<Ek>_M_in<Mb>_M_out<Mk>_dE<dE>_dM<dM>_depth<d>
 * (raw {in, out, k} int triples, or rows "in out +k" / "in out -k" when
 * human_readable), into <output_dir>/index_list_<id> for every list row of
 * the combination table; with skip_three_body the three-particle lists are
 * left out.  Lists Anicre did not write are reported on stderr and skipped,
 * as aurora.x does (src/Aurora/programs/aurora.c:21-96,
 * src/Aurora/index_list/index_list.c:21-112).  converted (may be NULL)
 * receives the number of lists written. */
jn_status jn_aurora(const char *combination_table_file, const char *anicre_dir, const char *output_dir,
		    int num_protons, int num_neutrons, int human_readable, int skip_three_body, int *converted);

/* Mars: an evaluation order ("BLOCK: in out list [list] me" rows) from the
 * CALCBLOCK rows of the combination table, two-body blocks and, unless
 * two_body_only, three-body blocks; one-body blocks are zero and left out
 * (src/Mars/programs/mars.c:64-199).  The rows come in the panel engine's
 * schedule order (output block, input block, most multiplications first)
 * instead of Mars' cache-reuse sort; the reference's Bacchus accepts any
 * order.  num_rows (may be NULL) receives the number of rows written. */
jn_status jn_mars(const char *combination_table_file, int num_protons, int num_neutrons, const char *output_file,
		  int two_body_only, int *num_rows);

/* Vulcan: <output_dir>/<id>_matrix_elements = sum_i coefficients[i] *
 * <operator_dirs[i]>/<id>_matrix_elements for every matrix-element block of
 * the combination table, a missing block counting as zero, in the
 * reference's block format (src/Vulcan/programs/vulcan.c:47-207). */
jn_status jn_vulcan(const char *combination_table_file, int num_protons, int num_neutrons, int num_operators,
		    const char *const *operator_dirs, const double *coefficients, const char *output_dir);

#ifdef __cplusplus
}
#endif
#endif
