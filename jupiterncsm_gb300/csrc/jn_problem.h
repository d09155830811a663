/*
 * jn_problem.h — host-side model of one JupiterNCSM Hamiltonian and the
 * device execution plan built from it.
 *
 * The files read are the reference's (src/Utilities/combination_table/
 * combination_table.c:419-640, src/Minerva/evaluation_order/evaluation_order.c:43-243,
 * src/Minerva/index_list/index_list.c:69-97, src/Minerva/matrix_block/matrix_block.c:22-62).
 * Everything is validated on the host so that no device access can leave
 * its buffer: every in/out index against the basis-block dimensions and every
 * connection index against its matrix-element block.
 *
 * The plan turns the evaluation order into output-owned work: each
 * instruction contributes a forward term to its output block and, when
 * off-diagonal, a transposed term to its input block
 * (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:212-462).
 * Output blocks are cut into element tiles; the terms touching a tile are
 * cut into chunks of similar work.  A chunk is one CTA's work unit; its
 * partial sums are added in chunk order by the reduction pass, so the
 * summation order of every output element is fixed by the files alone.
 */
#ifndef JN_PROBLEM_H
#define JN_PROBLEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { JN_KIND_N = 1, JN_KIND_P = 2, JN_KIND_NP = 3 };

typedef struct {
	int Ep, Mp, En, Mn;
	int64_t Np, Nn;
	int64_t offset;         /* first element in the full vector */
	int id;
} jn_block_t;

typedef struct {
	int kind;               /* JN_KIND_* */
	int bin, bout;          /* basis block indices (0-based) */
	int ln, lp;             /* list slots or -1 */
	int me;                 /* matrix-element slot */
} jn_instr_t;

/* one index list: file contents plus both CSR views */
typedef struct {
	int id;
	char type;              /* 'n' or 'p' */
	int64_t len;
	int32_t *triples;       /* len*3 as on disk: in, out, matrix_index */
	int32_t nin, nout;      /* sub-basis sizes it maps between */
	int64_t csr_out_ptr;    /* offsets into jn_plan_t.rowptr (nout+1 entries) */
	int64_t csr_in_ptr;     /* (nin+1 entries) */
	int64_t ent_out;        /* offsets into jn_plan_t.ent (len entries) */
	int64_t ent_in;
	int64_t walk_out, nwalk_out;    /* walks of the by-out view (first index, count) */
	int64_t walk_in, nwalk_in;      /* walks of the by-in view */
	int64_t pmeta;                  /* first packed entry in jn_plan_t.pmeta (by-out order) */
} jn_list_t;

typedef struct {
	int id;
	uint64_t nd_n, nd_p;    /* header dimensions */
	int64_t len;
	int64_t offset;         /* into jn_plan_t.me */
	int single;             /* used by single-species (n or p) instructions */
} jn_me_t;

/* device term descriptor: one direction of one instruction, seen from its
 * destination block.  Entry arrays hold (source index, matrix_index). */
typedef struct {
	int32_t kind;
	int32_t nd;             /* neutron matrix dimension (NP) */
	int64_t src_off;        /* source block offset in x */
	int32_t Nn_src, Nn_dst;
	int64_t p_ptr, p_ent;   /* CSR (by destination row) of the proton list */
	int64_t n_ptr, n_ent;   /* CSR (by destination column) of the neutron list */
	int64_t me_off;
	int32_t instr;          /* evaluation-order index */
	int32_t transpose;
	uint32_t n_e0, n_e1;    /* absolute range of the neutron entries (N, NP) */
	int64_t pw0, pw1;       /* walks of the proton list in this direction */
	int64_t nw0, nw1;       /* walks of the neutron list in this direction */
} jn_term_t;

typedef struct {
	int64_t dst_off;        /* block offset in y */
	int32_t Nn;             /* destination block columns */
	int32_t row0, nrows, col0, ncols;
	int32_t nchunks;
	int64_t partial;        /* first partial slot: chunk c, element e at partial + c*E + e */
	int32_t unit0;          /* first unit of this tile */
	int32_t pad;
} jn_tile_t;

typedef struct {
	int32_t tile;
	int32_t chunk;
	int64_t t0, t1;         /* range into jn_plan_t.unit_terms */
} jn_unit_t;

/* Block-tile plan (exact fixed-point accumulation).  A CTA owns rows
 * [row0, row0+nrows) of one destination block in shared memory and runs the
 * warp tasks [pc0, pc1).  A warp task gives each of its `count` lanes one
 * run: a list entry (or column / row) that stays fixed while the lane walks
 * the matching entries of the other list, all landing on one output
 * element.  Runs are summed in T arithmetic and added to the tile as 64-bit
 * integers in units of 2^-S, so the order of the runs does not change the
 * result. */
typedef struct {
	int64_t dst_off;
	int32_t Nn;
	int32_t row0, nrows;
	int32_t stride;         /* shared-memory row stride (odd) */
	int64_t pc0, pc1;       /* range into jn_plan_t.items */
} jn_btile_t;

/*
 * A walk is one non-empty row of a list's destination-ordered view: the
 * entries [w0, w0+len) that all map onto destination index `idx`, stored as
 * uint2 {w0, len | idx << 16}.  The product of a term restricted to output
 * (row, col) is the double walk P-walk(row) x N-walk(col).
 */
enum {
	JN_TASK_NP_A = 0,       /* lanes over N-walks (columns), loop over P-walks (rows) */
	JN_TASK_NP_B = 1,       /* lanes over P-walks (rows), loop over N-walks (columns) */
	JN_TASK_P_A = 2,        /* P: lanes over columns, loop over P-walks */
	JN_TASK_P_B = 3,        /* P: lanes over P-walks, loop over columns */
	JN_TASK_N_A = 4,        /* N: lanes over N-walks, loop over rows */
	JN_TASK_N_B = 5         /* N: lanes over rows, loop over N-walks */
};

/* 16-byte warp task */
typedef struct {
	uint32_t head;          /* term (bits 0-23) | kind (24-26) | count-1 (27-31) */
	uint32_t lane_base;     /* first lane's walk index / column / row */
	uint32_t loop_base;     /* first looped walk index / column / row */
	uint32_t loop_len;      /* looped walks / columns / rows */
} jn_piece_t;

#define JN_TASK_TERM(h) ((h) & 0xffffffu)
#define JN_TASK_KIND(h) (((h) >> 24) & 7u)
#define JN_TASK_COUNT(h) ((((h) >> 27) & 31u) + 1u)

/* compact term description read by the tile kernel (32 bytes) */
typedef struct {
	int64_t me_off;
	int32_t src_off;
	int32_t nd;
	int32_t Nn_src;
	int32_t transpose;
	int32_t pad0, pad1;
} jn_tterm_t;

/*
 * Panel engine.  Each instruction is a panel of rows x columns: NP rows are
 * the proton-list entries and columns the neutron-list entries, both in
 * by-out order; an N instruction has the spectator proton rows and its
 * neutron entries as columns; a P instruction its proton entries as rows and
 * the spectator neutron columns.  The coefficient of (row j, column i) is
 * s_p s_n M[k_n + Nd k_p] (NP), s_n M[k_n] (N, per column) or s_p M[k_p]
 * (P, per row), with the single-species |M| < 1e-12 skip stored as 0.  NP
 * coefficients are stored densely, row-major, so a product streams them
 * once; an NP panel whose neutron list is longer than its proton list is
 * stored transposed (JN_PANEL_ROWS_N), so that the columns are the shorter
 * list and a warp's lanes cover whole rows.  Forward: y[out + P_o Nn_out + N_o] += c x[in + P_i Nn_in + N_i];
 * off-diagonal panels also add c x[out + P_o Nn_out + N_o] into
 * y[in + P_i Nn_in + N_i].
 */
#define JN_PANEL_DIAG 8          /* input block == output block: no transpose */
#define JN_PANEL_ROWS_N 16       /* NP panel stored transposed: rows are neutron entries, columns proton entries */
#define JN_PANEL_ITER 32         /* rows a lane walks per task (default; the autotuner may choose another) */
#define JN_PANEL_MAX_DIM 26624   /* the accumulator (8 B per state, rows padded to an odd length) in shared memory */

typedef struct {
	int64_t c_off;          /* first coefficient */
	uint32_t row_meta;      /* first packed row entry (source | destination << 16) in pmeta (NP, P) */
	uint32_t col_meta;      /* first packed column entry in pmeta (NP, N) */
	int32_t out_off, in_off;        /* offsets of the output and input blocks */
	int32_t Nn_out, Nn_in;
	int32_t ncols, kind;    /* kind: JN_KIND_* | JN_PANEL_DIAG when input block == output block */
	int32_t out_blk, in_blk;        /* the output and input blocks (a CTA maps them to its accumulator) */
	int32_t nrows, instr;   /* rows; the evaluation-order index of the instruction */
	int32_t Np_out, Np_in;  /* proton dimensions: strides of the blocks' transposed copy of x */
} jn_panel_t;

/*
 * Walk engine (engine 5, jn_walk.c / jn_walk.cu).  Every instruction is
 * applied as one or two directed instructions: forward (input block ->
 * output block) and, off-diagonal, transpose (output block -> input block).
 * The longer list of an n x p instruction is the walk list: its view by
 * destination is cut into walks (entries with one destination) and each walk
 * into lane chunks of at most U entries (U = 8, 4 or 2, chosen per directed
 * instruction).  The other list gives the rows (source row -> destination
 * row, sign, connection index k).  Rows that share k read one row of the
 * matrix-element block, so rows are grouped by k and a group's element row
 * is gathered once per lane entry.  A single-species instruction walks its
 * list, and its rows are the spectators (identity, sign +, one group).  A
 * piece is a run of rows with at most JN_WALK_RS distinct destination rows;
 * a warp task is one piece times 32 lane chunks.  The lane records of a
 * walk view depend only on its list, the view and U: every directed
 * instruction that walks the same view points at one copy.  For every row
 * a lane sums its chunk's contributions in registers and adds the sum into its own
 * shared-memory slot (destination row, lane); at the end of the task the
 * warp sums each walk's lanes and adds one value per (destination row, walk)
 * into the global accumulator.
 *
 * Walk list = neutron list (wp = 0): D(r, w) = dst + r Nn_dst + w,
 * S(r, w) = src + r Nn_src + w in x; proton list (wp = 1): D(r, w) = dst +
 * w Nn_dst + r, and the source is read from the transposed view xT of x
 * (each block [n][p] instead of [p][n]), S(r, w) = src + r Np_src + w, so
 * that in both cases a row's walk entries index one contiguous row of the
 * source block.  The entries of a walk are dealt to its lanes in turn
 * (entry i of a walk spread over l lanes goes to lane i mod l, position
 * i / l): at every position neighbouring lanes read neighbouring sources.
 *
 * Coefficients come from the walk element array: the plan's matrix elements
 * (single-species elements below 1e-12 stored as 0, the reference's skip),
 * then a transposed copy [k_p][k_n] of every n x p block that a proton-walk
 * instruction uses.  The coefficient of (group g, entry e) is
 * s_e A[base_g + k_e]: base_g = block + Nd_walk-stride k_row, so that a
 * group reads one contiguous row of its block.
 */
#define JN_WALK_RS 16           /* distinct destination rows of a piece */
#define JN_WALK_GROUP_END 0x40000000u   /* row word: the last row of its group */
#define JN_WALK_ROW_SPARE 2             /* zero row words after the last: the kernel reads up to two ahead */
#define JN_WALK_POS 0x40000000u         /* lane entry multiplier +1 (bits 31:30 = 01) */
#define JN_WALK_NEG 0xC0000000u         /* lane entry multiplier -1 (bits 31:30 = 11); 00 is padding (0) */

/* lane record of a chunk set, word-major (32 lanes per word): the walk slot
 * | the entries' multipliers << 16 (2 bits for entry u at bit 16 + 2u), U / 2
 * words of packed 16-bit sources, U words of element offset (30 bits) |
 * multiplier << 30.  A multiplier is a 2-bit two's complement: +1 (01), -1
 * (11), or 0 for padding (00). */
#define JN_WALK_LANE_WORDS(U) (1 + (U) / 2 + (U))

typedef struct {                /* 32 bytes */
	int32_t src_off, dst_off;       /* offsets of the source and destination blocks in x and y */
	int32_t src_stride, Nn_dst;     /* row stride of the source view (Nn_src in x, Np_src in xT), Nn of the destination */
	int32_t row0;                   /* first row word in wrows */
	int32_t rdst0;                  /* destination of each slot row in wrdst */
	int32_t group0;                 /* element-row base of each group in wgroups */
	uint32_t meta;                  /* slot rows | walk list is the proton list << 8 | row groups << 9 */
} jn_wpiece_t;

typedef struct {                /* 16 bytes */
	uint32_t piece;
	uint32_t lanes;                 /* first word of the lane records */
	uint32_t walk0;                 /* walk table: the destination index of each walk slot */
	uint32_t meta;                  /* walk slots | U << 8 */
} jn_wtask_t;

typedef struct {
	/* problem */
	int Z, N;
	int nblocks;
	jn_block_t *blocks;
	int64_t dim;
	int ninstr;
	jn_instr_t *instr;
	int nlists;
	jn_list_t *lists;
	int nmes;
	jn_me_t *mes;
	/* flattened device arrays */
	int64_t n_rowptr;  uint32_t *rowptr;
	int64_t n_ent;     uint32_t *ent;      /* pairs: src, matrix_index */
	int64_t n_me;      double *me;
	int nterms;        jn_term_t *terms;
	/* engine 2 (jn_plan_build_units; empty until built) */
	int ntiles;        jn_tile_t *tiles;
	int nunits;        jn_unit_t *units;
	int64_t n_unit_terms; int32_t *unit_terms;
	int64_t n_partial;
	int nbtiles;       jn_btile_t *btiles;
	int btiles_off;                 /* no block tiles (engine 3 unavailable): a block row is wider than a tile */
	char btiles_why[256];
	int64_t npieces;   jn_piece_t *pieces;
	jn_tterm_t *tterms;             /* nterms compact term descriptions */
	int64_t nwalks;    uint32_t *walks;    /* pairs {w0, len | idx << 16} */
	int64_t nitems;    uint32_t *items;    /* warp items {first task, width | ntasks << 8} */
	int max_tile_elems;             /* shared-memory accumulator size needed */
	double abs_bound;               /* max over y elements of sum |M| over its contributions */
	int *term_dst;                  /* destination basis block of each term */
	/* accounting */
	int64_t list_entries;           /* sum of distinct list lengths */
	int64_t me_elements;            /* sum of distinct ME block lengths */
	int64_t me_referenced;          /* elements some list pair actually indexes */
	double visits;                  /* multiply-adds per product (both directions) */
	/* panel engine (built by jn_panels_build) */
	int npanels;       jn_panel_t *panels;
	int64_t nptasks;   uint32_t *ptasks;   /* 4 words per warp task: panel, j0, j1, i0 | lanes per row << 24 */
	int pgrid;         uint32_t *pcta;     /* pgrid + 1 task offsets: CTA b runs [pcta[b], pcta[b+1]) */
	uint32_t *pflush_ptr;                   /* pgrid + 1 offsets (in pairs) into pflush */
	int64_t npflush;   uint32_t *pflush;   /* the blocks a CTA touches: pairs {block, its offset in the CTA's accumulator} */
	int64_t pcta_words;                     /* the largest CTA accumulator: sum of Np * (Nn | 1) over its blocks */
	uint32_t *pblocks;                      /* per block: {offset in y, unused, Np, Nn} */
	int64_t psmem_words;                    /* the whole vector's accumulator length: sum of Np * (Nn | 1) */
	int64_t n_pmeta;   uint32_t *pmeta;    /* each list's entries in panel order (list_order in jn_panel.c) */
	uint32_t *pperm;                        /* per packed entry: its index in the list's by-out order */
	int64_t n_coef;                         /* coefficients of all panels */
	/* walk engine (built by jn_walk_build) */
	int64_t nwtasks;   jn_wtask_t *wtasks;  /* instructions by matrix-element block */
	int64_t nwpieces;  jn_wpiece_t *wpieces;
	int64_t n_wlanes;  uint32_t *wlanes;
	int64_t n_wwalks;  uint32_t *wwalks;
	int64_t n_wrows;   uint32_t *wrows;    /* source row | slot row << 16 | group end | sign << 31; JN_WALK_ROW_SPARE more */
	int32_t *wxperm;                        /* position in x of each element of the transposed view xT */
	int wxt;                                /* proton walks read xT */
	int64_t n_wrdst;   uint32_t *wrdst;
	int64_t n_wgroups; uint32_t *wgroups;  /* element-row base of each group */
	int32_t *wgblock;                       /* the matrix-element block of each group */
	int64_t n_wme;                          /* walk element array: n_me + transposed copies */
	int64_t *wtpos;                         /* per matrix-element block: offset of its transpose, or -1 */
	double wvisits;                         /* multiply-adds including padding */
	double wlane_slots;                     /* lane slots of all tasks x rows: multiply-adds including idle lanes */
} jn_plan_t;

typedef struct {
	char comb[4096], order[4096], lists[4096], mes[4096];
	char krylov[4096], eigvec[4096];
	int Z, N;
	long max_iterations;
	double tolerance;
	long target_eigenvector;
	int converge_eigenvectors;
	/* optional GPU group */
	int num_eigenvalues;
	int precision;          /* 64 or 32 */
	int reorthogonalize;    /* 1 full, 0 reference-style partial */
} jn_runfile_t;

int jn_read_runfile(const char *path, jn_runfile_t *rf, char *err, size_t errlen);
/* fn(i, arg) for every i < n on all host cores (at most 32 threads, or
 * fewer when the environment variable JN_HOST_THREADS caps them); items
 * are taken from a shared counter, so fn must not depend on their order */
void jn_par_for(int64_t n, void (*fn)(int64_t, void *), void *arg);
int jn_plan_build(jn_plan_t *plan, const char *comb, const char *order, const char *lists_dir,
		  const char *me_dir, int Z, int N, int target_units, char *err, size_t errlen);
void jn_plan_free(jn_plan_t *plan);
/* engine 2's tiles and work units (about target_units of them); a no-op
 * when they exist */
int jn_plan_build_units(jn_plan_t *plan, int target_units, char *err, size_t errlen);
/* abs_bound of the plan's lists with another set of matrix elements (same
 * layout as plan->me): the fixed-point scale of a product must use it.  With
 * me == NULL every |M| counts as 1: the largest number of contributions to
 * one element, so that abs_bound <= that * max|M| for any elements. */
double jn_plan_abs_bound(const jn_plan_t *plan, const double *me);
/* read the <id>_matrix_elements files of `dir` into out (plan->n_me values,
 * the plan's layout); every block must have the plan's dimensions */
int jn_plan_read_me(const jn_plan_t *plan, const char *dir, double *out, char *err, size_t errlen);
/* the panel plan for a persistent grid of `grid` CTAs whose warp tasks walk
 * `iter` rows per lane (dimension <= JN_PANEL_MAX_DIM).  The tasks and the
 * grid decide only who computes a contribution, never its rounding: every
 * schedule gives bit-identical products. */
int jn_panels_build(jn_plan_t *plan, int grid, int iter, char *err, size_t errlen);
void jn_panels_free(jn_plan_t *plan);
/* the CTA ranges and flush lists of the plan's tasks for a grid of `grid`
 * persistent CTAs (malloc'ed; the plan's own are those of plan->pgrid) */
int jn_panels_partition(const jn_plan_t *plan, int grid, uint32_t **cta, uint32_t **flush_ptr, uint32_t **flush,
			int64_t *nflush, int64_t *words);
/* panel coefficients from matrix elements in the plan's layout: FP64 into c64
 * and/or FP32 into c32 (either may be NULL), n_coef values each */
void jn_panels_coefficients(const jn_plan_t *plan, const double *me, double *c64, float *c32);
/* the 32-bit product's coefficients: c_int = round(c 2^Sc) with |c_int| <= 2^30,
 * and the shift k (>= 30) that rounds each product (c_int x_int) to a 32-bit
 * integer and keeps every element's sum below 2^62 for |x_int| <= 2^30
 * (from the plan's abs_bound).  Returns 0, or 1 when the host runs out of
 * memory. */
int jn_panels_coefficients_int(const jn_plan_t *plan, const double *me, int32_t *ci, int *Sc, int *k);
/* for every coefficient the matrix element it copies: index | sign << 31 |
 * (single-species block, where |M| < 1e-12 counts as zero) << 30; the plan
 * must hold fewer than 2^30 matrix elements */
void jn_panels_gather_index(const jn_plan_t *plan, uint32_t *gather);
/* the walk engine's plan (jn_walk.c); the walk element array must hold
 * fewer than 2^30 values.  jn_walk_free releases it (jn_plan_free does too). */
int jn_walk_build(jn_plan_t *plan, char *err, size_t errlen);
void jn_walk_free(jn_plan_t *plan);
/* the walk element array (plan->n_wme values) from matrix elements in the
 * plan's layout */
void jn_walk_elements(const jn_plan_t *plan, const double *me, double *out);
/* the integer path's elements: each element of the walk element array
 * (formed from matrix elements me in the plan's layout, as
 * jn_walk_elements forms it) scaled by its block's own 2^Sc_b so that
 * max|A| of the block is below 2^52, rounded, and split into {high 28 bits
 * (signed), low 24 bits} (two words per element); per group the shift
 * Sc_b - Sc_min (capped at 255) into gshift, and Sc_min (the smallest block
 * exponent) into *sc_min */
void jn_walk_int_elements(const jn_plan_t *plan, const double *me, int32_t *split, uint8_t *gshift, int *sc_min);

#ifdef __cplusplus
}
#endif
#endif
