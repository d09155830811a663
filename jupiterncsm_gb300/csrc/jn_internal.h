/*
 * jn_internal.h — state shared by the CUDA translation units of
 * libjncsm_gpu.so (not part of the public ABI).
 */
#ifndef JN_INTERNAL_H
#define JN_INTERNAL_H

#include <cuda_runtime.h>

#include "../../include/jncsm.h"
#include "jn_problem.h"

/* records the message of a failure for jn_last_error() and returns s (C
 * linkage: the host tools in C record their failures through it too) */
extern "C" jn_status jn_fail(jn_status s, const char *fmt, ...);

#define CUDA_TRY(call)                                                                          \
	do {                                                                                    \
		cudaError_t e_ = (call);                                                        \
		if (e_ != cudaSuccess)                                                          \
			return jn_fail(JN_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
	} while (0)

struct jn_lanczos_state;

struct jn_ctx {
	jn_plan_t plan;
	int device;
	int num_sms;
	cudaStream_t stream;
	uint32_t *d_rowptr;
	uint2 *d_ent;
	double *d_me;
	jn_term_t *d_terms;
	jn_tile_t *d_tiles;
	jn_unit_t *d_units;
	int32_t *d_unit_terms;
	double *d_partial;
	double *d_x, *d_y;      /* staging for the host-pointer entry points */
	double *h_pinned;       /* pinned staging for host copies */
	int precision;          /* 64: FP64 products; 32: FP32 matrix elements and x, compensated sums */
	float *d_me32;          /* FP32 copy of the matrix elements (built on first FP32 use) */
	float *d_x32;
	int engine;             /* the engine at the current precision: 4 panels, 5 walks, 3 block tiles, 2 warp pieces */
	int engine_of[2];       /* the engine at precision 64 [0] (default 5) and 32 [1] (default 4 up to
	                           JN_PANEL_MAX_DIM states, 5 above) */
	jn_btile_t *d_btiles;
	jn_piece_t *d_pieces;
	jn_tterm_t *d_tterms;
	uint2 *d_walks;
	unsigned int *d_items;
	int tile_grid;          /* persistent CTAs of the tile kernel */
	unsigned long long *d_gacc;     /* 64-bit fixed-point accumulator, zero between products */
	unsigned int *d_xmax;           /* [0] max|x| of the current product (FP32 bits), [1] tile counter */
	struct jn_lanczos_state *lz;
	/* panel engine (engine 4, jn_panel.cu) */
	jn_panel_t *d_panels;
	uint32_t *d_ptasks, *d_pcta, *d_pflush, *d_pflush_ptr, *d_pmeta, *d_pblocks;
	double *d_coef64;               /* panel coefficients, built on first FP64 use */
	int32_t *d_coefi;               /* and as 32-bit fixed-point integers on first 32-bit use */
	int32_t *d_xi;                  /* x as 32-bit fixed-point integers, [p][n] then transposed [n][p] */
	double *d_xt64;                 /* x with every block transposed to [n][p] (FP64 panel product) */
	int pint_sc, pint_k;            /* coefficient exponent and product shift of the 32-bit path */
	int panel_grid;                 /* persistent CTAs; 0 until set up */
	int panel_per_sm[2];            /* CTAs per SM of the FP64 [0] and FP32 [1] panel kernels (0: does not fit) */
	int panel_xs_limit;             /* dynamic shared memory the 32-bit kernel may take with x staged in it (0: never) */
	int tuned_iter[2], tuned_per[2]; /* the autotuner's panel schedule for FP64 [0] and 32-bit [1] (0: none) */
	int smem_per_sm;                /* shared memory of an SM, bytes */
	int panel_iter;                 /* rows a lane walks per panel task */
	uint32_t *d_pgather;            /* per coefficient: its matrix element | sign << 31 | skip << 30 (batched) */
	uint16_t *d_pelem;              /* per state: its basis block (the prep kernel's transposed copy) */
	/* products replayed as CUDA graphs, keyed by every argument their kernels take */
	struct jn_product_graph *graphs;
	int ngraphs, graph_next;
	cudaEvent_t prof_ev[4];         /* start, before and after the product kernel, end: recorded inside product graphs */
	/* walk engine (engine 5, jn_walk.cu) */
	int walk_ready;                 /* the walk plan is on the device */
	int walk_per_sm[3];             /* CTAs per SM of the FP32, FP64 and integer walk kernels */
	int walk_fp64;                  /* precision 64: 0 exact integers (default), 1 FP64 fused multiply-adds */
	int walk_sc;                    /* the integer path's smallest block exponent (the product's unit) */
	uint8_t *d_wgshift;             /* per row group: its block's exponent minus walk_sc */
	uint4 *d_wtasks, *d_wpieces;
	uint32_t *d_wlanes, *d_wwalks, *d_wrows, *d_wrdst, *d_wgroups;
	void *d_welem[3];               /* walk element arrays: FP32, FP64, split integers (built on first use) */
	int2 *d_wx;                     /* x converted for the product (FP32 or split 52-bit integers) */
	int2 *d_wxt;                    /* the transposed view of x that proton walks read, in the product's type */
	int32_t *d_wxperm;              /* position in x of each element of that view */
};

/* drop the cached product graphs (before any product buffer is freed) */
void jn_product_graphs_clear(jn_ctx *c);
/* install the autotuner's panel schedule for the context's precision, if it has one */
jn_status jn_panels_apply_tuned(jn_ctx *c);

/* enqueue y (+)= H x on stream st */
jn_status jn_launch_matvec(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st);

/* the block-tile product with caller-chosen scratch (see jn_matvec.cu); the
 * optional events `pre` and `mid` are recorded just before and just after
 * the tile kernel */
jn_status jn_enqueue_tiles(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st,
			   cudaEvent_t pre, cudaEvent_t mid, unsigned long long *gacc, unsigned int *ctrl, float *x32,
			   int clear_acc);

/* B products at once, instance i = blockIdx.y: y[i] = H_i x_i with the
 * context's lists and the matrix elements me + i * me_ld (FP32 when f32),
 * x_i = src + i * src_ld + (*d_sel) * sel_ld (d_sel may be NULL).
 * Scratch: x64 or x32 (B x dim), gacc (B x dim, zero on entry, left zero),
 * ctrl (2 B words).  Instances with d_active[i] == 0 are skipped.  abs_bound
 * must bound every instance's matrix elements (jn_plan_abs_bound). */
jn_status jn_enqueue_batched(jn_ctx *c, int B, int f32, const void *me, int64_t me_ld, const double *src,
			     int64_t src_ld, const int *d_sel, int64_t sel_ld, double *y, int64_t y_ld, double *x64,
			     float *x32, unsigned long long *gacc, unsigned int *ctrl, const int *d_active, double abs_bound,
			     cudaStream_t st);

/* max|x| into ctrl[0] (zeroed before) and the optional FP32 copy of x */
void jn_launch_prep(const double *d_x, float *x32, int64_t n, unsigned int *ctrl, cudaStream_t st);
/* y (+)= gacc * 2^-S with S from ctrl[0]; gacc is cleared */
void jn_launch_finalize(unsigned long long *gacc, double *d_y, int64_t n, const unsigned int *ctrl, double abs_bound,
			int accumulate, cudaStream_t st);

/* panel engine (jn_panel.cu): plan upload, coefficient reset after new
 * matrix elements, release, and the product on the context's scratch */
jn_status jn_panels_setup(jn_ctx *c);
int jn_panels_fit(const jn_ctx *c, int f32);
void jn_panels_invalidate(jn_ctx *c);
void jn_panels_release(jn_ctx *c);
jn_status jn_enqueue_panels(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st, cudaEvent_t pre,
			    cudaEvent_t mid);

/* batched panel products (jn_panel.cu): the 32-bit coefficients of B
 * instances' matrix elements (device, me + i me_ld, the context's layout)
 * into d_coef (B x n_coef) with their max|c| bits in d_cmax (B words); then
 * per step y_i = H_i x_i with x_i = src + i src_ld + (*d_sel) sel_ld.
 * Scratch: xbuf (B x 2 dim ints), gacc (B x dim, zero on entry, left zero),
 * ctrl (2 B words). */
typedef struct {
	int grid;               /* persistent CTAs per instance */
	int words;              /* the largest CTA accumulator of the partition */
	uint32_t *cta, *flush_ptr, *flush;      /* device copies of the partition */
} jn_panel_partition;
jn_status jn_panels_partition_upload(jn_ctx *c, int grid, jn_panel_partition *pp);
void jn_panels_partition_free(jn_panel_partition *pp);
jn_status jn_panels_batched_coefficients(jn_ctx *c, int B, const double *d_me, int64_t me_ld, int *d_coef,
					 unsigned long long *d_cmax, cudaStream_t st);
/* pp: the CTA partition of each instance (a batch gives each instance fewer,
 * larger chunks than a single product, so fewer blocks are cleared and
 * flushed); NULL for the context's own */
jn_status jn_enqueue_panels_batched(jn_ctx *c, int B, const int *d_coef, const unsigned long long *d_cmax,
				    const double *src, int64_t src_ld, const int *d_sel, int64_t sel_ld, double *y,
				    int64_t y_ld, int *xbuf, unsigned long long *gacc, unsigned int *ctrl,
				    const int *d_active, const jn_panel_partition *pp, cudaStream_t st);

/* walk engine (jn_walk.cu): plan upload (built on first use), coefficient
 * reset after new matrix elements, release, and the product */
jn_status jn_walk_setup(jn_ctx *c);
void jn_walk_invalidate(jn_ctx *c);
void jn_walk_release(jn_ctx *c);
jn_status jn_enqueue_walk(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st, cudaEvent_t pre,
			  cudaEvent_t mid);

/* Batched walk products over instances of several bases (all contexts on
 * one device): instance i runs on ctxs[inst_ctx[i]]'s walk plan with its own
 * matrix elements me[i] (host, that context's layout).  Per product:
 * y + i y_ld = H_i x_i with x_i = src + i src_ld + (*d_sel) sel_ld, in FP32
 * (mode 32; want32 at creation) or FP64 FMAs (mode 64), exact fixed-point
 * sums; inactive instances (d_active[i] == 0) are skipped.  max_dim bounds
 * every instance's dimension. */
struct jn_walk_batch;
jn_status jn_walk_batch_create(jn_ctx *const *ctxs, const int *inst_ctx, int B, const double *const *me, int want32,
			       struct jn_walk_batch **out);
jn_status jn_walk_batch_enqueue(struct jn_walk_batch *wb, int mode, const double *src, int64_t src_ld, const int *d_sel,
				int64_t sel_ld, double *y, int64_t y_ld, const int *d_active, int64_t max_dim,
				cudaStream_t st);
void jn_walk_batch_free(struct jn_walk_batch *wb);

/* Batched 32-bit panel products over instances of several bases: basis b
 * (ctxs[b], panel engine) has count[b] instances with FP64 matrix elements
 * d_me64[b] (device, count[b] x n_me).  Per product, as the walk batch;
 * possible when every context runs the panel engine. */
struct jn_panel_batch;
int jn_panel_batch_possible(jn_ctx *const *ctxs, int nbases);
jn_status jn_panel_batch_create(jn_ctx *const *ctxs, int nbases, const int *count, const double *const *d_me64,
				struct jn_panel_batch **out);
jn_status jn_panel_batch_enqueue(struct jn_panel_batch *pb, const double *src, int64_t src_ld, const int *d_sel,
				 int64_t sel_ld, double *y, int64_t y_ld, const int *d_active, int64_t max_dim,
				 cudaStream_t st);
void jn_panel_batch_free(struct jn_panel_batch *pb);

/* release the Lanczos state of a context */
void jn_lanczos_release(jn_ctx *c);

#endif
