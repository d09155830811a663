/*
 * jn_panel.cu — the panel engine: the index-list product as a stream over
 * compacted coefficients (engine 4; host plan in jn_panel.c).
 *
 * Semantics are the reference Minerva kernels'
 * (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:
 * n list :20-77, p list :79-132, n x p lists :134-210, off-diagonal
 * transposes :212-462, |M| < 1e-12 skip of single-species terms :52-53).
 *
 * GB300 organisation.  At set-up every instruction becomes a panel whose
 * coefficient of (proton entry, neutron entry) is s_p s_n M[k_n + Nd k_p],
 * stored densely and row-major with the shorter list as columns: the
 * product reads each coefficient once, coalesced, with streaming
 * (evict-first) loads, and the index lists only as 4-byte packed
 * (source, destination) pairs.  A warp task spreads up to 32 columns of a
 * panel over its lanes (and floor(32 / columns) rows side by side when a
 * panel is narrow) and walks rows, with the row entries and coefficients of four
 * rows in flight per lane.  Each CTA holds the blocks of y it touches as
 * 64-bit fixed-point integers in shared memory (the 32-bit product also
 * holds x there, on the same blocks), with block rows padded to an odd
 * length so that a warp walking a column touches 32 different banks: every
 * contribution is one rounding of c x 2^S to an integer (each has its own
 * coefficient), added as a 32-bit shared atomic whose rare carry goes to the
 * high word.  Integer addition is exact and
 * associative, so the result is bit-identical whatever the order in which
 * warps and CTAs run.  Persistent CTAs take contiguous runs of tasks that
 * touch few blocks, and at the end add only the touched ranges into the
 * global accumulator.
 */
#include <cooperative_groups.h>

#include "jn_internal.h"
#include "jn_fixed.cuh"

#define PANEL_THREADS 512
#define PANEL_UNROLL 4

template <typename T> __device__ __forceinline__ T load_stream(const T *p) { return __ldcs(p); }

/* One contribution c x as a 64-bit fixed-point integer.  FP64: (c x) 2^S
 * rounded once.  32-bit: c and x are 32-bit fixed-point integers; the product
 * is exact in 64 bits and is rounded once by the shift k. */
struct FixFp64 {
	double scale;
	__device__ __forceinline__ long long operator()(double c, double x) const { return to_fixed<double>(c * x * scale); }
};
#define PANEL_INT_SHIFT 30       /* the 32-bit product's rounding shift (jn_panels_coefficients_int) */
struct FixInt32 {
	__device__ __forceinline__ int operator()(int c, int x) const
	{
		return (int)(((long long)c * x + (1ll << (PANEL_INT_SHIFT - 1))) >> PANEL_INT_SHIFT);
	}
};

__device__ __forceinline__ void add_contribution(unsigned int *lo, unsigned int *hi, int i, long long v)
{
	add_fixed(lo, hi, i, v);
}
__device__ __forceinline__ void add_contribution(unsigned int *lo, unsigned int *hi, int i, int v)
{
	add_fixed32(lo, hi, i, v);
}

/* exponent Sx of the 32-bit fixed-point x: |x| 2^Sx < 2^30 for the bound max|x| in xmax_bits */
__device__ __forceinline__ int x_exponent(unsigned int xmax_bits)
{
	if (!(xmax_bits & 0x7fffffffu)) return 0;
	const int ex = (int)((xmax_bits >> 23) & 0xff) - 126;   /* xmax < 2^ex */
	const int Sx = 30 - ex;
	return Sx < -900 ? -900 : (Sx > 900 ? 900 : Sx);
}

/* round-half-even of v 2^Sx as a 32-bit integer, from the bits of v: the
 * same value as __double2int_rn(v * 2^Sx) for finite v whose scaled value
 * is below 2^31 (the scale guarantees it), without an FP64 instruction.
 * v = m 2^(e - 1075) with m the significand (implicit bit included, or the
 * subnormal's fraction with e = 1). */
__device__ __forceinline__ int fixed32_bits(double v, int Sx)
{
	const unsigned long long u = (unsigned long long)__double_as_longlong(v);
	const int ex = (int)((u >> 52) & 0x7ff);
	if (ex == 0x7ff) return __double2int_rn(v * ldexp(1.0, Sx));     /* inf, nan: as the FP64 conversion */
	unsigned long long m = u & 0xfffffffffffffull;
	int sh = Sx - 1075;
	if (ex) { m |= 1ull << 52; sh += ex; } else { sh += 1; }
	unsigned long long q;
	if (sh >= 0) {
		q = m << sh;
	} else {
		const int k = -sh;
		if (k > 63) {
			q = 0;
		} else {
			q = m >> k;
			const unsigned long long rem = m & ((1ull << k) - 1), half = 1ull << (k - 1);
			if (rem > half || (rem == half && (q & 1))) q++;
		}
	}
	const int r = (int)q;
	return (u >> 63) ? -r : r;
}

template <typename T, typename Fix, int KIND, bool DIAG, bool XS>
__device__ __forceinline__ void panel_task(const uint4 pa, const uint4 pb, const uint4 pc, const uint4 pd, uint32_t j0,
					   uint32_t j1, int R, int r, int i, unsigned int *__restrict__ lo,
					   unsigned int *__restrict__ hi, const T *__restrict__ x, const T *__restrict__ xt,
					   const T *__restrict__ coef, const uint32_t *__restrict__ meta, const Fix fix,
					   int out_soff, int in_soff, const T *__restrict__ xs)
{
	const int64_t c_off = (int64_t)pa.x | ((int64_t)pa.y << 32);
	const uint32_t row_meta = pa.z, col_meta = pa.w;
	const int out_off = (int)pb.x, in_off = (int)pb.y, Nn_out = (int)pb.z, Nn_in = (int)pb.w;
	const int ncols = (int)pc.x;
	const int Np_out = (int)pd.z, Np_in = (int)pd.w;
	/* element (row entry sr -> dr, column entry sc -> dc) reads x at (sr, sc) of the input block and
	   lands on y at (dr, dc) of the output block; the transpose swaps the two.  Lanes own columns, so
	   x is read from the copy in which a column is contiguous: x itself ([p][n]) when rows are proton
	   entries, the transposed copy ([n][p]) when they are neutron entries.  The accumulator keeps the
	   [p][n] layout with rows padded to Nn | 1 (odd: a stride-Po walk hits 32 banks). */
	const bool rows_n = KIND == JN_KIND_NP && (pc.y & JN_PANEL_ROWS_N);
	const T *__restrict__ xv = rows_n ? xt : x;
	const int Po = Nn_out | 1, Pi = Nn_in | 1;
	const int MRo = rows_n ? Np_out : Nn_out, MRi = rows_n ? Np_in : Nn_in, MCo = 1, MCi = 1;
	const int SRo = rows_n ? 1 : Po, SCo = rows_n ? Po : 1, SRi = rows_n ? 1 : Pi, SCi = rows_n ? Pi : 1;
	int sc, dc;
	if (KIND == JN_KIND_P) {
		sc = dc = i;
	} else {
		const uint32_t m = __ldg(meta + col_meta + i);
		sc = (int)(m & 0xffffu);
		dc = (int)(m >> 16);
	}
	const T *__restrict__ xi_base = xv + in_off + sc * MCi;
	const T *__restrict__ xo_base = xv + out_off + dc * MCo;
	const int ai_base = in_soff + sc * SCi, ao_base = out_soff + dc * SCo;
	const T ccol = KIND == JN_KIND_N ? __ldg(coef + c_off + i) : (T)0;
	const T *__restrict__ crow = coef + c_off + (KIND == JN_KIND_NP ? i : 0);
	for (uint32_t j = j0 + r; j < j1; j += PANEL_UNROLL * R) {
		uint32_t mr[PANEL_UNROLL];
		T cv[PANEL_UNROLL];
		/* issue the row entries and coefficients of the next rows first */
#pragma unroll
		for (int u = 0; u < PANEL_UNROLL; u++) {
			const uint32_t jj = j + u * R;
			mr[u] = jj * 0x10001u;
			cv[u] = 0;
			if (jj < j1) {
				if (KIND != JN_KIND_N) mr[u] = __ldg(meta + row_meta + jj);
				if (KIND == JN_KIND_NP) cv[u] = load_stream(crow + (int64_t)jj * ncols);
				else if (KIND == JN_KIND_P) cv[u] = __ldg(crow + jj);
				else cv[u] = ccol;
			}
		}
#pragma unroll
		for (int u = 0; u < PANEL_UNROLL; u++) {
			if (j + u * R >= j1) break;
			const int sr = (int)(mr[u] & 0xffffu), dr = (int)(mr[u] >> 16);
			/* x staged in shared memory sits at the accumulator's positions: x of the input
			   element where the transpose adds, x of the output element where the forward adds */
			const int ao = ao_base + dr * SRo, ai = ai_base + sr * SRi;
			add_contribution(lo, hi, ao, fix(cv[u], XS ? xs[ai] : __ldg(xi_base + sr * MRi)));
			if (!DIAG) add_contribution(lo, hi, ai, fix(cv[u], XS ? xs[ao] : __ldg(xo_base + dr * MRo)));
		}
	}
}

template <typename T, typename Fix, bool XS>
__device__ __forceinline__ void jn_panel_body(const uint4 *__restrict__ panels, const uint4 *__restrict__ tasks,
					      const uint32_t *__restrict__ cta_ptr, const uint32_t *__restrict__ flush,
					      const uint32_t *__restrict__ flush_ptr, const uint4 *__restrict__ blocks,
					      const uint32_t *__restrict__ meta, const T *__restrict__ coef,
					      const T *__restrict__ x, const T *__restrict__ xt,
					      unsigned long long *__restrict__ gacc, const Fix fix, int words)
{
	/* the CTA's accumulator holds only the blocks it touches (flush pairs
	   {block, offset}); bmap[block] is the block's offset in it.  With XS,
	   x of those blocks follows in the same padded layout (a CTA reads x
	   only on the blocks it adds into). */
	extern __shared__ unsigned int sacc[];
	__shared__ unsigned int next_task;
	unsigned int *lo = sacc, *hi = sacc + words, *bmap = sacc + (XS ? 3 : 2) * words;
	T *xs = XS ? (T *)(sacc + 2 * words) : NULL;
	const int lane = threadIdx.x & 31;
	const uint32_t f0 = flush_ptr[blockIdx.x], f1 = flush_ptr[blockIdx.x + 1];
	/* clear the blocks this CTA touches (padded rows) */
	for (uint32_t f = f0; f < f1; f++) {
		const uint32_t b = __ldg(flush + 2 * f), so = __ldg(flush + 2 * f + 1);
		const uint4 bk = __ldg(blocks + b);
		const uint32_t n = bk.z * (bk.w | 1u);
		if (threadIdx.x == 0) bmap[b] = so;
		for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
			lo[so + e] = 0u;
			hi[so + e] = 0u;
			if (XS) {
				const uint32_t Ns = bk.w | 1u, row = e / Ns, col = e - row * Ns;
				xs[so + e] = col < bk.w ? __ldg(x + bk.x + row * bk.w + col) : (T)0;
			}
		}
	}
	if (threadIdx.x == 0) next_task = 0;
	__syncthreads();
	const uint32_t t0 = cta_ptr[blockIdx.x], nt = cta_ptr[blockIdx.x + 1] - t0;
	for (;;) {
		uint32_t k = 0;
		if (lane == 0) k = atomicAdd(&next_task, 1u);
		k = __shfl_sync(0xffffffffu, k, 0);
		if (k >= nt) break;
		const uint4 tk = __ldg(tasks + t0 + k);
		const uint4 pa = __ldg(panels + 4 * tk.x), pb = __ldg(panels + 4 * tk.x + 1), pc = __ldg(panels + 4 * tk.x + 2);
		const uint4 pd = __ldg(panels + 4 * tk.x + 3);
		/* cw lanes per row, R = 32 / cw rows side by side: lane = r cw + c */
		const int cw = (int)(tk.w >> 24), R = 32 / cw, r = lane / cw;
		const int i = (int)(tk.w & 0xffffffu) + (lane - r * cw);
		if (r >= R || i >= (int)pc.x) continue;
		const int kind = (int)pc.y & 7;
		const bool diag = (pc.y & JN_PANEL_DIAG) != 0;
		const int so = (int)bmap[pc.z], si = (int)bmap[pc.w];
		if (kind == JN_KIND_NP) {
			if (diag) panel_task<T, Fix, JN_KIND_NP, true, XS>(pa, pb, pc, pd, tk.y, tk.z, R, r, i, lo, hi, x, xt, coef, meta, fix, so, si, xs);
			else panel_task<T, Fix, JN_KIND_NP, false, XS>(pa, pb, pc, pd, tk.y, tk.z, R, r, i, lo, hi, x, xt, coef, meta, fix, so, si, xs);
		} else if (kind == JN_KIND_N) {
			if (diag) panel_task<T, Fix, JN_KIND_N, true, XS>(pa, pb, pc, pd, tk.y, tk.z, R, r, i, lo, hi, x, xt, coef, meta, fix, so, si, xs);
			else panel_task<T, Fix, JN_KIND_N, false, XS>(pa, pb, pc, pd, tk.y, tk.z, R, r, i, lo, hi, x, xt, coef, meta, fix, so, si, xs);
		} else {
			if (diag) panel_task<T, Fix, JN_KIND_P, true, XS>(pa, pb, pc, pd, tk.y, tk.z, R, r, i, lo, hi, x, xt, coef, meta, fix, so, si, xs);
			else panel_task<T, Fix, JN_KIND_P, false, XS>(pa, pb, pc, pd, tk.y, tk.z, R, r, i, lo, hi, x, xt, coef, meta, fix, so, si, xs);
		}
	}
	__syncthreads();
	/* add the touched blocks into the global accumulator (unpadded layout) */
	for (uint32_t f = f0; f < f1; f++) {
		const uint32_t so = __ldg(flush + 2 * f + 1);
		const uint4 bk = __ldg(blocks + __ldg(flush + 2 * f));
		const uint32_t Nn = bk.w, Ns = bk.w | 1u, n = bk.z * Nn;
		for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
			const uint32_t s = so + (e / Nn) * Ns + e % Nn;
			const unsigned long long v = (unsigned long long)lo[s] | ((unsigned long long)hi[s] << 32);
			if (v) atomicAdd(gacc + bk.x + e, v);
		}
	}
}

/* the 32-bit product: coefficients and x are 32-bit fixed-point integers.
 * Batched products (many Hamiltonians on one set of lists) run instance
 * blockIdx.y with its own coefficients, x and accumulator at the given
 * strides; instances with active[i] == 0 are skipped.  XS: x staged in
 * shared memory (one more word per state) instead of gathered through L1. */
template <bool XS>
__global__ void __launch_bounds__(PANEL_THREADS, 3) jn_panel_kernel_i32(const uint4 *__restrict__ panels,
								     const uint4 *__restrict__ tasks,
								     const uint32_t *__restrict__ cta_ptr,
								     const uint32_t *__restrict__ flush,
								     const uint32_t *__restrict__ flush_ptr,
								     const uint4 *__restrict__ blocks,
								     const uint32_t *__restrict__ meta, const int *__restrict__ coef,
								     const int *__restrict__ x, const int *__restrict__ xt,
								     unsigned long long *__restrict__ gacc, const FixInt32 fix, int words,
								     int64_t coef_ld, int64_t x_ld, int64_t acc_ld,
								     const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	jn_panel_body<int, FixInt32, XS>(panels, tasks, cta_ptr, flush, flush_ptr, blocks, meta, coef + inst * coef_ld,
					 x + inst * x_ld, xt + inst * x_ld, gacc + inst * acc_ld, fix, words);
}

/* the FP64 product: the fixed-point scale 2^S comes from max|x| on the device */
__global__ void __launch_bounds__(PANEL_THREADS) jn_panel_kernel_fp64(const uint4 *__restrict__ panels,
								      const uint4 *__restrict__ tasks,
								      const uint32_t *__restrict__ cta_ptr,
								      const uint32_t *__restrict__ flush,
								      const uint32_t *__restrict__ flush_ptr,
								      const uint4 *__restrict__ blocks,
								      const uint32_t *__restrict__ meta,
								      const double *__restrict__ coef, const double *__restrict__ x,
								      const double *__restrict__ xt, unsigned long long *__restrict__ gacc,
								      const unsigned int *__restrict__ xmax_bits, double abs_bound,
								      int words)
{
	const FixFp64 fix = { ldexp(1.0, fixed_exponent(*xmax_bits, abs_bound)) };
	jn_panel_body<double, FixFp64, false>(panels, tasks, cta_ptr, flush, flush_ptr, blocks, meta, coef, x, xt, gacc, fix,
					      words);
}



/* One cluster of PREP_CTAS CTAs: max|x| into ctrl[0] (with the FP32 round-up
 * margin of the other engines' scale), then the panel kernels' copies of x:
 * the 32-bit fixed-point x in the [p][n] layout (xn, when not NULL) and the
 * copy with every block transposed to [n][p] (xt, when not NULL); FP64
 * copies x itself.
 * Each thread holds its PREP_PER states in registers across the cluster-wide
 * max (partial maxima meet in distributed shared memory), so x is read once;
 * elem[i] is the basis block of state i.  The work is integer: max|x| is the
 * largest bit pattern of |x| (NaN left out; the FP32 bound, monotone in |x|,
 * is taken once of the maximum) and the conversion works on the bits, because
 * a cluster's few SMs issue few FP64 operations per cycle on GB300. */
#define PREP_THREADS 1024
#define PREP_CTAS 8
#define PREP_PER 4
static_assert(PREP_THREADS * PREP_CTAS * PREP_PER >= JN_PANEL_MAX_DIM, "the prep cluster covers the panel engine's bases");
template <typename T>
__global__ void __cluster_dims__(PREP_CTAS, 1, 1) __launch_bounds__(PREP_THREADS)
	jn_panel_prep_kernel(const double *__restrict__ x, T *__restrict__ xn, T *__restrict__ xt,
			     const uint4 *__restrict__ blocks, const uint16_t *__restrict__ elem, int64_t dim,
			     unsigned int *__restrict__ ctrl)
{
	namespace cg = cooperative_groups;
	cg::cluster_group cluster = cg::this_cluster();
	__shared__ unsigned long long wmax[PREP_THREADS / 32];
	__shared__ unsigned long long cta_max;
	__shared__ unsigned int all_max;
	const int rank = (int)cluster.block_rank();
	double v[PREP_PER];
	unsigned long long m = 0;
#pragma unroll
	for (int u = 0; u < PREP_PER; u++) {
		const int64_t i = ((int64_t)u * PREP_CTAS + rank) * PREP_THREADS + threadIdx.x;
		v[u] = i < dim ? x[i] : 0.0;
		const unsigned long long a = (unsigned long long)__double_as_longlong(v[u]) & 0x7fffffffffffffffull;
		if (a <= 0x7ff0000000000000ull && a > m) m = a;
	}
	for (int o = 16; o; o >>= 1) {
		const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
		m = t > m ? t : m;
	}
	if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
	__syncthreads();
	if (threadIdx.x < 32) {
		m = wmax[threadIdx.x];
		for (int o = 16; o; o >>= 1) {
			const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
			m = t > m ? t : m;
		}
		if (threadIdx.x == 0) cta_max = m;
	}
	cluster.sync();
	if (threadIdx.x < 32) {
		m = threadIdx.x < PREP_CTAS ? *cluster.map_shared_rank(&cta_max, (unsigned int)threadIdx.x) : 0ull;
		for (int o = 16; o; o >>= 1) {
			const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
			m = t > m ? t : m;
		}
		if (threadIdx.x == 0) {
			const unsigned int b = __float_as_uint((float)__longlong_as_double((long long)m) * 1.0000002f);
			all_max = b;
			if (rank == 0) {
				ctrl[0] = b;
				ctrl[1] = 0u;
			}
		}
	}
	__syncthreads();
	const int Sx = x_exponent(all_max);
#pragma unroll
	for (int u = 0; u < PREP_PER; u++) {
		const int64_t i = ((int64_t)u * PREP_CTAS + rank) * PREP_THREADS + threadIdx.x;
		if (i < dim) {
			T t;
			if (sizeof(T) == 4) t = (T)fixed32_bits(v[u], Sx);
			else t = (T)v[u];
			if (xn) xn[i] = t;
			if (xt) {
				const uint4 bk = __ldg(blocks + __ldg(elem + i));
				const uint32_t e = (uint32_t)(i - bk.x), Nn = bk.w, Np = bk.z;
				xt[bk.x + (e % Nn) * Np + e / Nn] = t;
			}
		}
	}
	/* no CTA leaves while another may still read its partial maximum */
	cluster.sync();
}

/* y (+)= acc 2^(k - Sc - Sx); the accumulator is cleared for the next product */
__global__ void jn_int_finalize_kernel(unsigned long long *__restrict__ gacc, double *__restrict__ y, int64_t n,
				       const unsigned int *__restrict__ xmax_bits, int k_minus_sc, int accumulate)
{
	const double unit = ldexp(1.0, k_minus_sc - x_exponent(*xmax_bits));
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = (double)(long long)gacc[i] * unit;
		y[i] = accumulate ? y[i] + v : v;
		gacc[i] = 0ull;
	}
}

/* a CTA's accumulator (two 32-bit words per padded state of the blocks it
 * touches, at most `words`), with xs the staged 32-bit x (one word more),
 * and its block map (one word per block) */
static size_t panel_smem_words(const jn_plan_t *p, int64_t words, int xs)
{
	return (size_t)((words ? words : 1) * (xs ? 3 : 2) + p->nblocks) * sizeof(unsigned int);
}
/* The 32-bit kernel stages x in shared memory when its CTAs, `per` to an SM,
 * still fit; else it gathers x through L1. */
static int panel_use_xs(const jn_ctx *c, int64_t words, int per)
{
	const size_t s = panel_smem_words(&c->plan, words, 1);
	return c->panel_xs_limit > 0 && s <= (size_t)c->panel_xs_limit &&
	       (size_t)(per > 0 ? per : 1) * (s + 1024) <= (size_t)c->smem_per_sm;
}
static int panel_per_sm_of(const jn_ctx *c, int grid) { return c->num_sms > 0 ? (grid + c->num_sms - 1) / c->num_sms : 1; }

/* ------------------------------------------------------------------ */
template <typename T>
static jn_status upload_n(T **dst, const void *src, size_t n)
{
	size_t bytes = (n ? n : 1) * sizeof(T);
	cudaError_t e = cudaMalloc((void **)dst, bytes);
	if (e != cudaSuccess) return jn_fail(JN_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
	if (n && src) {
		e = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
		if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "cudaMemcpy failed: %s", cudaGetErrorString(e));
	}
	return JN_OK;
}

void jn_panels_release(jn_ctx *c)
{
	cudaFree(c->d_panels); cudaFree(c->d_ptasks); cudaFree(c->d_pcta); cudaFree(c->d_pflush);
	cudaFree(c->d_pflush_ptr); cudaFree(c->d_pmeta); cudaFree(c->d_coef64); cudaFree(c->d_coefi);
	cudaFree(c->d_pblocks); cudaFree(c->d_xi); cudaFree(c->d_xt64); cudaFree(c->d_pgather); cudaFree(c->d_pelem);
	c->d_pgather = NULL;
	c->d_pelem = NULL;
	c->d_pblocks = NULL;
	c->d_xi = NULL;
	c->d_xt64 = NULL;
	c->d_panels = NULL; c->d_ptasks = NULL; c->d_pcta = NULL; c->d_pflush = NULL;
	c->d_pflush_ptr = NULL; c->d_pmeta = NULL; c->d_coef64 = NULL; c->d_coefi = NULL;
	c->panel_grid = 0;
	c->panel_per_sm[0] = c->panel_per_sm[1] = 0;
}

int jn_panels_fit(const jn_ctx *c, int f32) { return c->panel_grid > 0 && c->panel_per_sm[f32 ? 1 : 0] > 0; }

/* Ask for the smallest shared-memory carveout that still holds the CTAs an
 * SM runs: the rest of the SM's unified memory serves as L1, which caches x
 * and the list entries for the product kernels.  The carveout is an
 * attribute of the kernel, shared by every context of the process, so it
 * only grows: the largest any context needs (occupancy queries run at the
 * full carveout, see jn_panels_setup).  A hint: the runtime takes a larger
 * carveout where a launch needs one. */
static int g_carveout[3];
static void set_carveout(jn_ctx *c)
{
	const int max_smem = c->smem_per_sm;
	if (max_smem <= 0) return;
	const int per = panel_per_sm_of(c, c->panel_grid);
	/* [0] FP64, [1] 32-bit with x through L1, [2] 32-bit with x in shared memory */
	for (int v = 0; v < 3; v++) {
		if (v == 2 && !panel_use_xs(c, c->plan.pcta_words, per)) continue;
		const size_t smem = panel_smem_words(&c->plan, c->plan.pcta_words, v == 2) + 1024;   /* and the runtime's per-CTA reserve */
		int pct = (int)((100 * per * smem + max_smem - 1) / max_smem);
		if (pct > 100) pct = 100;
		if (pct > g_carveout[v]) g_carveout[v] = pct;
		if (v == 0) cudaFuncSetAttribute(jn_panel_kernel_fp64, cudaFuncAttributePreferredSharedMemoryCarveout, g_carveout[0]);
		else if (v == 1) cudaFuncSetAttribute(jn_panel_kernel_i32<false>, cudaFuncAttributePreferredSharedMemoryCarveout, g_carveout[1]);
		else cudaFuncSetAttribute(jn_panel_kernel_i32<true>, cudaFuncAttributePreferredSharedMemoryCarveout, g_carveout[2]);
	}
	cudaGetLastError();
}

jn_status jn_panels_setup(jn_ctx *c)
{
	jn_plan_t *p = &c->plan;
	if (p->dim > JN_PANEL_MAX_DIM) return jn_fail(JN_ERR_INVALID, "dimension %lld is above the panel engine's %d",
						       (long long)p->dim, JN_PANEL_MAX_DIM);
	if (c->panel_grid) return JN_OK;
	/* CTAs per SM at each precision; the FP64 kernel may not fit where the FP32 one does */
	int per[2] = { 0, 0 };
	char err[512] = { 0 };
	/* the accumulator layout does not depend on the grid: plan once to size it */
	if (jn_panels_build(p, 1, JN_PANEL_ITER, err, sizeof err)) return jn_fail(JN_ERR_NOMEM, "panel plan: %s", err);
	for (int f32 = 0; f32 < 2; f32++) {
		const size_t smem = panel_smem_words(p, p->pcta_words, 0);
		/* the occupancy query follows the carveout hint: ask at the full carveout */
		if (f32) cudaFuncSetAttribute(jn_panel_kernel_i32<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
		else cudaFuncSetAttribute(jn_panel_kernel_fp64, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
		/* the kernels' dynamic shared-memory limit is shared by every context of the
		   process as well: it only grows */
		static size_t g_smem_limit[2];
		if (smem > g_smem_limit[f32]) g_smem_limit[f32] = smem;
		cudaError_t e = f32 ? cudaFuncSetAttribute(jn_panel_kernel_i32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
							   (int)g_smem_limit[1])
				    : cudaFuncSetAttribute(jn_panel_kernel_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
							   (int)g_smem_limit[0]);
		if (e == cudaSuccess)
			e = f32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[1], jn_panel_kernel_i32<false>, PANEL_THREADS, smem)
				: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[0], jn_panel_kernel_fp64, PANEL_THREADS, smem);
		if (e != cudaSuccess) {
			per[f32] = 0;
			cudaGetLastError();
		}
	}
	if (per[1] < 1) return jn_fail(JN_ERR_INVALID, "the panel kernel does not fit on an SM for dimension %lld", (long long)p->dim);
	c->panel_per_sm[0] = per[0];
	c->panel_per_sm[1] = per[1];
	/* the 32-bit kernel with x in shared memory: allowed up to the whole
	   vector's need (the grid-1 plan above), within the per-CTA maximum;
	   each launch takes it where its CTAs still fit (panel_use_xs) */
	{
		int optin = 0, smsm = 0;
		if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device) != cudaSuccess ||
		    cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device) != cudaSuccess)
			optin = smsm = 0;
		c->smem_per_sm = smsm;
		size_t want = panel_smem_words(p, p->pcta_words, 1);
		if (want > (size_t)optin) want = (size_t)optin;
		static size_t g_xs_limit;
		if (want > g_xs_limit) g_xs_limit = want;
		c->panel_xs_limit = 0;
		if (g_xs_limit > 0 && cudaFuncSetAttribute(jn_panel_kernel_i32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
							   (int)g_xs_limit) == cudaSuccess)
			c->panel_xs_limit = (int)g_xs_limit;
		cudaGetLastError();
	}
	/* the task split is the same for every grid; CTAs take contiguous runs of the FP32 grid */
	if (jn_panels_build(p, c->num_sms * per[1], JN_PANEL_ITER, err, sizeof err))
		return jn_fail(JN_ERR_NOMEM, "panel plan: %s", err);
	c->panel_iter = JN_PANEL_ITER;
	jn_status s;
	if ((s = upload_n(&c->d_panels, p->panels, (size_t)p->npanels)) ||
	    (s = upload_n(&c->d_ptasks, p->ptasks, (size_t)p->nptasks * 4)) ||
	    (s = upload_n(&c->d_pcta, p->pcta, (size_t)p->pgrid + 1)) ||
	    (s = upload_n(&c->d_pflush_ptr, p->pflush_ptr, (size_t)p->pgrid + 1)) ||
	    (s = upload_n(&c->d_pflush, p->pflush, (size_t)p->npflush * 2)) ||
	    (s = upload_n(&c->d_pblocks, p->pblocks, (size_t)p->nblocks * 4)) ||
	    (s = upload_n(&c->d_pmeta, p->pmeta, (size_t)p->n_pmeta))) {
		jn_panels_release(c);
		return s;
	}
	{
		uint16_t *elem = (uint16_t *)malloc((size_t)(p->dim ? p->dim : 1) * sizeof(uint16_t));
		if (!elem) {
			jn_panels_release(c);
			return jn_fail(JN_ERR_NOMEM, "out of host memory");
		}
		for (int b = 0; b < p->nblocks; b++)
			for (int64_t i = 0; i < p->blocks[b].Np * p->blocks[b].Nn; i++) elem[p->blocks[b].offset + i] = (uint16_t)b;
		s = upload_n(&c->d_pelem, elem, (size_t)p->dim);
		free(elem);
		if (s) {
			jn_panels_release(c);
			return s;
		}
	}
	c->panel_grid = p->pgrid;
	set_carveout(c);
	return JN_OK;
}

/* coefficients of the context's matrix elements (built on first use at each
 * precision and after the matrix elements change): FP64, or 32-bit
 * fixed-point integers with their exponent Sc and product shift k */
static jn_status ensure_coefficients(jn_ctx *c, int f32)
{
	const jn_plan_t *p = &c->plan;
	if (f32 ? c->d_coefi != NULL : c->d_coef64 != NULL) return JN_OK;
	const size_t n = (size_t)(p->n_coef ? p->n_coef : 1);
	void *h = malloc(n * (f32 ? sizeof(int32_t) : sizeof(double)));
	if (!h) return jn_fail(JN_ERR_NOMEM, "out of host memory for %zu panel coefficients", n);
	jn_status s = JN_OK;
	if (f32) {
		if (jn_panels_coefficients_int(p, p->me, (int32_t *)h, &c->pint_sc, &c->pint_k))
			s = jn_fail(JN_ERR_NOMEM, "out of host memory for %zu panel coefficients", n);
		else if (c->pint_k != PANEL_INT_SHIFT)
			s = jn_fail(JN_ERR_INVALID, "32-bit panel product: the matrix elements need a rounding shift of %d", c->pint_k);
		if (!s) s = upload_n(&c->d_coefi, h, (size_t)p->n_coef);
	} else {
		jn_panels_coefficients(p, p->me, (double *)h, NULL);
		s = upload_n(&c->d_coef64, h, (size_t)p->n_coef);
	}
	free(h);
	return s;
}

void jn_panels_invalidate(jn_ctx *c)
{
	cudaFree(c->d_coef64);
	cudaFree(c->d_coefi);
	c->d_coef64 = NULL;
	c->d_coefi = NULL;
}

/* Everything the three kernels of one product take: a cached graph whose
 * signature equals the current one launches exactly what direct launches
 * would (device arrays are read when the graph runs, not when it is made). */
typedef struct {
	const void *x, *y, *panels, *tasks, *cta, *flush, *flush_ptr, *blocks, *meta, *coef, *xi, *xt, *gacc, *ctrl, *elem;
	const void *stream, *start, *pre, *mid, *end;
	int64_t dim;
	double abs_bound;
	size_t smem;
	int f32, xs, accumulate, grid, words, kshift, fin_grid;
} panel_sig_t;

struct jn_product_graph {
	panel_sig_t sig;
	cudaGraphExec_t exec;
};

#define PRODUCT_GRAPHS 8

void jn_product_graphs_clear(jn_ctx *c)
{
	for (int i = 0; i < c->ngraphs; i++) cudaGraphExecDestroy(c->graphs[i].exec);
	free(c->graphs);
	c->graphs = NULL;
	c->ngraphs = c->graph_next = 0;
}

static void panel_launch(const panel_sig_t *g, int has_tasks, int capturing)
{
	const unsigned int evflags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
	cudaStream_t st = (cudaStream_t)g->stream;
	const uint4 *blocks = (const uint4 *)g->blocks;
	unsigned int *ctrl = (unsigned int *)g->ctrl;
	if (g->start) cudaEventRecordWithFlags((cudaEvent_t)g->start, st, evflags);
	if (g->f32)
		/* the kernel that stages x in shared memory reads only the [p][n] copy */
		jn_panel_prep_kernel<int><<<PREP_CTAS, PREP_THREADS, 0, st>>>((const double *)g->x, (int *)g->xi,
									 g->xs && has_tasks ? NULL : (int *)g->xt, blocks,
									 (const uint16_t *)g->elem, g->dim, ctrl);
	else
		jn_panel_prep_kernel<double><<<PREP_CTAS, PREP_THREADS, 0, st>>>((const double *)g->x, NULL, (double *)g->xt, blocks,
									    (const uint16_t *)g->elem, g->dim, ctrl);
	if (g->pre) cudaEventRecordWithFlags((cudaEvent_t)g->pre, st, evflags);
	if (has_tasks) {
		if (g->f32) {
			const FixInt32 fix = {};
			(g->xs ? jn_panel_kernel_i32<true> : jn_panel_kernel_i32<false>)<<<g->grid, PANEL_THREADS, g->smem, st>>>(
				(const uint4 *)g->panels, (const uint4 *)g->tasks, (const uint32_t *)g->cta, (const uint32_t *)g->flush,
				(const uint32_t *)g->flush_ptr, blocks, (const uint32_t *)g->meta, (const int *)g->coef,
				(const int *)g->xi, (const int *)g->xt, (unsigned long long *)g->gacc, fix, g->words, 0, 0, 0, NULL);
		} else {
			jn_panel_kernel_fp64<<<g->grid, PANEL_THREADS, g->smem, st>>>(
				(const uint4 *)g->panels, (const uint4 *)g->tasks, (const uint32_t *)g->cta, (const uint32_t *)g->flush,
				(const uint32_t *)g->flush_ptr, blocks, (const uint32_t *)g->meta, (const double *)g->coef,
				(const double *)g->x, (const double *)g->xt, (unsigned long long *)g->gacc, ctrl, g->abs_bound, g->words);
		}
	}
	if (g->mid) cudaEventRecordWithFlags((cudaEvent_t)g->mid, st, evflags);
	if (g->f32)
		jn_int_finalize_kernel<<<g->fin_grid, 256, 0, st>>>((unsigned long long *)g->gacc, (double *)g->y, g->dim, ctrl,
								   g->kshift, g->accumulate);
	else
		jn_launch_finalize((unsigned long long *)g->gacc, (double *)g->y, g->dim, ctrl, g->abs_bound, g->accumulate, st);
	if (g->end) cudaEventRecordWithFlags((cudaEvent_t)g->end, st, evflags);
}

/* y (+)= H x on the panel engine.  The product runs as a cached CUDA graph
 * (one launch instead of three kernels) unless the stream is already being
 * captured, in which case its kernels join that capture.  Profiled
 * products (the context's profiling events as `pre` and `mid`) record their
 * start, kernel and end events from inside the graph; other events are
 * recorded by direct launches. */
jn_status jn_enqueue_panels(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st, cudaEvent_t pre,
			    cudaEvent_t mid)
{
	const jn_plan_t *p = &c->plan;
	const int f32 = c->precision == 32;
	jn_status s = jn_panels_setup(c);
	if (!s && !jn_panels_fit(c, f32)) s = jn_fail(JN_ERR_INVALID, "the FP64 panel kernel does not fit for dimension %lld",
						      (long long)p->dim);
	if (!s) s = ensure_coefficients(c, f32);
	if (!s && !c->d_xi) s = upload_n(&c->d_xi, NULL, (size_t)p->dim * 2);
	if (!s && !c->d_xt64) s = upload_n(&c->d_xt64, NULL, (size_t)p->dim);
	if (s) return s;
	if (!p->dim) return JN_OK;
	panel_sig_t g;
	memset(&g, 0, sizeof g);
	g.x = d_x; g.y = d_y; g.panels = c->d_panels; g.tasks = c->d_ptasks; g.cta = c->d_pcta; g.flush = c->d_pflush;
	g.flush_ptr = c->d_pflush_ptr; g.blocks = c->d_pblocks; g.meta = c->d_pmeta; g.gacc = c->d_gacc; g.ctrl = c->d_xmax;
	g.elem = c->d_pelem; g.stream = st; g.pre = pre; g.mid = mid; g.dim = p->dim; g.f32 = f32;
	if (pre == c->prof_ev[1] && mid == c->prof_ev[2]) {
		/* profiled: the product's own start and end, recorded on the device */
		g.start = c->prof_ev[0];
		g.end = c->prof_ev[3];
	}
	g.accumulate = accumulate; g.grid = c->panel_grid; g.words = (int)p->pcta_words;
	g.xs = f32 && panel_use_xs(c, p->pcta_words, panel_per_sm_of(c, c->panel_grid));
	g.smem = panel_smem_words(p, p->pcta_words, g.xs);
	g.fin_grid = (int)((p->dim + 255) / 256);
	if (g.fin_grid > 1024) g.fin_grid = 1024;
	if (f32) {
		g.coef = c->d_coefi; g.xi = c->d_xi; g.xt = c->d_xi + p->dim; g.kshift = c->pint_k - c->pint_sc;
	} else {
		g.coef = c->d_coef64; g.xt = c->d_xt64; g.abs_bound = p->abs_bound;
	}
	const int has_tasks = p->nptasks > 0;
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	const int graphable = (!pre || pre == c->prof_ev[1]) && (!mid || mid == c->prof_ev[2]) &&
			      cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
	cudaGetLastError();
	if (!graphable) {
		panel_launch(&g, has_tasks, 0);
	} else {
		int hit = -1;
		for (int i = 0; i < c->ngraphs && hit < 0; i++)
			if (!memcmp(&c->graphs[i].sig, &g, sizeof g)) hit = i;
		if (hit < 0) {
			cudaGraph_t graph = NULL;
			cudaGraphExec_t exec = NULL;
			if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
				panel_launch(&g, has_tasks, 1);
				if (cudaStreamEndCapture(st, &graph) == cudaSuccess && graph &&
				    cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
					exec = NULL;
				if (graph) cudaGraphDestroy(graph);
			}
			cudaGetLastError();
			if (exec) {
				if (!c->graphs) c->graphs = (struct jn_product_graph *)calloc(PRODUCT_GRAPHS, sizeof *c->graphs);
				if (c->graphs) {
					hit = c->ngraphs < PRODUCT_GRAPHS ? c->ngraphs++ : c->graph_next;
					if (hit == c->graph_next && c->ngraphs == PRODUCT_GRAPHS && c->graphs[hit].exec)
						cudaGraphExecDestroy(c->graphs[hit].exec);
					c->graph_next = (hit + 1) % PRODUCT_GRAPHS;
					c->graphs[hit].sig = g;
					c->graphs[hit].exec = exec;
				} else {
					cudaGraphExecDestroy(exec);
				}
			}
		}
		if (hit >= 0) {
			cudaError_t e = cudaGraphLaunch(c->graphs[hit].exec, st);
			if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "panel product graph launch: %s", cudaGetErrorString(e));
		} else {
			panel_launch(&g, has_tasks, 0);   /* capture unavailable: launch directly */
		}
	}
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "panel product launch: %s", cudaGetErrorString(e));
	return JN_OK;
}

/* ------------------------------------------------------------------ */
/* schedule and autotuner                                              */
/* ------------------------------------------------------------------ */
/* replace the task split and the persistent grid of the panel plan (the
 * panels, list entries, blocks and coefficients stay) */
static jn_status panel_schedule(jn_ctx *c, int iter, int per_sm)
{
	jn_plan_t *p = &c->plan;
	char err[512] = { 0 };
	if (per_sm < 1 || per_sm > c->panel_per_sm[1] || (c->panel_per_sm[0] && per_sm > c->panel_per_sm[0]))
		return jn_fail(JN_ERR_INVALID, "%d CTAs per SM: the panel kernels fit %d (FP64 %d)", per_sm, c->panel_per_sm[1],
			       c->panel_per_sm[0]);
	if (iter < 1 || iter > 4096) return jn_fail(JN_ERR_INVALID, "%d rows per lane: must be in 1..4096", iter);
	if (jn_panels_build(p, c->num_sms * per_sm, iter, err, sizeof err)) {
		/* the host plan is gone: drop the device side too, products fall back to block tiles */
		jn_panels_release(c);
		return jn_fail(JN_ERR_NOMEM, "panel plan: %s", err);
	}
	cudaFree(c->d_ptasks); cudaFree(c->d_pcta); cudaFree(c->d_pflush); cudaFree(c->d_pflush_ptr);
	c->d_ptasks = c->d_pcta = c->d_pflush = c->d_pflush_ptr = NULL;
	jn_status s;
	if ((s = upload_n(&c->d_ptasks, p->ptasks, (size_t)p->nptasks * 4)) ||
	    (s = upload_n(&c->d_pcta, p->pcta, (size_t)p->pgrid + 1)) ||
	    (s = upload_n(&c->d_pflush_ptr, p->pflush_ptr, (size_t)p->pgrid + 1)) ||
	    (s = upload_n(&c->d_pflush, p->pflush, (size_t)p->npflush * 2))) {
		jn_panels_release(c);
		return s;
	}
	c->panel_grid = p->pgrid;
	c->panel_iter = iter;
	set_carveout(c);
	return JN_OK;
}

extern "C" jn_status jn_set_panel_schedule(jn_ctx *c, int rows_per_lane, int ctas_per_sm)
{
	if (!c) return jn_fail(JN_ERR_INVALID, "null argument");
	jn_status s = jn_panels_setup(c);
	/* an explicit schedule holds at both precisions */
	c->tuned_iter[0] = c->tuned_iter[1] = 0;
	return s ? s : panel_schedule(c, rows_per_lane, ctas_per_sm);
}

jn_status jn_panels_apply_tuned(jn_ctx *c)
{
	const int f32 = c->precision == 32;
	const int it = c->tuned_iter[f32], per = c->tuned_per[f32];
	if (!c->panel_grid || !it || (it == c->panel_iter && c->num_sms * per == c->panel_grid)) return JN_OK;
	return panel_schedule(c, it, per);
}

/* median CUDA-event time of the product kernel over `trials` products (after
 * one warm-up), each product after a write of `flush_bytes` at `flush` (when
 * not NULL) that leaves L2 holding none of the product's data */
static jn_status time_product(jn_ctx *c, int trials, float *ms, void *flush, size_t flush_bytes)
{
	float t[64];
	if (trials > 64) trials = 64;
	for (int k = -1; k < trials; k++) {
		float m[2];
		if (flush) CUDA_TRY(cudaMemsetAsync(flush, k & 0xff, flush_bytes, c->stream));
		jn_status s = jn_matvec_profile(c, c->d_x, c->d_y, 0, m);
		if (s) return s;
		if (k >= 0) t[k] = m[0];
	}
	for (int i = 1; i < trials; i++)
		for (int j = i; j > 0 && t[j] < t[j - 1]; j--) { float u = t[j]; t[j] = t[j - 1]; t[j - 1] = u; }
	*ms = t[trials / 2];
	return JN_OK;
}

__global__ void jn_tune_x_kernel(double *x, int64_t n)
{
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		x[i] = 1.0 + 0.5 * sin(0.37 * (double)i);
}

static jn_status autotune(jn_ctx *c, int trials, int tune_engine, jn_tuning *out, void *flush, size_t flush_bytes);

/* The candidates are timed with L2 flushed before every product: the
 * schedule that is fastest with the coefficients resident in L2 (they fit
 * there for small bases) can be a slow one when they stream from HBM. */
extern "C" jn_status jn_autotune(jn_ctx *c, int trials, int tune_engine, jn_tuning *out)
{
	if (!c || !out) return jn_fail(JN_ERR_INVALID, "null argument");
	int l2 = 0;
	void *flush = NULL;
	size_t bytes = 0;
	if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device) == cudaSuccess && l2 > 0) {
		bytes = 2 * (size_t)l2;
		if (cudaMalloc(&flush, bytes) != cudaSuccess) flush = NULL;
	}
	cudaGetLastError();
	/* the panel schedule is tuned at both precisions (the FP64 kernel is
	   bound by the FP64 pipe, the 32-bit one by instruction issue: they
	   favour different task lengths); jn_set_precision installs the other
	   one.  `out` reports the context's own precision. */
	const int prec0 = c->precision, f32_0 = prec0 == 32;
	c->tuned_iter[0] = c->tuned_iter[1] = 0;
	jn_status s = autotune(c, trials, tune_engine, out, flush, bytes);
	if (!s) c->engine_of[f32_0] = c->engine;      /* the choice holds for this precision */
	if (!s && out->engine == 4) {
		c->tuned_iter[f32_0] = out->rows_per_lane;
		c->tuned_per[f32_0] = out->ctas_per_sm;
		jn_tuning other;
		const int prec1 = f32_0 ? 64 : 32;
		if (jn_panels_fit(c, !f32_0) && jn_set_precision(c, prec1) == JN_OK) {
			if (autotune(c, trials, 0, &other, flush, bytes) == JN_OK && other.engine == 4) {
				c->tuned_iter[!f32_0] = other.rows_per_lane;
				c->tuned_per[!f32_0] = other.ctas_per_sm;
			}
			c->precision = prec0;
			c->engine = c->engine_of[f32_0];
			s = panel_schedule(c, out->rows_per_lane, out->ctas_per_sm);
		}
	}
	if (flush) {
		cudaStreamSynchronize(c->stream);
		cudaFree(flush);
	}
	return s;
}

static jn_status autotune(jn_ctx *c, int trials, int tune_engine, jn_tuning *out, void *flush, size_t flush_bytes)
{
	if (trials < 1) trials = 5;
	memset(out, 0, sizeof *out);
	const jn_plan_t *p = &c->plan;
	const int f32 = c->precision == 32;
	jn_tune_x_kernel<<<64, 256, 0, c->stream>>>(c->d_x, p->dim);
	CUDA_TRY(cudaGetLastError());
	const int engine0 = c->engine;
	float best = 3.4e38f;
	int best_engine = engine0, best_iter = c->panel_iter, best_per = c->panel_grid / (c->num_sms ? c->num_sms : 1);
	if (jn_panels_setup(c) == JN_OK && jn_panels_fit(c, f32) && (engine0 == 4 || tune_engine)) {
		const int iters[] = { 8, 16, 32, 64, 128 };
		const int maxper = c->panel_per_sm[0] && c->panel_per_sm[0] < c->panel_per_sm[1] ? c->panel_per_sm[0]
												    : c->panel_per_sm[1];
		c->engine = 4;
		for (size_t a = 0; a < sizeof iters / sizeof iters[0]; a++)
			for (int per = 1; per <= maxper; per++) {
				float ms;
				jn_status s = panel_schedule(c, iters[a], per);
				if (!s) s = time_product(c, trials, &ms, flush, flush_bytes);
				if (s) { c->engine = engine0; return s; }
				out->candidates++;
				if (ms < best) { best = ms; best_engine = 4; best_iter = iters[a]; best_per = per; }
			}
	}
	/* the walk and block-tile engines have no schedule to tune: each is one candidate */
	for (int eng = 5; eng >= 3; eng -= 2) {
		if (!(tune_engine || engine0 == eng)) continue;
		if (eng == 5 && jn_walk_setup(c) != JN_OK) continue;
		if (eng == 3 && p->btiles_off) continue;        /* no block tiles for this plan */
		float ms;
		c->engine = eng;
		jn_status s = time_product(c, trials, &ms, flush, flush_bytes);
		if (s) { c->engine = engine0; return s; }
		out->candidates++;
		if (ms < best) { best = ms; best_engine = eng; }
	}
	c->engine = best_engine;
	if (best_engine == 4) {
		jn_status s = panel_schedule(c, best_iter, best_per);
		if (s) return s;
	}
	out->engine = best_engine;
	out->rows_per_lane = best_engine == 4 ? best_iter : 0;
	out->ctas_per_sm = best_engine == 4 ? best_per : 0;
	out->ms = best;
	return JN_OK;
}

/* ------------------------------------------------------------------ */
/* batched products: many Hamiltonians on the context's lists           */
/* ------------------------------------------------------------------ */
/* per coefficient: the matrix element it comes from, bit 31 its sign, bit 30
 * the single-species |M| < 1e-12 skip */
jn_status jn_panels_gather(jn_ctx *c)
{
	jn_plan_t *p = &c->plan;
	if (c->d_pgather) return JN_OK;
	jn_status s = jn_panels_setup(c);
	if (s) return s;
	if (p->n_me >= (1ll << 30)) return jn_fail(JN_ERR_INVALID, "%lld matrix elements: too many for the batched panel product",
						 (long long)p->n_me);
	uint32_t *g = (uint32_t *)malloc((p->n_coef ? p->n_coef : 1) * sizeof(uint32_t));
	if (!g) return jn_fail(JN_ERR_NOMEM, "out of host memory");
	jn_panels_gather_index(p, g);
	s = upload_n(&c->d_pgather, g, (size_t)p->n_coef);
	free(g);
	return s;
}

/* bits of max |coefficient| of instance blockIdx.y (non-negative doubles order as their bits) */
__global__ void jn_coef_max_kernel(const uint32_t *__restrict__ gather, int64_t n, const double *__restrict__ me,
				   int64_t me_ld, unsigned long long *__restrict__ cmax)
{
	const int inst = blockIdx.y;
	const double *m = me + inst * me_ld;
	double v = 0.0;
	for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
		const uint32_t g = gather[e];
		double a = fabs(m[g & 0x3fffffffu]);
		if ((g & 0x40000000u) && a < 1e-12) a = 0.0;
		v = fmax(v, a);
	}
	for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
	if ((threadIdx.x & 31) == 0 && v > 0.0) atomicMax(cmax + inst, (unsigned long long)__double_as_longlong(v));
}

/* coefficient exponent Sc = 30 - e with cmax < 2^e (0 for an all-zero instance) */
__device__ __forceinline__ int coef_exponent(unsigned long long cmax_bits)
{
	if (!cmax_bits) return 0;
	return 30 - ((int)((cmax_bits >> 52) & 0x7ff) - 1022);
}

__global__ void jn_coef_build_kernel(const uint32_t *__restrict__ gather, int64_t n, const double *__restrict__ me,
				     int64_t me_ld, const unsigned long long *__restrict__ cmax, int *__restrict__ coef,
				     int64_t coef_ld)
{
	const int inst = blockIdx.y;
	const double *m = me + inst * me_ld;
	const double s = ldexp(1.0, coef_exponent(cmax[inst]));
	int *out = coef + inst * coef_ld;
	for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
		const uint32_t g = gather[e];
		double v = m[g & 0x3fffffffu];
		if ((g & 0x40000000u) && fabs(v) < 1e-12) v = 0.0;
		if (g & 0x80000000u) v = -v;
		out[e] = (int)__double2ll_rn(v * s);
	}
}

jn_status jn_panels_batched_coefficients(jn_ctx *c, int B, const double *d_me, int64_t me_ld, int *d_coef,
					 unsigned long long *d_cmax, cudaStream_t st)
{
	const jn_plan_t *p = &c->plan;
	jn_status s = jn_panels_gather(c);
	if (s) return s;
	CUDA_TRY(cudaMemsetAsync(d_cmax, 0, (size_t)B * sizeof(unsigned long long), st));
	const int g = (int)(p->n_coef / 256 + 1 < 256 ? p->n_coef / 256 + 1 : 256);
	if (p->n_coef) {
		jn_coef_max_kernel<<<dim3(g, B), 256, 0, st>>>(c->d_pgather, p->n_coef, d_me, me_ld, d_cmax);
		jn_coef_build_kernel<<<dim3(g, B), 256, 0, st>>>(c->d_pgather, p->n_coef, d_me, me_ld, d_cmax, d_coef,
								   p->n_coef);
	}
	CUDA_TRY(cudaGetLastError());
	return JN_OK;
}

/* instance blockIdx.y: max|x| of x_i = src + i src_ld + (*sel) sel_ld into ctrl[2 i] */
__global__ void jn_xmax_batched_kernel(const double *__restrict__ src, int64_t src_ld, const int *__restrict__ sel,
				       int64_t sel_ld, int64_t n, unsigned int *__restrict__ ctrl,
				       const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const double *x = src + inst * src_ld + (sel ? (int64_t)(*sel) * sel_ld : 0);
	float m = 0.0f;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		m = fmaxf(m, (float)fabs(x[i]) * 1.0000002f);
	for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(ctrl + 2 * inst, __float_as_uint(m));
}

/* block blockIdx.x of instance blockIdx.y: x_i as 32-bit fixed point, [p][n] and transposed [n][p] */
__global__ void jn_panel_x_batched_kernel(const double *__restrict__ src, int64_t src_ld, const int *__restrict__ sel,
					  int64_t sel_ld, int *__restrict__ xi, int64_t dim, const uint4 *__restrict__ blocks,
					  const unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const double *x = src + inst * src_ld + (sel ? (int64_t)(*sel) * sel_ld : 0);
	int *xn = xi + inst * 2 * dim, *xt = xn + dim;
	const uint4 bk = blocks[blockIdx.x];
	const uint32_t Np = bk.z, Nn = bk.w, n = Np * Nn;
	const double s = ldexp(1.0, x_exponent(ctrl[2 * inst]));
	for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
		const int t = __double2int_rn(x[bk.x + e] * s);
		xn[bk.x + e] = t;
		xt[bk.x + (e % Nn) * Np + e / Nn] = t;
	}
}

/* y_i (=) acc_i 2^(30 - Sc_i - Sx_i); the accumulator is cleared */
__global__ void jn_int_finalize_batched_kernel(unsigned long long *__restrict__ gacc, double *__restrict__ y, int64_t y_ld,
					       int64_t n, const unsigned int *__restrict__ ctrl,
					       const unsigned long long *__restrict__ cmax, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const double unit = ldexp(1.0, PANEL_INT_SHIFT - coef_exponent(cmax[inst]) - x_exponent(ctrl[2 * inst]));
	unsigned long long *g = gacc + inst * n;
	double *yy = y + inst * y_ld;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		yy[i] = (double)(long long)g[i] * unit;
		g[i] = 0ull;
	}
}

jn_status jn_panels_partition_upload(jn_ctx *c, int grid, jn_panel_partition *pp)
{
	memset(pp, 0, sizeof *pp);
	jn_status s = jn_panels_setup(c);
	if (s) return s;
	uint32_t *cta = NULL, *fptr = NULL, *flush = NULL;
	int64_t nf = 0, words = 0;
	if (jn_panels_partition(&c->plan, grid, &cta, &fptr, &flush, &nf, &words))
		return jn_fail(JN_ERR_NOMEM, "out of host memory");
	pp->words = (int)words;
	if ((s = upload_n(&pp->cta, cta, (size_t)grid + 1)) || (s = upload_n(&pp->flush_ptr, fptr, (size_t)grid + 1)) ||
	    (s = upload_n(&pp->flush, flush, (size_t)nf * 2)))
		jn_panels_partition_free(pp);
	else
		pp->grid = grid;
	free(cta); free(fptr); free(flush);
	return s;
}

void jn_panels_partition_free(jn_panel_partition *pp)
{
	cudaFree(pp->cta); cudaFree(pp->flush_ptr); cudaFree(pp->flush);
	memset(pp, 0, sizeof *pp);
}

jn_status jn_enqueue_panels_batched(jn_ctx *c, int B, const int *d_coef, const unsigned long long *d_cmax,
				    const double *src, int64_t src_ld, const int *d_sel, int64_t sel_ld, double *y,
				    int64_t y_ld, int *xbuf, unsigned long long *gacc, unsigned int *ctrl,
				    const int *d_active, const jn_panel_partition *pp, cudaStream_t st)
{
	const jn_plan_t *p = &c->plan;
	if (!jn_panels_fit(c, 1)) return jn_fail(JN_ERR_INVALID, "the panel engine is not set up for this context");
	if (B < 1 || B > 65535) return jn_fail(JN_ERR_INVALID, "batch of %d instances", B);
	if (!p->dim) return JN_OK;
	int g = (int)((p->dim + 255) / 256);
	if (g > 256) g = 256;
	CUDA_TRY(cudaMemsetAsync(ctrl, 0, (size_t)2 * B * sizeof(unsigned int), st));
	jn_xmax_batched_kernel<<<dim3(g, B), 256, 0, st>>>(src, src_ld, d_sel, sel_ld, p->dim, ctrl, d_active);
	jn_panel_x_batched_kernel<<<dim3(p->nblocks, B), 256, 0, st>>>(src, src_ld, d_sel, sel_ld, xbuf, p->dim,
									 (const uint4 *)c->d_pblocks, ctrl, d_active);
	if (p->nptasks) {
		const FixInt32 fix = {};
		const int grid = pp ? pp->grid : c->panel_grid;
		const int64_t words = pp ? pp->words : p->pcta_words;
		const int xs = panel_use_xs(c, words, panel_per_sm_of(c, grid));
		(xs ? jn_panel_kernel_i32<true> : jn_panel_kernel_i32<false>)<<<dim3(grid, B), PANEL_THREADS,
									      panel_smem_words(p, words, xs), st>>>(
			(const uint4 *)c->d_panels, (const uint4 *)c->d_ptasks, pp ? pp->cta : c->d_pcta,
			pp ? pp->flush : c->d_pflush, pp ? pp->flush_ptr : c->d_pflush_ptr,
			(const uint4 *)c->d_pblocks, c->d_pmeta, d_coef, xbuf, xbuf + p->dim, gacc, fix, (int)words,
			p->n_coef, 2 * p->dim, p->dim, d_active);
	}
	jn_int_finalize_batched_kernel<<<dim3(g, B), 256, 0, st>>>(gacc, y, y_ld, p->dim, ctrl, d_cmax, d_active);
	CUDA_TRY(cudaGetLastError());
	return JN_OK;
}

/* ------------------------------------------------------------------ */
/* batched 32-bit products over instances of several bases              */
/* ------------------------------------------------------------------ */
/* One instance of a several-bases panel product: its basis's panels, tasks
 * and CTA partition (on the basis's context), its coefficients, x buffers,
 * accumulator and coefficient scale (112 bytes). */
struct jn_panel_inst {
	const uint4 *panels, *tasks;
	const uint32_t *cta, *flush, *flush_ptr;
	const uint4 *blocks;
	const uint32_t *meta;
	const int *coef;
	int *xi;                        /* x as 32-bit fixed point, [p][n] then [n][p] (2 dim words) */
	unsigned long long *gacc;
	const unsigned long long *cmax; /* max|c| bits of the instance's coefficients */
	int64_t dim;
	int grid, words, nblocks;
	int owner;                      /* the first instance of a basis owns the basis's coefficient arrays */
};
static_assert(sizeof(jn_panel_inst) == 112, "one descriptor is 112 bytes");

struct jn_panel_batch {
	int B;
	jn_panel_inst *h, *d;
	unsigned int *d_ctrl;           /* max|x| bits of instance i at 2 i */
	int max_grid, max_blocks;
	size_t smem;
	jn_panel_partition *parts;      /* one per basis */
	int nbases;
};

/* instance blockIdx.y; CTAs beyond the instance's grid have no work */
__global__ void __launch_bounds__(PANEL_THREADS, 3)
	jn_panel_multi_kernel(const jn_panel_inst *__restrict__ I, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const jn_panel_inst d = I[inst];
	if ((int)blockIdx.x >= d.grid) return;
	const FixInt32 fix = {};
	jn_panel_body<int, FixInt32, false>(d.panels, d.tasks, d.cta, d.flush, d.flush_ptr, d.blocks, d.meta, d.coef, d.xi,
					    d.xi + d.dim, d.gacc, fix, d.words);
}

__global__ void jn_panel_multi_xmax_kernel(const jn_panel_inst *__restrict__ I, const double *__restrict__ src,
					   int64_t src_ld, const int *__restrict__ sel, int64_t sel_ld,
					   unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const int64_t n = I[inst].dim;
	const double *x = src + inst * src_ld + (sel ? (int64_t)(*sel) * sel_ld : 0);
	float m = 0.0f;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		m = fmaxf(m, (float)fabs(x[i]) * 1.0000002f);
	for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(ctrl + 2 * inst, __float_as_uint(m));
}

/* block blockIdx.x of instance blockIdx.y: x_i as 32-bit fixed point, [p][n] and transposed [n][p] */
__global__ void jn_panel_multi_x_kernel(const jn_panel_inst *__restrict__ I, const double *__restrict__ src,
					int64_t src_ld, const int *__restrict__ sel, int64_t sel_ld,
					const unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const jn_panel_inst d = I[inst];
	if ((int)blockIdx.x >= d.nblocks) return;
	const double *x = src + inst * src_ld + (sel ? (int64_t)(*sel) * sel_ld : 0);
	int *xn = d.xi, *xt = d.xi + d.dim;
	const uint4 bk = d.blocks[blockIdx.x];
	const uint32_t Np = bk.z, Nn = bk.w, n = Np * Nn;
	const double s = ldexp(1.0, x_exponent(ctrl[2 * inst]));
	for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
		const int t = __double2int_rn(x[bk.x + e] * s);
		xn[bk.x + e] = t;
		xt[bk.x + (e % Nn) * Np + e / Nn] = t;
	}
}

/* y_i = acc_i 2^(30 - Sc_i - Sx_i) (y + i y_ld); the accumulators are cleared */
__global__ void jn_panel_multi_finalize_kernel(const jn_panel_inst *__restrict__ I, double *__restrict__ y, int64_t y_ld,
					       const unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const jn_panel_inst d = I[inst];
	const double unit = ldexp(1.0, PANEL_INT_SHIFT - coef_exponent(*d.cmax) - x_exponent(ctrl[2 * inst]));
	double *yy = y + inst * y_ld;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.dim; i += (int64_t)gridDim.x * blockDim.x) {
		yy[i] = (double)(long long)d.gacc[i] * unit;
		d.gacc[i] = 0ull;
	}
}

void jn_panel_batch_free(jn_panel_batch *pb)
{
	if (!pb) return;
	if (pb->h)
		for (int i = 0; i < pb->B; i++) {
			if (pb->h[i].owner) {
				cudaFree((void *)pb->h[i].coef);
				cudaFree((void *)pb->h[i].cmax);
			}
			cudaFree(pb->h[i].xi);
			cudaFree(pb->h[i].gacc);
		}
	if (pb->parts)
		for (int b = 0; b < pb->nbases; b++) jn_panels_partition_free(&pb->parts[b]);
	free(pb->parts);
	free(pb->h);
	cudaFree(pb->d);
	cudaFree(pb->d_ctrl);
	free(pb);
}

int jn_panel_batch_possible(jn_ctx *const *ctxs, int nbases)
{
	for (int b = 0; b < nbases; b++)
		if (ctxs[b]->engine_of[1] != 4 || jn_panels_setup(ctxs[b]) != JN_OK || !jn_panels_fit(ctxs[b], 1)) {
			cudaGetLastError();
			return 0;
		}
	return 1;
}

jn_status jn_panel_batch_create(jn_ctx *const *ctxs, int nbases, const int *count, const double *const *d_me64,
				jn_panel_batch **out)
{
	*out = NULL;
	int B = 0;
	for (int b = 0; b < nbases; b++) B += count[b];
	if (B < 1 || B > 65535) return jn_fail(JN_ERR_INVALID, "batch of %d instances", B);
	jn_panel_batch *pb = (jn_panel_batch *)calloc(1, sizeof *pb);
	if (!pb) return jn_fail(JN_ERR_NOMEM, "out of host memory");
	pb->B = B;
	pb->nbases = nbases;
	pb->h = (jn_panel_inst *)calloc((size_t)B, sizeof(jn_panel_inst));
	pb->parts = (jn_panel_partition *)calloc((size_t)nbases, sizeof(jn_panel_partition));
	jn_status s = (!pb->h || !pb->parts) ? jn_fail(JN_ERR_NOMEM, "out of host memory") : JN_OK;
	/* CTAs: the resident CTAs of the 32-bit kernel shared out by each instance's coefficients */
	double work = 0.0;
	for (int b = 0; b < nbases && !s; b++) {
		if ((s = jn_panels_setup(ctxs[b]))) break;
		work += (double)count[b] * (double)(ctxs[b]->plan.n_coef ? ctxs[b]->plan.n_coef : 1);
	}
	const int resident = !s ? ctxs[0]->num_sms * ctxs[0]->panel_per_sm[1] : 0;
	for (int b = 0, i0 = 0; b < nbases && !s; i0 += count[b], b++) {
		jn_ctx *c = ctxs[b];
		const jn_plan_t *p = &c->plan;
		int g = (int)(resident * (double)(p->n_coef ? p->n_coef : 1) / work);
		if (g < 8) g = 8;
		if ((s = jn_panels_partition_upload(c, g, &pb->parts[b]))) break;
		const jn_panel_partition *pp = &pb->parts[b];
		int *coef = NULL;
		unsigned long long *cmax = NULL;
		const int64_t nc = p->n_coef ? p->n_coef : 1;
		if (cudaMalloc((void **)&coef, (size_t)count[b] * nc * sizeof(int)) != cudaSuccess ||
		    cudaMalloc((void **)&cmax, (size_t)count[b] * sizeof(unsigned long long)) != cudaSuccess) {
			cudaFree(coef);
			s = jn_fail(JN_ERR_NOMEM, "cudaMalloc of batched panel coefficients failed");
			break;
		}
		pb->h[i0].owner = 1;
		s = jn_panels_batched_coefficients(c, count[b], d_me64[b], p->n_me, coef, cmax, c->stream);
		for (int j = 0; j < count[b]; j++) {
			jn_panel_inst *d = &pb->h[i0 + j];
			d->coef = coef + (size_t)j * nc;
			d->cmax = cmax + j;
			d->panels = (const uint4 *)c->d_panels;
			d->tasks = (const uint4 *)c->d_ptasks;
			d->cta = pp->cta;
			d->flush = pp->flush;
			d->flush_ptr = pp->flush_ptr;
			d->blocks = (const uint4 *)c->d_pblocks;
			d->meta = c->d_pmeta;
			d->dim = p->dim;
			d->grid = pp->grid;
			d->words = pp->words;
			d->nblocks = p->nblocks;
		}
		if (s) break;
		for (int j = 0; j < count[b] && !s; j++) {
			jn_panel_inst *d = &pb->h[i0 + j];
			if (cudaMalloc((void **)&d->xi, (size_t)2 * (p->dim ? p->dim : 1) * sizeof(int)) != cudaSuccess ||
			    cudaMalloc((void **)&d->gacc, (size_t)(p->dim ? p->dim : 1) * sizeof(unsigned long long)) != cudaSuccess ||
			    cudaMemset(d->gacc, 0, (size_t)(p->dim ? p->dim : 1) * sizeof(unsigned long long)) != cudaSuccess)
				s = jn_fail(JN_ERR_NOMEM, "cudaMalloc of batched panel buffers failed");
		}
		const size_t sm = panel_smem_words(p, pp->words, 0);
		if (sm > pb->smem) pb->smem = sm;
		if (pp->grid > pb->max_grid) pb->max_grid = pp->grid;
		if (p->nblocks > pb->max_blocks) pb->max_blocks = p->nblocks;
	}
	if (!s && (cudaMalloc((void **)&pb->d, (size_t)B * sizeof(jn_panel_inst)) != cudaSuccess ||
		   cudaMalloc((void **)&pb->d_ctrl, (size_t)2 * B * sizeof(unsigned int)) != cudaSuccess))
		s = jn_fail(JN_ERR_NOMEM, "cudaMalloc of the batch descriptors failed");
	if (!s && cudaMemcpy(pb->d, pb->h, (size_t)B * sizeof(jn_panel_inst), cudaMemcpyHostToDevice) != cudaSuccess)
		s = jn_fail(JN_ERR_CUDA, "upload of the batch descriptors failed");
	if (!s) {
		cudaError_t e = cudaFuncSetAttribute(jn_panel_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pb->smem);
		if (e == cudaSuccess) e = cudaDeviceSynchronize();
		if (e != cudaSuccess) s = jn_fail(JN_ERR_CUDA, "batched panel set-up: %s", cudaGetErrorString(e));
	}
	if (s) {
		jn_panel_batch_free(pb);
		return s;
	}
	*out = pb;
	return JN_OK;
}

jn_status jn_panel_batch_enqueue(jn_panel_batch *pb, const double *src, int64_t src_ld, const int *d_sel, int64_t sel_ld,
				 double *y, int64_t y_ld, const int *d_active, int64_t max_dim, cudaStream_t st)
{
	const int B = pb->B;
	int g = (int)((max_dim + 255) / 256);
	if (g > 256) g = 256;
	if (g < 1) g = 1;
	CUDA_TRY(cudaMemsetAsync(pb->d_ctrl, 0, (size_t)2 * B * sizeof(unsigned int), st));
	jn_panel_multi_xmax_kernel<<<dim3(g, B), 256, 0, st>>>(pb->d, src, src_ld, d_sel, sel_ld, pb->d_ctrl, d_active);
	jn_panel_multi_x_kernel<<<dim3(pb->max_blocks > 0 ? pb->max_blocks : 1, B), 256, 0, st>>>(pb->d, src, src_ld, d_sel,
												      sel_ld, pb->d_ctrl, d_active);
	jn_panel_multi_kernel<<<dim3(pb->max_grid, B), PANEL_THREADS, pb->smem, st>>>(pb->d, d_active);
	jn_panel_multi_finalize_kernel<<<dim3(g, B), 256, 0, st>>>(pb->d, y, y_ld, pb->d_ctrl, d_active);
	CUDA_TRY(cudaGetLastError());
	return JN_OK;
}
