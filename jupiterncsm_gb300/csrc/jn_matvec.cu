/*
 * jn_matvec.cu — sm_103a kernels for the index-list block matrix-vector
 * product and the C ABI around them (include/jncsm.h).
 *
 * Semantics are the reference Minerva kernels'
 * (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c):
 *   neutron list  y[n_o + Nn p] += s M[k] x[n_i + Nn p]       (:20-77)
 *   proton list   y[Nn p_o + n] += s M[k] x[Nn p_i + n]       (:79-132)
 *   n x p lists   y[n_o + Nn_o p_o] += s_n s_p M[k_n + Nd k_p] x[n_i + Nn_i p_i]   (:134-210)
 *   off-diagonal instructions also apply the transpose into the input block
 *   (:212-462); single-species terms skip |M| < 1e-12 (:52-53, 107-108).
 *
 * GB300 organisation (see jn_problem.h): the host plan turns every
 * instruction into terms owned by their destination block; destination
 * blocks are cut into tiles of at most 512 elements; the terms of a tile are
 * cut into chunks of similar work.  One CTA computes one (tile, chunk):
 * every output element is owned by one thread (or a fixed group of threads
 * reduced in fixed order through shared memory), which walks the CSR rows
 * of the lists in list order.  Partial sums land in a scratch array and the
 * reduction pass adds them in chunk order, so no atomics are used and the
 * result is bit-identical from run to run.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "jn_internal.h"
#include "jn_fixed.cuh"

#define JN_VERSION "jncsm-gb300 0.1"

static thread_local char g_last_error[1024];

extern "C" jn_status jn_fail(jn_status s, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
	va_end(ap);
	return s;
}
#define fail jn_fail

extern "C" const char *jn_last_error(void) { return g_last_error; }
extern "C" const char *jn_version(void) { return JN_VERSION; }

/* ------------------------------------------------------------------ */
/* kernels                                                             */
/* ------------------------------------------------------------------ */
#define MASK31 0x7fffffffu

struct DevPlan {
	const uint32_t *__restrict__ rowptr;
	const uint2 *__restrict__ ent;
	const double *__restrict__ me;
	const jn_term_t *__restrict__ terms;
	const jn_tile_t *__restrict__ tiles;
	const jn_unit_t *__restrict__ units;
	const int32_t *__restrict__ unit_terms;
};

#define WARPS 8
#define TINY_BITS 0x3D719799812DEA11ull   /* bit pattern of 1e-12 */
#define TINY_BITS32 0x2B8CBCCCu          /* bit pattern of 1e-12f */

__device__ __forceinline__ double flip_sign(double m, uint32_t sbit)
{
	return __longlong_as_double(__double_as_longlong(m) ^ ((unsigned long long)(sbit & 0x80000000u) << 32));
}
__device__ __forceinline__ float flip_sign(float m, uint32_t sbit)
{
	return __uint_as_float(__float_as_uint(m) ^ (sbit & 0x80000000u));
}
/* |m| < 1e-12, decided on the bit pattern (no floating-point instruction) */
__device__ __forceinline__ bool tiny(double m)
{
	return ((unsigned long long)__double_as_longlong(m) & 0x7fffffffffffffffull) < TINY_BITS;
}
__device__ __forceinline__ bool tiny(float m) { return false; /* pre-zeroed on upload */ }

/*
 * Contribution of term t to element (p, n) of its destination block, summed
 * into acc in list order.  One floating-point instruction per multiply-add:
 * signs are applied with integer XORs and the reference's |M| < 1e-12 skip
 * of single-species terms is a bit-pattern compare.
 */
template <typename T>
__device__ __forceinline__ T term_element(const DevPlan &P, const jn_term_t &t, const T *__restrict__ x,
					  const T *__restrict__ me_all, int p, int n)
{
	const T *__restrict__ xs = x + t.src_off;
	const T *__restrict__ me = me_all + t.me_off;
	const uint32_t *__restrict__ rp = P.rowptr;
	T acc = 0;
	if (t.kind == JN_KIND_P) {
		const uint32_t j0 = __ldg(rp + t.p_ptr + p), j1 = __ldg(rp + t.p_ptr + p + 1);
		for (uint32_t j = j0; j < j1; j++) {
			const uint2 e = __ldg(P.ent + j);
			T m = __ldg(me + (e.y & MASK31));
			if (tiny(m)) continue;
			const uint32_t src = e.x & 0xffffu;
			acc = fma(flip_sign(m, e.y), __ldg(xs + (size_t)src * t.Nn_src + n), acc);
		}
	} else if (t.kind == JN_KIND_N) {
		const uint32_t j0 = __ldg(rp + t.n_ptr + n), j1 = __ldg(rp + t.n_ptr + n + 1);
		const T *__restrict__ xrow = xs + (size_t)p * t.Nn_src;
		for (uint32_t j = j0; j < j1; j++) {
			const uint2 e = __ldg(P.ent + j);
			T m = __ldg(me + (e.y & MASK31));
			if (tiny(m)) continue;
			const uint32_t src = e.x & 0xffffu;
			acc = fma(flip_sign(m, e.y), __ldg(xrow + src), acc);
		}
	} else {
		const uint32_t j0 = __ldg(rp + t.n_ptr + n), j1 = __ldg(rp + t.n_ptr + n + 1);
		if (j0 == j1) return acc;
		const uint32_t i0 = __ldg(rp + t.p_ptr + p), i1 = __ldg(rp + t.p_ptr + p + 1);
		for (uint32_t i = i0; i < i1; i++) {
			const uint2 ep = __ldg(P.ent + i);
			const T *__restrict__ mrow = me + (size_t)t.nd * (ep.y & MASK31);
			const uint32_t psrc = ep.x & 0xffffu;
			const T *__restrict__ xrow = xs + (size_t)psrc * t.Nn_src;
			for (uint32_t j = j0; j < j1; j++) {
				const uint2 en = __ldg(P.ent + j);
				const T m = __ldg(mrow + (en.y & MASK31));
				const uint32_t nsrc = en.x & 0xffffu;
				acc = fma(flip_sign(m, ep.y ^ en.y), __ldg(xrow + nsrc), acc);
			}
		}
	}
	return acc;
}

/*
 * One warp per work unit.  A unit is a piece of a destination block (R rows
 * x W columns, R*W <= 32, one element per lane) and a chunk of the terms that
 * touch it.  FP64: the lane accumulates every multiply-add in FP64.  FP32:
 * matrix elements and x in FP32, each term's sum in FP32, terms combined by
 * error-free TwoSum into an FP32 sum and FP32 compensation.
 */
template <bool F32>
__global__ void __launch_bounds__(WARPS * 32) jn_pieces_kernel(DevPlan P, const void *__restrict__ xv,
							       const void *__restrict__ mev,
							       double *__restrict__ partial, int nunits)
{
	const int lane = threadIdx.x & 31;
	const int ui = blockIdx.x * WARPS + (threadIdx.x >> 5);
	if (ui >= nunits) return;
	const jn_unit_t u = P.units[ui];
	const jn_tile_t tile = P.tiles[u.tile];
	const int E = tile.nrows * tile.ncols;
	if (lane >= E) return;
	const int p = tile.row0 + lane / tile.ncols, n = tile.col0 + lane % tile.ncols;
	double result;
	if (!F32) {
		const double *x = (const double *)xv, *me = (const double *)mev;
		double acc = 0.0;
		for (int64_t q = u.t0; q < u.t1; q++) {
			const jn_term_t t = P.terms[__ldg(P.unit_terms + q)];
			acc += term_element<double>(P, t, x, me, p, n);
		}
		result = acc;
	} else {
		const float *x = (const float *)xv, *me = (const float *)mev;
		float s = 0.0f, c = 0.0f;
		for (int64_t q = u.t0; q < u.t1; q++) {
			const jn_term_t t = P.terms[__ldg(P.unit_terms + q)];
			const float v = term_element<float>(P, t, x, me, p, n);
			const float s2 = s + v, bp = s2 - s;
			c += (s - (s2 - bp)) + (v - bp);
			s = s2;
		}
		result = (double)s + (double)c;
	}
	partial[tile.partial + (int64_t)u.chunk * E + lane] = result;
}

/* y (+)= sum of the unit partials of each piece, in chunk order; one warp per piece */
__global__ void __launch_bounds__(WARPS * 32) jn_reduce_kernel(const jn_tile_t *__restrict__ tiles, int ntiles,
							       const double *__restrict__ partial,
							       double *__restrict__ y, int accumulate)
{
	const int lane = threadIdx.x & 31;
	const int ti = blockIdx.x * WARPS + (threadIdx.x >> 5);
	if (ti >= ntiles) return;
	const jn_tile_t t = tiles[ti];
	const int E = t.nrows * t.ncols;
	if (lane >= E) return;
	double s = 0.0;
	for (int c = 0; c < t.nchunks; c++) s += partial[t.partial + (int64_t)c * E + lane];
	const int64_t at = t.dst_off + (int64_t)(t.row0 + lane / t.ncols) * t.Nn + t.col0 + lane % t.ncols;
	y[at] = accumulate ? y[at] + s : s;
}

__global__ void jn_to_f32_kernel(const double *__restrict__ x, float *__restrict__ y, int64_t n)
{
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		y[i] = (float)x[i];
}

/* ------------------------------------------------------------------ */
/* block-tile kernels: exact 64-bit fixed-point accumulation           */
/* ------------------------------------------------------------------ */
#define TILE_THREADS 256

/* x (FP64) -> optional FP32 copy, and max|x| into *xmax_bits (zeroed before) */
__global__ void jn_prep_kernel(const double *__restrict__ x, float *__restrict__ x32, int64_t n,
			       unsigned int *__restrict__ xmax_bits)
{
	float m = 0.0f;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = x[i];
		if (x32) x32[i] = (float)v;
		m = fmaxf(m, (float)fabs(v) * 1.0000002f);  /* round-up margin of the FP32 conversion */
	}
	for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(xmax_bits, __float_as_uint(m));
}

__device__ __forceinline__ int pow2_at_least(int v)
{
	int b = 1;
	while (b < v) b <<= 1;
	return b;
}

/*
 * One CTA per block tile (rows [row0, row0+nrows) of one destination block).
 * Each warp takes pieces in turn and spreads a piece over its lanes as an
 * (a x b) grid: b lanes over the neutron entries (or columns), a lanes over
 * contiguous sub-ranges of the proton entries (or rows).  A lane sums the run
 * of consecutive proton entries that share a destination row in T
 * arithmetic, scales by 2^S, rounds to a 64-bit integer and adds it into the
 * tile's shared-memory accumulator; the tile is then added into the global
 * 64-bit accumulator.  Integer addition is exact and associative, so the
 * result does not depend on the order in which warps and CTAs run.
 */
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS) jn_tile_kernel(DevPlan P, const jn_btile_t *__restrict__ tiles, int ntiles,
							       unsigned int *__restrict__ tile_counter,
							       const uint2 *__restrict__ items,
							       const jn_piece_t *__restrict__ tasks,
							       const jn_tterm_t *__restrict__ tterms,
							       const uint2 *__restrict__ walks,
							       const T *__restrict__ x, const T *__restrict__ me,
							       unsigned long long *__restrict__ gacc,
							       const unsigned int *__restrict__ xmax_bits, double abs_bound,
							       int64_t inst_stride, int64_t me_stride,
							       const int *__restrict__ active)
{
	extern __shared__ unsigned int sacc[];
	__shared__ int next_item, cur_tile;
	/* batched products: instance blockIdx.y owns x, me and gacc at its strides
	   and the control words (max|x| bits, tile counter) at 2 * instance */
	if (gridDim.y > 1 || active) {
		const int inst = blockIdx.y;
		if (active && !active[inst]) return;
		x += inst * inst_stride;
		me += inst * me_stride;
		gacc += inst * inst_stride;
		tile_counter += 2 * inst;
		xmax_bits += 2 * inst;
	}
	const int S = fixed_exponent(*xmax_bits, abs_bound);
	const T scale = (T)ldexp(1.0, S);
	const int lane = threadIdx.x & 31;
	const uint4 *__restrict__ tq4 = (const uint4 *)tasks;
	const uint4 *__restrict__ tt4 = (const uint4 *)tterms;
	const uint2 *__restrict__ ent = P.ent;
	for (;;) {
		/* persistent CTAs take tiles heaviest first */
		if (threadIdx.x == 0) {
			cur_tile = (int)atomicAdd(tile_counter, 1u);
			next_item = 0;
		}
		__syncthreads();
		const int ti = cur_tile;
		if (ti >= ntiles) break;
		const jn_btile_t tl = tiles[ti];
		const int Nn = tl.Nn, stride = tl.stride;
		const int Ep = tl.nrows * stride;
		unsigned int *lo = sacc, *hi = sacc + Ep;
		for (int i = threadIdx.x; i < 2 * Ep; i += blockDim.x) sacc[i] = 0u;
		__syncthreads();
		const int nitem = (int)(tl.pc1 - tl.pc0);
		const int rbase = -tl.row0 * stride;
		for (;;) {
			int k = 0;
			if (lane == 0) k = atomicAdd(&next_item, 1);
			k = __shfl_sync(0xffffffffu, k, 0);
			if (k >= nitem) break;
			const uint2 it = __ldg(items + tl.pc0 + k);
			const uint32_t w = it.y & 0xffu, nsub = it.y >> 8;
			const uint32_t sub = (uint32_t)lane / w, sl = (uint32_t)lane & (w - 1u);
			if (sub >= nsub) continue;
			const uint4 tq = __ldg(tq4 + it.x + sub);
			const uint32_t kind = JN_TASK_KIND(tq.x), count = JN_TASK_COUNT(tq.x), term = JN_TASK_TERM(tq.x);
			if (sl >= count) continue;
			const uint4 ta = __ldg(tt4 + 2 * term), tb = __ldg(tt4 + 2 * term + 1);
			const T *__restrict__ mb = me + ((int64_t)ta.x | ((int64_t)ta.y << 32));
			const T *__restrict__ xs = x + (int)ta.z;
			const int nd = (int)ta.w, Ns = (int)tb.x;
			const uint32_t lb = tq.y + sl, l0 = tq.z, nl = tq.w;
		if (kind == JN_TASK_NP_A) {
			const uint2 nw = __ldg(walks + lb);
			const uint32_t n0 = nw.x, n1 = nw.x + (nw.y & 0xffffu);
			const int dcol = (int)(nw.y >> 16);
			for (uint32_t q = 0; q < nl; q++) {
				const uint2 pw = __ldg(walks + l0 + q);
				const uint32_t p0 = pw.x, p1 = pw.x + (pw.y & 0xffffu);
				const int drow = (int)(pw.y >> 16);
				T run = 0;
				for (uint32_t j = n0; j < n1; j++) {
					const uint2 qn = __ldg(ent + j);
					const int scol = (int)(qn.x & 0xffffu);
					const T *__restrict__ mcol = mb + (qn.y & MASK31);
					for (uint32_t i = p0; i < p1; i++) {
						const uint2 qp = __ldg(ent + i);
						const int srow = (int)(qp.x & 0xffffu);
						const T m = __ldg(mcol + nd * (qp.y & MASK31));
						run = fma(flip_sign(m, qp.y ^ qn.y), __ldg(xs + srow * Ns + scol), run);
					}
				}
				add_fixed(lo, hi, rbase + drow * stride + dcol, to_fixed<T>(run * scale));
			}
		} else if (kind == JN_TASK_NP_B) {
			const uint2 pw = __ldg(walks + lb);
			const uint32_t p0 = pw.x, p1 = pw.x + (pw.y & 0xffffu);
			const int drow = (int)(pw.y >> 16);
			for (uint32_t q = 0; q < nl; q++) {
				const uint2 nw = __ldg(walks + l0 + q);
				const uint32_t n0 = nw.x, n1 = nw.x + (nw.y & 0xffffu);
				const int dcol = (int)(nw.y >> 16);
				T run = 0;
				for (uint32_t i = p0; i < p1; i++) {
					const uint2 qp = __ldg(ent + i);
					const int srow = (int)(qp.x & 0xffffu);
					const T *__restrict__ mrow = mb + nd * (qp.y & MASK31);
					const T *__restrict__ xrow = xs + srow * Ns;
					for (uint32_t j = n0; j < n1; j++) {
						const uint2 qn = __ldg(ent + j);
						const int scol = (int)(qn.x & 0xffffu);
						const T m = __ldg(mrow + (qn.y & MASK31));
						run = fma(flip_sign(m, qp.y ^ qn.y), __ldg(xrow + scol), run);
					}
				}
				add_fixed(lo, hi, rbase + drow * stride + dcol, to_fixed<T>(run * scale));
			}
		} else if (kind == JN_TASK_P_A) {
			const int c = (int)lb;
			for (uint32_t q = 0; q < nl; q++) {
				const uint2 pw = __ldg(walks + l0 + q);
				const uint32_t p0 = pw.x, p1 = pw.x + (pw.y & 0xffffu);
				const int drow = (int)(pw.y >> 16);
				T run = 0;
				for (uint32_t i = p0; i < p1; i++) {
					const uint2 qp = __ldg(ent + i);
					const int srow = (int)(qp.x & 0xffffu);
					const T m = __ldg(mb + (qp.y & MASK31));
					if (tiny(m)) continue;
					run = fma(flip_sign(m, qp.y), __ldg(xs + srow * Ns + c), run);
				}
				add_fixed(lo, hi, rbase + drow * stride + c, to_fixed<T>(run * scale));
			}
		} else if (kind == JN_TASK_P_B) {
			const uint2 pw = __ldg(walks + lb);
			const uint32_t p0 = pw.x, p1 = pw.x + (pw.y & 0xffffu);
			const int drow = (int)(pw.y >> 16);
			for (uint32_t q = 0; q < nl; q++) {
				const int c = (int)(l0 + q);
				T run = 0;
				for (uint32_t i = p0; i < p1; i++) {
					const uint2 qp = __ldg(ent + i);
					const int srow = (int)(qp.x & 0xffffu);
					const T m = __ldg(mb + (qp.y & MASK31));
					if (tiny(m)) continue;
					run = fma(flip_sign(m, qp.y), __ldg(xs + srow * Ns + c), run);
				}
				add_fixed(lo, hi, rbase + drow * stride + c, to_fixed<T>(run * scale));
			}
		} else if (kind == JN_TASK_N_A) {
			const uint2 nw = __ldg(walks + lb);
			const uint32_t n0 = nw.x, n1 = nw.x + (nw.y & 0xffffu);
			const int dcol = (int)(nw.y >> 16);
			for (uint32_t q = 0; q < nl; q++) {
				const int r = (int)(l0 + q);
				const T *__restrict__ xrow = xs + r * Ns;
				T run = 0;
				for (uint32_t j = n0; j < n1; j++) {
					const uint2 qn = __ldg(ent + j);
					const int scol = (int)(qn.x & 0xffffu);
					const T m = __ldg(mb + (qn.y & MASK31));
					if (tiny(m)) continue;
					run = fma(flip_sign(m, qn.y), __ldg(xrow + scol), run);
				}
				add_fixed(lo, hi, rbase + r * stride + dcol, to_fixed<T>(run * scale));
			}
		} else {
			const int r = (int)lb;
			const T *__restrict__ xrow = xs + r * Ns;
			for (uint32_t q = 0; q < nl; q++) {
				const uint2 nw = __ldg(walks + l0 + q);
				const uint32_t n0 = nw.x, n1 = nw.x + (nw.y & 0xffffu);
				const int dcol = (int)(nw.y >> 16);
				T run = 0;
				for (uint32_t j = n0; j < n1; j++) {
					const uint2 qn = __ldg(ent + j);
					const int scol = (int)(qn.x & 0xffffu);
					const T m = __ldg(mb + (qn.y & MASK31));
					if (tiny(m)) continue;
					run = fma(flip_sign(m, qn.y), __ldg(xrow + scol), run);
				}
				add_fixed(lo, hi, rbase + r * stride + dcol, to_fixed<T>(run * scale));
			}
		}
		}
		__syncthreads();
		unsigned long long *g = gacc + tl.dst_off + (int64_t)tl.row0 * Nn;
		const int E = tl.nrows * Nn;
		for (int i = threadIdx.x; i < E; i += blockDim.x) {
			const int si = (i / Nn) * stride + i % Nn;
			const unsigned long long v = (unsigned long long)lo[si] | ((unsigned long long)hi[si] << 32);
			if (v) atomicAdd(g + i, v);
		}
		__syncthreads();
	}
}

/* y (+)= acc * 2^-S, and the accumulator is cleared for the next product */
__global__ void jn_finalize_kernel(unsigned long long *__restrict__ gacc, double *__restrict__ y, int64_t n,
				   const unsigned int *__restrict__ xmax_bits, double abs_bound, int accumulate)
{
	const int S = fixed_exponent(*xmax_bits, abs_bound);
	const double unit = ldexp(1.0, -S);
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = (double)(long long)gacc[i] * unit;
		y[i] = accumulate ? y[i] + v : v;
		gacc[i] = 0ull;
	}
}

void jn_launch_prep(const double *d_x, float *x32, int64_t n, unsigned int *ctrl, cudaStream_t st)
{
	int g = (int)((n + 255) / 256);
	if (g > 1024) g = 1024;
	if (n > 0) jn_prep_kernel<<<g, 256, 0, st>>>(d_x, x32, n, ctrl);
}

void jn_launch_finalize(unsigned long long *gacc, double *d_y, int64_t n, const unsigned int *ctrl, double abs_bound,
			int accumulate, cudaStream_t st)
{
	int g = (int)((n + 255) / 256);
	if (g > 1024) g = 1024;
	if (n > 0) jn_finalize_kernel<<<g, 256, 0, st>>>(gacc, d_y, n, ctrl, abs_bound, accumulate);
}

/* Batched products (instance = blockIdx.y).  The source vector of instance
 * i is src + i * src_ld + (*sel) * sel_ld: the Lanczos vector v_k of a batched
 * solve, with k read on the device so that a captured graph can be replayed
 * at every step.  It is copied to x64 (FP64 products) or converted to x32
 * (FP32 products); max|x| goes to ctrl[2 i]. */
__global__ void jn_prep_batched_kernel(const double *__restrict__ src, int64_t src_ld, const int *__restrict__ sel,
				       int64_t sel_ld, double *__restrict__ x64, float *__restrict__ x32, int64_t n,
				       unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const double *x = src + inst * src_ld + (sel ? (int64_t)(*sel) * sel_ld : 0);
	float m = 0.0f;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = x[i];
		if (x32) x32[inst * n + i] = (float)v;
		else x64[inst * n + i] = v;
		m = fmaxf(m, (float)fabs(v) * 1.0000002f);
	}
	for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(ctrl + 2 * inst, __float_as_uint(m));
}

__global__ void jn_finalize_batched_kernel(unsigned long long *__restrict__ gacc, double *__restrict__ y,
					   int64_t y_ld, int64_t n, const unsigned int *__restrict__ ctrl, double abs_bound,
					   const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const int S = fixed_exponent(ctrl[2 * inst], abs_bound);
	const double unit = ldexp(1.0, -S);
	unsigned long long *g = gacc + inst * n;
	double *yy = y + inst * y_ld;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		yy[i] = (double)(long long)g[i] * unit;
		g[i] = 0ull;
	}
}

/* ------------------------------------------------------------------ */
/* host side                                                           */
/* ------------------------------------------------------------------ */
template <typename T>
static jn_status upload(T **dst, const void *src, size_t n)
{
	size_t bytes = (n ? n : 1) * sizeof(T);
	cudaError_t e = cudaMalloc((void **)dst, bytes);
	if (e != cudaSuccess) return fail(JN_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
	if (n && src) {
		e = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
		if (e != cudaSuccess) return fail(JN_ERR_CUDA, "cudaMemcpy failed: %s", cudaGetErrorString(e));
	}
	return JN_OK;
}

extern "C" void jn_close(jn_ctx *c)
{
	if (!c) return;
	cudaFree(c->d_rowptr); cudaFree(c->d_ent); cudaFree(c->d_me); cudaFree(c->d_terms);
	cudaFree(c->d_tiles); cudaFree(c->d_units); cudaFree(c->d_unit_terms); cudaFree(c->d_partial);
	cudaFree(c->d_x); cudaFree(c->d_y); cudaFree(c->d_me32); cudaFree(c->d_x32);
	cudaFree(c->d_btiles); cudaFree(c->d_pieces); cudaFree(c->d_gacc); cudaFree(c->d_xmax); cudaFree(c->d_tterms); cudaFree(c->d_walks); cudaFree(c->d_items);
	if (c->h_pinned) cudaFreeHost(c->h_pinned);
	jn_product_graphs_clear(c);
	for (int i = 0; i < 4; i++)
		if (c->prof_ev[i]) cudaEventDestroy(c->prof_ev[i]);
	jn_panels_release(c);
	jn_walk_release(c);
	jn_lanczos_release(c);
	if (c->stream) cudaStreamDestroy(c->stream);
	jn_plan_free(&c->plan);
	free(c);
}

extern "C" jn_status jn_open_files(const char *comb, const char *order, const char *lists_dir, const char *me_dir,
				   int Z, int N, jn_ctx **out)
{
	if (!comb || !order || !lists_dir || !me_dir || !out) return fail(JN_ERR_INVALID, "null argument");
	*out = NULL;
	int ndev = 0;
	cudaError_t ce = cudaGetDeviceCount(&ndev);
	if (ce != cudaSuccess || ndev == 0)
		return fail(JN_ERR_CUDA, "no usable CUDA device (%s)", ce == cudaSuccess ? "0 devices" : cudaGetErrorString(ce));
	jn_ctx *c = (jn_ctx *)calloc(1, sizeof *c);
	char err[1024] = { 0 };
	int sms = 0;
	CUDA_TRY(cudaGetDevice(&c->device));
	CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
	c->num_sms = sms;
	c->precision = 64;
	if (jn_plan_build(&c->plan, comb, order, lists_dir, me_dir, Z, N, sms * 48, err, sizeof err)) {
		free(c);
		int io = strstr(err, "open") != NULL;
		return fail(io ? JN_ERR_IO : JN_ERR_FORMAT, "%s", err);
	}
	jn_plan_t *p = &c->plan;
	jn_status s;
	if ((s = upload(&c->d_rowptr, p->rowptr, p->n_rowptr)) ||
	    (s = upload(&c->d_ent, p->ent, p->n_ent)) ||
	    (s = upload(&c->d_me, p->me, p->n_me)) ||
	    (s = upload(&c->d_terms, p->terms, p->nterms)) ||
	    (s = upload(&c->d_x, (const void *)NULL, p->dim)) ||
	    (s = upload(&c->d_y, (const void *)NULL, p->dim)) ||
	    (s = upload(&c->d_btiles, p->btiles, p->nbtiles)) ||
	    (s = upload(&c->d_pieces, p->pieces, p->npieces)) ||
	    (s = upload(&c->d_tterms, p->tterms, p->nterms)) ||
	    (s = upload(&c->d_walks, p->walks, p->nwalks)) ||
	    (s = upload(&c->d_gacc, (const void *)NULL, p->dim)) ||
	    (s = upload(&c->d_items, p->items, 2 * p->nitems)) ||
	    (s = upload(&c->d_xmax, (const void *)NULL, 2))) {
		jn_close(c);
		return s;
	}
	{
		cudaError_t z = cudaMemset(c->d_gacc, 0, (p->dim ? p->dim : 1) * sizeof(unsigned long long));
		size_t smem = (size_t)(p->max_tile_elems ? p->max_tile_elems : 1) * 2 * sizeof(unsigned int);
		if (z == cudaSuccess)
			z = cudaFuncSetAttribute(jn_tile_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (z == cudaSuccess)
			z = cudaFuncSetAttribute(jn_tile_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		int per_sm_f = 1, per_sm_d = 1;
		if (z == cudaSuccess)
			z = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_f, jn_tile_kernel<float>, TILE_THREADS, smem);
		if (z == cudaSuccess)
			z = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_d, jn_tile_kernel<double>, TILE_THREADS, smem);
		if (z != cudaSuccess) { jn_close(c); return fail(JN_ERR_CUDA, "tile kernel set-up: %s", cudaGetErrorString(z)); }
		int per_sm = per_sm_f < per_sm_d ? per_sm_f : per_sm_d;
		if (per_sm < 1) per_sm = 1;
		c->tile_grid = c->num_sms * per_sm;
		if (c->tile_grid > p->nbtiles) c->tile_grid = p->nbtiles > 0 ? p->nbtiles : 1;
	}
	/* 32-bit products: the panel engine where the whole accumulator fits in
	   shared memory, else the walk engine; FP64-grade products: the walk
	   engine's exact integers (its plan is built on the first product) */
	c->engine_of[0] = c->engine_of[1] = 5;
	if (p->dim <= JN_PANEL_MAX_DIM) {
		if (jn_panels_setup(c) == JN_OK) c->engine_of[1] = 4;
		else jn_panels_release(c);
	}
	c->engine = c->engine_of[c->precision == 32];
	cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
	if (e != cudaSuccess) { jn_close(c); return fail(JN_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
	e = cudaMallocHost((void **)&c->h_pinned, (p->dim ? p->dim : 1) * sizeof(double));
	if (e != cudaSuccess) { jn_close(c); return fail(JN_ERR_NOMEM, "cudaMallocHost: %s", cudaGetErrorString(e)); }
	*out = c;
	return JN_OK;
}

extern "C" jn_status jn_open(const char *conf, jn_ctx **out)
{
	jn_runfile_t rf;
	char err[1024] = { 0 };
	if (!conf || !out) return fail(JN_ERR_INVALID, "null argument");
	if (jn_read_runfile(conf, &rf, err, sizeof err)) return fail(JN_ERR_FORMAT, "%s", err);
	return jn_open_files(rf.comb, rf.order, rf.lists, rf.mes, rf.Z, rf.N, out);
}

extern "C" size_t jn_dimension(const jn_ctx *c) { return c ? (size_t)c->plan.dim : 0; }
extern "C" int jn_num_blocks(const jn_ctx *c) { return c ? c->plan.nblocks : 0; }

extern "C" jn_status jn_block_info(const jn_ctx *c, int b, int *id, size_t *offset, size_t *length)
{
	if (!c || b < 0 || b >= c->plan.nblocks) return fail(JN_ERR_INVALID, "block index out of range");
	const jn_block_t *B = &c->plan.blocks[b];
	if (id) *id = B->id;
	if (offset) *offset = (size_t)B->offset;
	if (length) *length = (size_t)(B->Np * B->Nn);
	return JN_OK;
}

static jn_status ensure_f32(jn_ctx *c)
{
	const jn_plan_t *p = &c->plan;
	if (c->d_me32) return JN_OK;
	float *h = (float *)malloc((p->n_me ? p->n_me : 1) * sizeof(float));
	if (!h) return fail(JN_ERR_NOMEM, "out of host memory");
	for (int b = 0; b < p->nmes; b++) {
		const jn_me_t *M = &p->mes[b];
		for (int64_t e = 0; e < M->len; e++) {
			double v = p->me[M->offset + e];
			/* single-species terms skip |M| < 1e-12 (matrix_vector_multiplication.c:52-53) */
			h[M->offset + e] = (M->single && fabs(v) < 1e-12) ? 0.0f : (float)v;
		}
	}
	jn_status s = upload(&c->d_me32, h, p->n_me);
	free(h);
	if (s) return s;
	return upload(&c->d_x32, (const void *)NULL, p->dim);
}

/* enqueue the two kernels of one product; `mid` (optional) is recorded between them */
/* The block-tile product with caller-chosen scratch: gacc (dim 64-bit
 * words, zero on entry unless clear_acc), ctrl (2 words: max|x| bits and
 * the tile counter), x32 (dim floats, FP32 precision only).  Enqueues only;
 * never allocates. */
jn_status jn_enqueue_tiles(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st,
			   cudaEvent_t pre, cudaEvent_t mid, unsigned long long *gacc, unsigned int *ctrl, float *x32,
			   int clear_acc)
{
	const jn_plan_t *p = &c->plan;
	if (p->btiles_off) return fail(JN_ERR_INVALID, "no block-tile engine: %s", p->btiles_why);
	DevPlan P = { c->d_rowptr, c->d_ent, c->d_me, c->d_terms, c->d_tiles, c->d_units, c->d_unit_terms };
	const int f32 = c->precision == 32;
	if (f32 && !c->d_me32) return fail(JN_ERR_INVALID, "FP32 matrix elements are not set up");
	int g = (int)((p->dim + 255) / 256);
	if (g > 1024) g = 1024;
	if (g < 1) g = 1;
	const size_t smem = (size_t)(p->max_tile_elems ? p->max_tile_elems : 1) * 2 * sizeof(unsigned int);
	cudaError_t e0 = cudaMemsetAsync(ctrl, 0, 2 * sizeof(unsigned int), st);
	if (e0 == cudaSuccess && clear_acc && p->dim)
		e0 = cudaMemsetAsync(gacc, 0, (size_t)p->dim * sizeof(unsigned long long), st);
	if (e0 != cudaSuccess) return fail(JN_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e0));
	if (p->dim) jn_prep_kernel<<<g, 256, 0, st>>>(d_x, f32 ? x32 : NULL, p->dim, ctrl);
	if (pre) cudaEventRecord(pre, st);
	if (p->nbtiles) {
		if (f32)
			jn_tile_kernel<float><<<c->tile_grid, TILE_THREADS, smem, st>>>(
				P, c->d_btiles, p->nbtiles, ctrl + 1, (const uint2 *)c->d_items, c->d_pieces, c->d_tterms,
				c->d_walks, x32, c->d_me32, gacc, ctrl, p->abs_bound, 0, 0, NULL);
		else
			jn_tile_kernel<double><<<c->tile_grid, TILE_THREADS, smem, st>>>(
				P, c->d_btiles, p->nbtiles, ctrl + 1, (const uint2 *)c->d_items, c->d_pieces, c->d_tterms,
				c->d_walks, d_x, c->d_me, gacc, ctrl, p->abs_bound, 0, 0, NULL);
	}
	if (mid) cudaEventRecord(mid, st);
	if (p->dim) jn_finalize_kernel<<<g, 256, 0, st>>>(gacc, d_y, p->dim, ctrl, p->abs_bound, accumulate);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return fail(JN_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
	return JN_OK;
}

jn_status jn_enqueue_batched(jn_ctx *c, int B, int f32, const void *me, int64_t me_ld, const double *src,
			     int64_t src_ld, const int *d_sel, int64_t sel_ld, double *y, int64_t y_ld, double *x64,
			     float *x32, unsigned long long *gacc, unsigned int *ctrl, const int *d_active, double abs_bound,
			     cudaStream_t st)
{
	const jn_plan_t *p = &c->plan;
	if (B < 1 || B > 65535) return fail(JN_ERR_INVALID, "batch of %d instances", B);
	if (p->btiles_off) return fail(JN_ERR_INVALID, "no block-tile engine: %s", p->btiles_why);
	DevPlan P = { c->d_rowptr, c->d_ent, c->d_me, c->d_terms, c->d_tiles, c->d_units, c->d_unit_terms };
	int g = (int)((p->dim + 255) / 256);
	if (g > 256) g = 256;
	if (g < 1) g = 1;
	int gx = (c->tile_grid + B - 1) / B;
	if (gx > p->nbtiles) gx = (int)p->nbtiles;
	if (gx < 1) gx = 1;
	const size_t smem = (size_t)(p->max_tile_elems ? p->max_tile_elems : 1) * 2 * sizeof(unsigned int);
	cudaError_t e = cudaMemsetAsync(ctrl, 0, (size_t)2 * B * sizeof(unsigned int), st);
	if (e != cudaSuccess) return fail(JN_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
	if (!p->dim) return JN_OK;
	jn_prep_batched_kernel<<<dim3(g, B), 256, 0, st>>>(src, src_ld, d_sel, sel_ld, x64, f32 ? x32 : NULL, p->dim, ctrl,
							     d_active);
	if (p->nbtiles) {
		if (f32)
			jn_tile_kernel<float><<<dim3(gx, B), TILE_THREADS, smem, st>>>(
				P, c->d_btiles, p->nbtiles, ctrl + 1, (const uint2 *)c->d_items, c->d_pieces, c->d_tterms,
				c->d_walks, x32, (const float *)me, gacc, ctrl, abs_bound, p->dim, me_ld, d_active);
		else
			jn_tile_kernel<double><<<dim3(gx, B), TILE_THREADS, smem, st>>>(
				P, c->d_btiles, p->nbtiles, ctrl + 1, (const uint2 *)c->d_items, c->d_pieces, c->d_tterms,
				c->d_walks, x64, (const double *)me, gacc, ctrl, abs_bound, p->dim, me_ld, d_active);
	}
	jn_finalize_batched_kernel<<<dim3(g, B), 256, 0, st>>>(gacc, y, y_ld, p->dim, ctrl, abs_bound, d_active);
	e = cudaGetLastError();
	if (e != cudaSuccess) return fail(JN_ERR_CUDA, "batched product launch: %s", cudaGetErrorString(e));
	return JN_OK;
}

static jn_status enqueue(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st, cudaEvent_t pre,
		       cudaEvent_t mid)
{
	const jn_plan_t *p = &c->plan;
	DevPlan P = { c->d_rowptr, c->d_ent, c->d_me, c->d_terms, c->d_tiles, c->d_units, c->d_unit_terms };
	const int f32 = c->precision == 32;
	if (c->engine == 5) return jn_enqueue_walk(c, d_x, d_y, accumulate, st, pre, mid);
	if (f32 && !(c->engine == 4 && jn_panels_fit(c, 1))) {
		jn_status s = ensure_f32(c);
		if (s) return s;
	}
	int g = (int)((p->dim + 255) / 256);
	if (g > 1024) g = 1024;
	if (g < 1) g = 1;
	if (c->engine == 2) {
		const int ug = (p->nunits + WARPS - 1) / WARPS, tg = (p->ntiles + WARPS - 1) / WARPS;
		if (f32 && p->dim) jn_to_f32_kernel<<<g, 256, 0, st>>>(d_x, c->d_x32, p->dim);
		if (pre) cudaEventRecord(pre, st);
		if (f32) {
			if (p->nunits) jn_pieces_kernel<true><<<ug, WARPS * 32, 0, st>>>(P, c->d_x32, c->d_me32, c->d_partial, p->nunits);
		} else if (p->nunits) {
			jn_pieces_kernel<false><<<ug, WARPS * 32, 0, st>>>(P, d_x, c->d_me, c->d_partial, p->nunits);
		}
		if (mid) cudaEventRecord(mid, st);
		if (p->ntiles) jn_reduce_kernel<<<tg, WARPS * 32, 0, st>>>(c->d_tiles, p->ntiles, c->d_partial, d_y, accumulate);
	} else if (c->engine == 4 && jn_panels_fit(c, f32)) {
		jn_status s = jn_enqueue_panels(c, d_x, d_y, accumulate, st, pre, mid);
		if (s) return s;
	} else {
		jn_status s = jn_enqueue_tiles(c, d_x, d_y, accumulate, st, pre, mid, c->d_gacc, c->d_xmax, c->d_x32, 0);
		if (s) return s;
	}
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return fail(JN_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
	return JN_OK;
}

/* engine 2's plan and device arrays, built when it is first selected */
static jn_status units_setup(jn_ctx *c)
{
	jn_plan_t *p = &c->plan;
	if (c->d_units) return JN_OK;
	char err[1024] = { 0 };
	if (jn_plan_build_units(p, c->num_sms * 48, err, sizeof err)) return fail(JN_ERR_NOMEM, "%s", err);
	jn_status s;
	if ((s = upload(&c->d_tiles, p->tiles, p->ntiles)) || (s = upload(&c->d_unit_terms, p->unit_terms, p->n_unit_terms)) ||
	    (s = upload(&c->d_partial, (const void *)NULL, p->n_partial)) || (s = upload(&c->d_units, p->units, p->nunits))) {
		cudaFree(c->d_tiles); cudaFree(c->d_unit_terms); cudaFree(c->d_partial); cudaFree(c->d_units);
		c->d_tiles = NULL; c->d_unit_terms = NULL; c->d_partial = NULL; c->d_units = NULL;
		return s;
	}
	return JN_OK;
}

extern "C" jn_status jn_set_engine(jn_ctx *c, int engine)
{
	if (!c || engine < 2 || engine > 5) return fail(JN_ERR_INVALID, "engine must be 2, 3, 4 or 5");
	if (engine == 3 && c->plan.btiles_off) return fail(JN_ERR_INVALID, "no block-tile engine: %s", c->plan.btiles_why);
	if (engine == 2) {
		jn_status s = units_setup(c);
		if (s) return s;
	}
	if (engine == 4) {
		jn_status s = jn_panels_setup(c);
		if (s) return s;
	}
	if (engine == 5) {
		jn_status s = jn_walk_setup(c);
		if (s) return s;
	}
	c->engine = c->engine_of[0] = c->engine_of[1] = engine;
	return JN_OK;
}

extern "C" int jn_active_engine(const jn_ctx *c)
{
	if (!c) return -1;
	if (c->engine == 4 && !jn_panels_fit(c, c->precision == 32)) return 3;
	return c->engine;
}

jn_status jn_launch_matvec(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st)
{
	return enqueue(c, d_x, d_y, accumulate, st, NULL, NULL);
}

extern "C" jn_status jn_set_precision(jn_ctx *c, int precision)
{
	if (!c || (precision != 32 && precision != 64)) return fail(JN_ERR_INVALID, "precision must be 32 or 64");
	if (precision == 32) {
		/* the block-tile engine's FP32 copy, which the allocation-free product also reads */
		jn_status s = ensure_f32(c);
		if (s) return s;
	}
	c->precision = precision;
	c->engine = c->engine_of[precision == 32];
	return jn_panels_apply_tuned(c);
}

extern "C" jn_status jn_matvec_device(jn_ctx *c, const double *d_x, double *d_y, int accumulate, void *stream)
{
	if (!c || !d_x || !d_y) return fail(JN_ERR_INVALID, "null argument");
	if (d_x == d_y) return fail(JN_ERR_INVALID, "x and y must not alias");
	return jn_launch_matvec(c, d_x, d_y, accumulate, stream ? (cudaStream_t)stream : c->stream);
}

extern "C" jn_status jn_matvec_profile(jn_ctx *c, const double *d_x, double *d_y, int accumulate, float ms[2])
{
	if (!c || !d_x || !d_y || !ms) return fail(JN_ERR_INVALID, "null argument");
	if (d_x == d_y) return fail(JN_ERR_INVALID, "x and y must not alias");
	/* the events belong to the context, so that a product that runs as a
	 * cached graph records them from inside it: ms[0] is the product kernel,
	 * ms[1] the rest of the product (its other kernels and the gaps between
	 * them), both device time.  Engines launched kernel by kernel record the
	 * start and end events from the host around the launches. */
	for (int i = 0; i < 4; i++)
		if (!c->prof_ev[i]) CUDA_TRY(cudaEventCreate(&c->prof_ev[i]));
	const int in_graph = c->engine == 4 && jn_panels_fit(c, c->precision == 32);
	if (!in_graph) CUDA_TRY(cudaEventRecord(c->prof_ev[0], c->stream));
	jn_status s = enqueue(c, d_x, d_y, accumulate, c->stream, c->prof_ev[1], c->prof_ev[2]);
	if (s) return s;
	if (!in_graph) CUDA_TRY(cudaEventRecord(c->prof_ev[3], c->stream));
	CUDA_TRY(cudaEventSynchronize(c->prof_ev[3]));
	float total = 0.f;
	CUDA_TRY(cudaEventElapsedTime(&ms[0], c->prof_ev[1], c->prof_ev[2]));
	CUDA_TRY(cudaEventElapsedTime(&total, c->prof_ev[0], c->prof_ev[3]));
	ms[1] = total - ms[0];
	return JN_OK;
}

/* The fixed-point products (every engine but engine 2 at precision 64) bound
 * max|x| as an FP32 number and choose their unit 2^-S from abs_bound *
 * max|x|, with S kept in [-60, 100].  They are exact to FP64 level while
 * max|x| < 2^127 and abs_bound * max|x| lies in [2^-47, 2^121) (below 2^-38
 * the largest element still keeps at least 53 bits); outside that range a
 * result would be wrong or degraded, so the host-array entry points refuse
 * it.  x = 0 and all-zero matrix elements give exact zeros. */
static jn_status check_x_range(const jn_ctx *c, const double *x)
{
	if (c->engine == 2 && c->precision == 64) return JN_OK;
	double m = 0.0;
	for (int64_t i = 0; i < c->plan.dim; i++) {
		const double a = fabs(x[i]);
		if (!(a <= m)) m = a;           /* NaN is kept */
	}
	if (m == 0.0 || c->plan.abs_bound == 0.0) return JN_OK;
	if (!(m < 0x1p127))
		return fail(JN_ERR_INVALID, "max|x| = %g: the product bounds x in FP32 and needs max|x| < 2^127 "
			    "(scale x by a power of two, or select engine 2 at precision 64)", m);
	const double yb = c->plan.abs_bound * m;
	if (!(yb >= 0x1p-47 && yb < 0x1p121))
		return fail(JN_ERR_INVALID, "abs_bound * max|x| = %g is outside the fixed-point product's range [2^-47, 2^121) "
			    "(scale x by a power of two, or select engine 2 at precision 64)", yb);
	return JN_OK;
}

extern "C" jn_status jn_matvec(jn_ctx *c, const double *x, double *y)
{
	if (!c || !x || !y) return fail(JN_ERR_INVALID, "null argument");
	jn_status rs = check_x_range(c, x);
	if (rs) return rs;
	const size_t bytes = (size_t)c->plan.dim * sizeof(double);
	CUDA_TRY(cudaMemcpyAsync(c->d_x, x, bytes, cudaMemcpyHostToDevice, c->stream));
	CUDA_TRY(cudaMemcpyAsync(c->d_y, y, bytes, cudaMemcpyHostToDevice, c->stream));
	jn_status s = jn_launch_matvec(c, c->d_x, c->d_y, 1, c->stream);
	if (s) return s;
	CUDA_TRY(cudaMemcpyAsync(y, c->d_y, bytes, cudaMemcpyDeviceToHost, c->stream));
	CUDA_TRY(cudaStreamSynchronize(c->stream));
	return JN_OK;
}

extern "C" jn_status jn_synchronize(jn_ctx *c)
{
	if (!c) return fail(JN_ERR_INVALID, "null argument");
	CUDA_TRY(cudaStreamSynchronize(c->stream));
	return JN_OK;
}

static jn_status read_vec_file(const char *dir, int id, double *dst, size_t n)
{
	char path[8192];
	snprintf(path, sizeof path, "%s/vec_%d", dir, id);
	FILE *f = fopen(path, "rb");
	if (!f) return fail(JN_ERR_IO, "Could not open vector block file %s", path);
	size_t got = fread(dst, sizeof(double), n, f);
	fclose(f);
	if (got != n) return fail(JN_ERR_IO, "Could not read elements of block %d in %s", id, dir);
	return JN_OK;
}

extern "C" jn_status jn_matvec_files(jn_ctx *c, const char *out_dir, const char *in_dir)
{
	if (!c || !out_dir || !in_dir) return fail(JN_ERR_INVALID, "null argument");
	const jn_plan_t *p = &c->plan;
	double *x = (double *)malloc((p->dim ? p->dim : 1) * sizeof(double));
	double *y = (double *)malloc((p->dim ? p->dim : 1) * sizeof(double));
	jn_status s = JN_OK;
	if (!x || !y) { s = fail(JN_ERR_NOMEM, "out of host memory"); goto done; }
	for (int b = 0; b < p->nblocks && !s; b++) {
		const jn_block_t *B = &p->blocks[b];
		size_t n = (size_t)(B->Np * B->Nn);
		s = read_vec_file(in_dir, B->id, x + B->offset, n);
		if (!s) s = read_vec_file(out_dir, B->id, y + B->offset, n);
	}
	if (!s) s = jn_matvec(c, x, y);
	for (int b = 0; b < p->nblocks && !s; b++) {
		const jn_block_t *B = &p->blocks[b];
		size_t n = (size_t)(B->Np * B->Nn);
		char path[8192];
		snprintf(path, sizeof path, "%s/vec_%d", out_dir, B->id);
		FILE *f = fopen(path, "wb");
		if (!f) { s = fail(JN_ERR_IO, "Could not open vector block file %s", path); break; }
		if (fwrite(y + B->offset, sizeof(double), n, f) != n) s = fail(JN_ERR_IO, "Could not write elements to block %d in %s", B->id, out_dir);
		fclose(f);
	}
done:
	free(x); free(y);
	return s;
}

static void fill_stats(const jn_plan_t *p, jn_plan_stats *st)
{
	memset(st, 0, sizeof *st);
	st->dimension = (size_t)p->dim;
	st->num_blocks = p->nblocks;
	st->num_instructions = p->ninstr;
	st->list_entries = (size_t)p->list_entries;
	st->me_elements = (size_t)p->me_elements;
	st->me_referenced = (size_t)p->me_referenced;
	st->multiply_adds = p->visits;
	st->algorithmic_bytes = 12.0 * (double)p->list_entries + 8.0 * (double)p->me_referenced + 16.0 * (double)p->dim;
	st->num_work_units = p->nunits;
	st->num_tiles = p->ntiles;
}

extern "C" jn_status jn_get_plan_stats(const jn_ctx *c, jn_plan_stats *st)
{
	if (!c || !st) return fail(JN_ERR_INVALID, "null argument");
	fill_stats(&c->plan, st);
	return JN_OK;
}

extern "C" jn_status jn_inspect_files(const char *comb, const char *order, const char *lists_dir, const char *me_dir,
				      int Z, int N, jn_plan_stats *st)
{
	if (!comb || !order || !lists_dir || !me_dir || !st) return fail(JN_ERR_INVALID, "null argument");
	jn_plan_t plan;
	char err[1024] = { 0 };
	if (jn_plan_build(&plan, comb, order, lists_dir, me_dir, Z, N, 152 * 8, err, sizeof err))
		return fail(strstr(err, "open") ? JN_ERR_IO : JN_ERR_FORMAT, "%s", err);
	if (jn_plan_build_units(&plan, 152 * 8, err, sizeof err)) {
		jn_plan_free(&plan);
		return fail(JN_ERR_NOMEM, "%s", err);
	}
	fill_stats(&plan, st);
	jn_plan_free(&plan);
	return JN_OK;
}

extern "C" jn_status jn_read_settings(const char *conf, jn_run_settings *s)
{
	if (!conf || !s) return fail(JN_ERR_INVALID, "null argument");
	jn_runfile_t rf;
	char err[1024] = { 0 };
	if (jn_read_runfile(conf, &rf, err, sizeof err)) return fail(strstr(err, "could not read") ? JN_ERR_IO : JN_ERR_FORMAT, "%s", err);
	memset(s, 0, sizeof *s);
	snprintf(s->combination_table_file, sizeof s->combination_table_file, "%s", rf.comb);
	snprintf(s->evaluation_order_file, sizeof s->evaluation_order_file, "%s", rf.order);
	snprintf(s->index_lists_base_directory, sizeof s->index_lists_base_directory, "%s", rf.lists);
	snprintf(s->matrix_file_base_directory, sizeof s->matrix_file_base_directory, "%s", rf.mes);
	s->num_protons = rf.Z;
	s->num_neutrons = rf.N;
	snprintf(s->krylow_vector_directory, sizeof s->krylow_vector_directory, "%s", rf.krylov);
	s->max_num_lanczos_iterations = (int)rf.max_iterations;
	s->convergence_tolerance = rf.tolerance;
	s->target_eigenvector = (int)rf.target_eigenvector;
	s->converge_eigenvectors = rf.converge_eigenvectors;
	snprintf(s->eigenvector_directory, sizeof s->eigenvector_directory, "%s", rf.eigvec);
	s->gpu_num_eigenvalues = rf.num_eigenvalues;
	s->gpu_precision = rf.precision;
	s->gpu_full_reorthogonalization = rf.reorthogonalize;
	return JN_OK;
}
