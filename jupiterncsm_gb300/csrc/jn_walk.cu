/*
 * jn_walk.cu — the walk engine (engine 5): the index-list product with the
 * contributions summed in registers before they reach memory (host plan in
 * jn_walk.c, layout in jn_problem.h).
 *
 * Semantics are the reference Minerva kernels'
 * (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:
 * n list :20-77, p list :79-132, n x p lists :134-210, off-diagonal
 * transposes :212-462, |M| < 1e-12 skip of single-species terms :52-53).
 *
 * GB300 organisation.  A warp task is 32 lane chunks (up to U = 8, 4 or 2
 * entries of one walk each: one destination column; a walk's entries are
 * dealt to its lanes in turn) times the rows of a piece.  The rows are
 * grouped by their connection index: a group reads one contiguous row of its
 * matrix-element block (of its transposed copy for proton walks), so a lane
 * gathers the coefficients of its chunk from that row once per group,
 * through L1, and reuses them for every row of the group.  Warps take tasks
 * from a counter, so the tasks in flight are a narrow window of the plan's
 * order, which keeps the instructions that share a block together: L2 serves
 * each element to all of them.  For each row the lane gathers its chunk's x
 * values, sums the U products in registers, rounds the sum once to the
 * 64-bit fixed-point unit and adds it into its own slot (destination row,
 * lane) in shared memory: no atomics, no bank conflicts.  After the task a
 * segmented sum over the lanes of each walk gives one global add per
 * (destination row, walk).  A CTA is one warp, so the register file alone
 * sets how many warps an SM holds.
 *
 * Arithmetic (the template parameter MODE):
 *   32  FP32 coefficients and x, fused multiply-adds in entry order;
 *   64  FP64 coefficients and x, fused multiply-adds (GB300's FP64 pipe is
 *       narrow: this mode is bound by it);
 *   1   exact integers: coefficients and x as 52-bit fixed-point integers
 *       (each matrix-element block scaled to its own max|M|, x to max|x|)
 *       split into a signed high part (28 bits) and a low part (24 bits);
 *       c x = ch xh 2^48 + (ch xl + cl xh) 2^24 + cl xl, summed over the
 *       chunk in two 64-bit registers with three 32 x 32 -> 64-bit integer
 *       multiply-adds per contribution (cl xl < 2^48 is dropped), and the
 *       sum rounded once to the nearest output unit.  This is the FP64-grade
 *       product: its inputs keep 52 bits against their block's max|c| and
 *       against max|x|, every
 *       sum is exact, and it runs on the integer pipe.
 * Every row sum is rounded once, at a place fixed by the plan, and the
 * rounded sums are added as integers: the result is bit-identical from run
 * to run and independent of the grid.
 */
#include "jn_internal.h"
#include "jn_fixed.cuh"

#include <type_traits>

#define WALK_WARPS 1     /* one warp a CTA: 32 resident CTAs an SM, the most the integer path's 63 registers allow too */
#define WALK_THREADS (WALK_WARPS * 32)
#define WALK_SLOTS (JN_WALK_RS * 32)    /* per warp: one 64-bit slot per (destination row, lane) */
#define WALK_SMEM ((size_t)WALK_WARPS * WALK_SLOTS * sizeof(unsigned long long))

static_assert(sizeof(jn_wtask_t) == 16 && sizeof(jn_wpiece_t) == 32, "tasks are read as one uint4, pieces as two");

/* exponent of the 52-bit fixed-point x: |x| 2^Sx < 2^52 for the bound max|x| in xmax_bits */
__device__ __forceinline__ int walk_x_exponent(unsigned int xmax_bits)
{
	if (!(xmax_bits & 0x7fffffffu)) return 0;
	return 52 - ((int)((xmax_bits >> 23) & 0xff) - 126);
}

/* The output unit 2^-S and, for the integer path, the shift of a row sum
 * A 2^48 + B 2^24 (in units of 2^-(Sc + Sx)) down to it: S is the usual
 * fixed-point exponent (|y| 2^S < 2^62), lowered where needed so that the
 * shift is at least 49 bits (48 + sh, sh >= 1). */
__device__ __forceinline__ void walk_scales(unsigned int xmax_bits, double abs_bound, int Sc, int mode, int *S, int *sh)
{
	int s = fixed_exponent(xmax_bits, abs_bound), k = 0;
	if (mode == 1) {
		const int Sx = walk_x_exponent(xmax_bits);
		if (Sc + Sx - s < 49) s = Sc + Sx - 49;
		k = Sc + Sx - s - 48;
		if (k > 63) k = 63;
	}
	*S = s;
	*sh = k;
}

template <int MODE> struct WalkT;
template <> struct WalkT<32> { typedef float C; typedef float X; };
template <> struct WalkT<64> { typedef double C; typedef double X; };
template <> struct WalkT<1> { typedef int2 C; typedef int2 X; };

/* the sum of one row over a lane's chunk, rounded once to a 64-bit integer in output units */
template <int MODE, int U>
__device__ __forceinline__ long long walk_row(const typename WalkT<MODE>::C *c, const typename WalkT<MODE>::X *xv, uint32_t row,
					      int sh, float scalef, double scale)
{
	long long v;
	if constexpr (MODE == 1) {
		long long A = 0, B = 0;
#pragma unroll
		for (int u = 0; u < U; u++) {
			A += (long long)c[u].x * xv[u].x;
			B += (long long)c[u].x * xv[u].y;
			B += (long long)c[u].y * xv[u].x;
		}
		/* A 2^48 + B 2^24 rounded to the nearest multiple of 2^(48 + sh), sh >= 1
		   (ties up), then given the row's sign */
		const long long q = A + (B >> 24), m = (long long)((int)row >> 31);
		v = (((q + (1ll << (sh - 1))) >> sh) ^ m) - m;
	} else if constexpr (MODE == 32) {
		float acc = 0.0f;
#pragma unroll
		for (int u = 0; u < U; u++) acc = __fmaf_rn(c[u], xv[u], acc);
		v = __float2ll_rn(acc * ((row >> 31) ? -scalef : scalef));
	} else {
		double acc = 0.0;
#pragma unroll
		for (int u = 0; u < U; u++) acc = __fma_rn(c[u], xv[u], acc);
		v = __double2ll_rn(acc * ((row >> 31) ? -scale : scale));
	}
	return v;
}

/* the coefficient of lane entry u from its raw element and the lane's
 * multipliers (2 bits per entry, a two's complement: +1, -1, or 0 for
 * padding) */
template <int MODE>
__device__ __forceinline__ typename WalkT<MODE>::C walk_coef(typename WalkT<MODE>::C v, uint32_t mul, int u)
{
	const int m = (int)(mul << (30 - 2 * u)) >> 30;
	if constexpr (MODE == 1) {
		return make_int2(v.x * m, v.y * m);
	} else {
		if (!m) v = 0;
		return m < 0 ? -v : v;
	}
}

/* one warp task with chunks of U entries (see the file comment).  Rows are
 * taken two at a time, so that two rows' gathers of x are in flight at once;
 * up to two words after a group's last row are read ahead (the plan keeps
 * JN_WALK_ROW_SPARE zero words after the last row) and not used.  A group's first row pair issues its
 * gathers of x before the coefficients (loaded at the top of the group) are
 * first used, so the two latencies overlap. */
template <int MODE, int U>
__device__ __forceinline__ void walk_task(const uint4 ta, const uint4 pa, const uint4 pb, const uint32_t *__restrict__ lanes,
					  const uint32_t *__restrict__ walks, const uint32_t *__restrict__ rows,
					  const uint32_t *__restrict__ rdst, const uint32_t *__restrict__ groups,
					  const uint8_t *__restrict__ gshift, const typename WalkT<MODE>::C *__restrict__ elem,
					  const typename WalkT<MODE>::X *__restrict__ x, const typename WalkT<MODE>::X *__restrict__ xt,
					  unsigned long long *__restrict__ gacc, unsigned long long *__restrict__ slots, int lane,
					  int sh, float scalef, double scale)
{
	typedef typename WalkT<MODE>::C C;
	typedef typename WalkT<MODE>::X X;
	const int src_off = (int)pa.x, dst_off = (int)pa.y, stride = (int)pa.z, Nn_dst = (int)pa.w;
	const int rs = (int)(pb.w & 0xffu), wp = (int)((pb.w >> 8) & 1u), ngroups = (int)(pb.w >> 9);
	const uint32_t *__restrict__ L = lanes + ta.y + lane;
	const uint32_t head = __ldg(L);
	const int ws = (int)(head & 0xffffu);
	const uint32_t mul = head >> 16;
	int off[U];
#pragma unroll
	for (int k = 0; k < U / 2; k++) {
		const uint32_t w = __ldg(L + (1 + k) * 32);
		off[2 * k] = (int)(w & 0xffffu);
		off[2 * k + 1] = (int)(w >> 16);
	}
	/* proton walks read the transposed view: a row's entries index one row of the source block */
	const X *__restrict__ xs = (wp ? xt : x) + src_off;
	int j = (int)pb.x;
	uint32_t row = __ldg(rows + j);
	for (int g = 0; g < ngroups; g++) {
		const C *__restrict__ er = elem + __ldg(groups + (int)pb.z + g);
		/* the integer path scales each block by its own exponent: its rows shift further */
		int shg = sh;
		if constexpr (MODE == 1) {
			shg += (int)__ldg(gshift + (int)pb.z + g);
			if (shg > 62) shg = 62;
		}
		C c[U];
#pragma unroll
		for (int u = 0; u < U; u++) c[u] = __ldg(er + (__ldg(L + (1 + U / 2 + u) * 32) & 0x3fffffffu));
		for (bool first = true;; first = false) {
			/* this row and the next one of the group (if any) */
			const uint32_t row2 = __ldg(rows + j + 1);
			const bool two = !(row & JN_WALK_GROUP_END);
			const X *__restrict__ xb = xs + (int)(row & 0xffffu) * stride;
			const X *__restrict__ xb2 = xs + (two ? (int)(row2 & 0xffffu) * stride : 0);
			X xv[U], xv2[U];
#pragma unroll
			for (int u = 0; u < U; u++) xv[u] = __ldg(xb + off[u]);
#pragma unroll
			for (int u = 0; u < U; u++) xv2[u] = __ldg(xb2 + off[u]);
			const uint32_t next = __ldg(rows + j + 2);
			/* the coefficients' multipliers, applied after this pair's gathers are issued */
			if (first) {
#pragma unroll
				for (int u = 0; u < U; u++) c[u] = walk_coef<MODE>(c[u], mul, u);
			}
			slots[(int)((row >> 16) & 31u) * 32 + lane] += (unsigned long long)walk_row<MODE, U>(c, xv, row, shg, scalef, scale);
			if (two)
				slots[(int)((row2 >> 16) & 31u) * 32 + lane] +=
					(unsigned long long)walk_row<MODE, U>(c, xv2, row2, shg, scalef, scale);
			const bool end = !two || (row2 & JN_WALK_GROUP_END);
			j += two ? 2 : 1;
			row = two ? next : row2;
			if (end) break;
		}
	}
	__syncwarp();
	/* the task's slots into the global accumulator; slots are left zero.  The
	   lanes of one walk are a run of neighbouring lanes: a segmented sum over
	   each run (shuffles down, log2 of the longest run steps) leaves the
	   walk's total in the run's first lane, which adds it */
	const int ws_prev = __shfl_up_sync(0xffffffffu, ws, 1);     /* every lane takes part */
	const unsigned int starts = __ballot_sync(0xffffffffu, lane == 0 || ws != ws_prev);
	const unsigned int after = lane == 31 ? 0u : starts >> (lane + 1);
	const int end = after ? lane + __ffs(after) : 32;
	const bool first = (starts >> lane) & 1u;
	const int longest = __reduce_max_sync(0xffffffffu, first ? (unsigned int)(end - lane) : 0u);
	const int dw = (int)__ldg(walks + ta.z + ws);
	for (int r = 0; r < rs; r++) {
		unsigned long long v = slots[r * 32 + lane];
		slots[r * 32 + lane] = 0ull;
		for (int d = 1; d < longest; d <<= 1) {
			const unsigned long long t = __shfl_down_sync(0xffffffffu, v, d);
			if (lane + d < end) v += t;
		}
		if (first && v) {
			const int dr = (int)__ldg(rdst + (int)pb.y + r);
			atomicAdd(gacc + dst_off + (wp ? dw * Nn_dst + dr : dr * Nn_dst + dw), v);
		}
	}
	__syncwarp();
}

/* FP32: 32 warps an SM (64 registers); the 64-bit paths need more registers: 28 (72) */
template <int MODE>
__global__ void __launch_bounds__(WALK_THREADS, MODE == 32 ? 32 : 28)
	jn_walk_kernel(const uint4 *__restrict__ tasks, const uint4 *__restrict__ pieces, const uint32_t *__restrict__ lanes,
		       const uint32_t *__restrict__ walks, const uint32_t *__restrict__ rows,
		       const uint32_t *__restrict__ rdst, const uint32_t *__restrict__ groups,
		       const uint8_t *__restrict__ gshift, const typename WalkT<MODE>::C *__restrict__ elem,
		       const typename WalkT<MODE>::X *__restrict__ x, const typename WalkT<MODE>::X *__restrict__ xt,
		       unsigned long long *__restrict__ gacc, unsigned int *__restrict__ ctrl, long long ntasks,
		       double abs_bound, int Sc)
{
	extern __shared__ unsigned long long wslots[];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	unsigned long long *slots = wslots + warp * WALK_SLOTS;
	for (int i = lane; i < WALK_SLOTS; i += 32) slots[i] = 0ull;
	__syncwarp();
	int S, sh;
	walk_scales(ctrl[0], abs_bound, Sc, MODE, &S, &sh);
	const float scalef = MODE == 32 ? __int_as_float((127 + (S < -126 ? -126 : (S > 127 ? 127 : S))) << 23) : 0.0f;
	const double scale = MODE == 64 ? ldexp(1.0, S) : 0.0;
	/* warps take the next task from a counter (ctrl[1], zero at launch), so
	   the tasks in flight stay a window of about two tasks per warp: the
	   instructions that read one matrix-element block run together and L2
	   serves the block's rows to all of them (a fixed assignment lets warps
	   drift apart by many tasks, and the window with them) */
	unsigned int t = 0, tn = 0;
	if (lane == 0) t = atomicAdd(ctrl + 1, 1u);
	t = __shfl_sync(0xffffffffu, t, 0);
	for (; (long long)t < ntasks; t = __shfl_sync(0xffffffffu, tn, 0)) {
		if (lane == 0) tn = atomicAdd(ctrl + 1, 1u);
		const uint4 ta = __ldg(tasks + t);
		const uint4 pa = __ldg(pieces + 2 * ta.x), pb = __ldg(pieces + 2 * ta.x + 1);
		const uint32_t U = (ta.w >> 8) & 0xffu;
		if (U == 8)
			walk_task<MODE, 8>(ta, pa, pb, lanes, walks, rows, rdst, groups, gshift, elem, x, xt, gacc, slots, lane, sh, scalef,
					       scale);
		else if (U == 4)
			walk_task<MODE, 4>(ta, pa, pb, lanes, walks, rows, rdst, groups, gshift, elem, x, xt, gacc, slots, lane, sh, scalef,
					       scale);
		else
			walk_task<MODE, 2>(ta, pa, pb, lanes, walks, rows, rdst, groups, gshift, elem, x, xt, gacc, slots, lane, sh, scalef,
					       scale);
	}
}

/* x as 52-bit fixed-point integers {high 28 bits (signed), low 24 bits} */
__device__ __forceinline__ int2 walk_xsplit(double v, double s)
{
	const long long q = __double2ll_rn(v * s);
	return make_int2((int)(q >> 24), (int)(q & 0xffffff));
}

/* the x views the walk kernel reads in the arithmetic MODE: the integer
 * path's split copy of x (MODE 1; MODE 32 gets its FP32 copy from the max|x|
 * pass), and, where proton walks exist (perm != NULL), the transposed view
 * xT[i] = x[perm[i]] */
template <int MODE>
__global__ void jn_walk_xview_kernel(const double *__restrict__ x, const int32_t *__restrict__ perm,
				     typename WalkT<MODE>::X *__restrict__ xv, typename WalkT<MODE>::X *__restrict__ xt, int64_t n,
				     const unsigned int *__restrict__ ctrl)
{
	const double s = MODE == 1 ? ldexp(1.0, walk_x_exponent(ctrl[0])) : 1.0;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		if constexpr (MODE == 1) {
			xv[i] = walk_xsplit(x[i], s);
			if (perm) xt[i] = walk_xsplit(__ldg(x + __ldg(perm + i)), s);
		} else {
			xt[i] = (typename WalkT<MODE>::X)__ldg(x + __ldg(perm + i));
		}
	}
}

/* y (+)= acc 2^-S with the integer path's unit; the accumulator is cleared */
__global__ void jn_walk_finalize_kernel(unsigned long long *__restrict__ gacc, double *__restrict__ y, int64_t n,
					const unsigned int *__restrict__ ctrl, double abs_bound, int Sc, int mode,
					int accumulate)
{
	int S, sh;
	walk_scales(ctrl[0], abs_bound, Sc, mode, &S, &sh);
	const double unit = ldexp(1.0, -S);
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = (double)(long long)gacc[i] * unit;
		y[i] = accumulate ? y[i] + v : v;
		gacc[i] = 0ull;
	}
}

/* the walk element array in FP32 */
__global__ void jn_walk_f32_kernel(const double *__restrict__ a, int64_t n, float *__restrict__ out)
{
	for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
		out[e] = (float)a[e];
}

/* ------------------------------------------------------------------ */
/* host side                                                           */
/* ------------------------------------------------------------------ */
template <typename T>
static jn_status wupload(T **dst, const void *src, size_t n)
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

static int walk_mode(const jn_ctx *c) { return c->precision == 32 ? 32 : (c->walk_fp64 ? 64 : 1); }
static int walk_slot(int mode) { return mode == 32 ? 0 : (mode == 64 ? 1 : 2); }

void jn_walk_release(jn_ctx *c)
{
	cudaFree(c->d_wtasks); cudaFree(c->d_wpieces); cudaFree(c->d_wlanes); cudaFree(c->d_wwalks); cudaFree(c->d_wrows);
	cudaFree(c->d_wrdst); cudaFree(c->d_wgroups); cudaFree(c->d_wgshift); cudaFree(c->d_wx); cudaFree(c->d_wxt);
	cudaFree(c->d_wxperm);
	for (int i = 0; i < 3; i++) cudaFree(c->d_welem[i]);
	c->d_wtasks = NULL; c->d_wpieces = NULL; c->d_wlanes = NULL; c->d_wwalks = NULL; c->d_wrows = NULL;
	c->d_wrdst = NULL; c->d_wgroups = NULL; c->d_wgshift = NULL; c->d_wx = NULL; c->d_wxt = NULL; c->d_wxperm = NULL;
	for (int i = 0; i < 3; i++) c->d_welem[i] = NULL;
	c->walk_ready = 0;
}

void jn_walk_invalidate(jn_ctx *c)
{
	for (int i = 0; i < 3; i++) {
		cudaFree(c->d_welem[i]);
		c->d_welem[i] = NULL;
	}
}

jn_status jn_walk_setup(jn_ctx *c)
{
	if (c->walk_ready) return JN_OK;
	jn_plan_t *p = &c->plan;
	char err[512] = { 0 };
	if (jn_walk_build(p, err, sizeof err)) return jn_fail(JN_ERR_NOMEM, "walk plan: %s", err);
	jn_status s;
	if ((s = wupload(&c->d_wtasks, p->wtasks, (size_t)p->nwtasks)) ||
	    (s = wupload(&c->d_wpieces, p->wpieces, (size_t)p->nwpieces * 2)) ||
	    (s = wupload(&c->d_wlanes, p->wlanes, (size_t)p->n_wlanes)) ||
	    (s = wupload(&c->d_wwalks, p->wwalks, (size_t)p->n_wwalks)) ||
	    (s = wupload(&c->d_wrows, p->wrows, (size_t)p->n_wrows + JN_WALK_ROW_SPARE)) ||
	    (s = wupload(&c->d_wrdst, p->wrdst, (size_t)p->n_wrdst)) ||
	    (s = wupload(&c->d_wgroups, p->wgroups, (size_t)p->n_wgroups)) ||
	    (s = wupload(&c->d_wx, (const void *)NULL, (size_t)(p->dim ? p->dim : 1))) ||
	    (p->wxt && (s = wupload(&c->d_wxt, (const void *)NULL, (size_t)(p->dim ? p->dim : 1)))) ||
	    (p->wxt && (s = wupload(&c->d_wxperm, p->wxperm, (size_t)p->dim)))) {
		jn_walk_release(c);
		return s;
	}
	int per[3] = { 0, 0, 0 };
	cudaError_t e = cudaFuncSetAttribute(jn_walk_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WALK_SMEM);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(jn_walk_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WALK_SMEM);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(jn_walk_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WALK_SMEM);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[0], jn_walk_kernel<32>, WALK_THREADS, WALK_SMEM);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[1], jn_walk_kernel<64>, WALK_THREADS, WALK_SMEM);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[2], jn_walk_kernel<1>, WALK_THREADS, WALK_SMEM);
	if (e != cudaSuccess) {
		jn_walk_release(c);
		return jn_fail(JN_ERR_CUDA, "walk kernel set-up: %s", cudaGetErrorString(e));
	}
	for (int i = 0; i < 3; i++) {
		if (per[i] < 1) {
			jn_walk_release(c);
			return jn_fail(JN_ERR_CUDA, "the walk kernel does not fit on an SM");
		}
		c->walk_per_sm[i] = per[i];
	}
	c->walk_ready = 1;
	return JN_OK;
}

/* the walk element array of the current matrix elements for one arithmetic
 * (built on first use and after the matrix elements change): FP64
 * (arithmetic 64) from the FP64 array built on the host; FP32, converted on
 * the device from the FP64 copy when that exists, else on the host; the
 * integer path's split 52-bit values with their per-group shifts, formed on
 * the host straight from the plan's elements (only these reach the device
 * for it) */
static jn_status walk_elements(jn_ctx *c, int mode)
{
	const jn_plan_t *p = &c->plan;
	const int slot = walk_slot(mode);
	if (c->d_welem[slot]) return JN_OK;
	const int64_t n = p->n_wme;
	if (mode == 32 && c->d_welem[1]) {
		const double *a = (const double *)c->d_welem[1];
		cudaError_t e = cudaMalloc(&c->d_welem[0], (size_t)(n ? n : 1) * sizeof(float));
		if (e != cudaSuccess) {
			c->d_welem[0] = NULL;
			return jn_fail(JN_ERR_NOMEM, "cudaMalloc of %lld walk matrix elements: %s", (long long)n, cudaGetErrorString(e));
		}
		const int g = (int)(n / 256 + 1 < 4096 ? n / 256 + 1 : 4096);
		if (n) jn_walk_f32_kernel<<<g, 256, 0, c->stream>>>(a, n, (float *)c->d_welem[0]);
		e = cudaGetLastError();
		if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
		if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "walk matrix elements: %s", cudaGetErrorString(e));
		return JN_OK;
	}
	/* the exact integer path splits the plan's elements directly; the FP64
	   and FP32 paths start from the FP64 walk element array */
	double *h = NULL;
	if (mode == 64 || mode == 32) {
		h = (double *)malloc((size_t)(n ? n : 1) * sizeof(double));
		if (!h) return jn_fail(JN_ERR_NOMEM, "out of host memory for %lld walk matrix elements", (long long)n);
		jn_walk_elements(p, p->me, h);
	}
	jn_status s = JN_OK;
	if (mode == 64) {
		double *d = NULL;
		if (!(s = wupload(&d, h, (size_t)n))) c->d_welem[1] = d;
	} else if (mode == 32) {
		float *f = (float *)malloc((size_t)(n ? n : 1) * sizeof(float));
		if (!f) {
			s = jn_fail(JN_ERR_NOMEM, "out of host memory for %lld walk matrix elements", (long long)n);
		} else {
			for (int64_t e = 0; e < n; e++) f[e] = (float)h[e];
			float *d = NULL;
			if (!(s = wupload(&d, f, (size_t)n))) c->d_welem[0] = d;
			free(f);
		}
	} else {
		/* per-block exponents: every block keeps 52 bits against its own max|A| */
		int32_t *sp = (int32_t *)malloc((size_t)(n ? n : 1) * 2 * sizeof(int32_t));
		uint8_t *gs = (uint8_t *)malloc((size_t)(p->n_wgroups ? p->n_wgroups : 1));
		if (!sp || !gs) {
			s = jn_fail(JN_ERR_NOMEM, "out of host memory for %lld walk matrix elements", (long long)n);
		} else {
			jn_walk_int_elements(p, p->me, sp, gs, &c->walk_sc);
			int2 *d = NULL;
			s = wupload(&d, sp, (size_t)n);
			if (!s) {
				c->d_welem[2] = d;
				cudaFree(c->d_wgshift);
				c->d_wgshift = NULL;
				s = wupload(&c->d_wgshift, gs, (size_t)p->n_wgroups);
			}
		}
		free(sp); free(gs);
	}
	free(h);
	return s;
}

/* y (+)= H x on the walk engine: max|x| (and the converted copy of x), the
 * walk kernel, the conversion of the accumulator into y */
jn_status jn_enqueue_walk(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st, cudaEvent_t pre,
			  cudaEvent_t mid)
{
	const jn_plan_t *p = &c->plan;
	jn_status s = jn_walk_setup(c);
	const int mode = walk_mode(c);
	if (!s) s = walk_elements(c, mode);
	if (s) return s;
	int g = (int)((p->dim + 255) / 256);
	if (g > 1024) g = 1024;
	if (g < 1) g = 1;
	CUDA_TRY(cudaMemsetAsync(c->d_xmax, 0, 2 * sizeof(unsigned int), st));
	if (p->dim) {
		jn_launch_prep(d_x, mode == 32 ? (float *)c->d_wx : NULL, p->dim, c->d_xmax, st);
		const int32_t *perm = p->wxt ? c->d_wxperm : NULL;
		if (mode == 1)
			jn_walk_xview_kernel<1><<<g, 256, 0, st>>>(d_x, perm, c->d_wx, c->d_wxt, p->dim, c->d_xmax);
		else if (perm && mode == 32)
			jn_walk_xview_kernel<32><<<g, 256, 0, st>>>(d_x, perm, NULL, (float *)c->d_wxt, p->dim, c->d_xmax);
		else if (perm)
			jn_walk_xview_kernel<64><<<g, 256, 0, st>>>(d_x, perm, NULL, (double *)c->d_wxt, p->dim, c->d_xmax);
	}
	if (pre) cudaEventRecord(pre, st);
	if (p->nwtasks) {
		const int grid = c->num_sms * c->walk_per_sm[walk_slot(mode)];
		const uint4 *T = (const uint4 *)c->d_wtasks, *P = (const uint4 *)c->d_wpieces;
		if (mode == 32)
			jn_walk_kernel<32><<<grid, WALK_THREADS, WALK_SMEM, st>>>(
				T, P, c->d_wlanes, c->d_wwalks, c->d_wrows, c->d_wrdst, c->d_wgroups, NULL, (const float *)c->d_welem[0],
				(const float *)c->d_wx, (const float *)c->d_wxt, c->d_gacc, c->d_xmax, p->nwtasks, p->abs_bound, 0);
		else if (mode == 64)
			jn_walk_kernel<64><<<grid, WALK_THREADS, WALK_SMEM, st>>>(
				T, P, c->d_wlanes, c->d_wwalks, c->d_wrows, c->d_wrdst, c->d_wgroups, NULL, (const double *)c->d_welem[1],
				d_x, (const double *)c->d_wxt, c->d_gacc, c->d_xmax, p->nwtasks, p->abs_bound, 0);
		else
			jn_walk_kernel<1><<<grid, WALK_THREADS, WALK_SMEM, st>>>(
				T, P, c->d_wlanes, c->d_wwalks, c->d_wrows, c->d_wrdst, c->d_wgroups, c->d_wgshift, (const int2 *)c->d_welem[2],
				c->d_wx, c->d_wxt, c->d_gacc, c->d_xmax, p->nwtasks, p->abs_bound, c->walk_sc);
	}
	if (mid) cudaEventRecord(mid, st);
	if (p->dim) jn_walk_finalize_kernel<<<g, 256, 0, st>>>(c->d_gacc, d_y, p->dim, c->d_xmax, p->abs_bound, c->walk_sc, mode,
								accumulate);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "walk product launch: %s", cudaGetErrorString(e));
	return JN_OK;
}

/* ------------------------------------------------------------------ */
/* batched products over instances of several bases                    */
/* ------------------------------------------------------------------ */
/* One instance of a batched walk product: its basis's plan (on the
 * basis's context), its own walk element arrays, x views, accumulator and
 * scale bound, and its range of the batch's task list (128 bytes). */
struct jn_walk_inst {
	const uint4 *tasks, *pieces;
	const uint32_t *lanes, *walks, *rows, *rdst, *groups;
	const double *elem64;
	const float *elem32;
	float *x32;                     /* FP32 copy of the instance's x (arithmetic 32) */
	void *xt;                       /* transposed view of x in the arithmetic's type, NULL without proton walks */
	const int32_t *perm;            /* position in x of each element of that view */
	unsigned long long *gacc;
	int64_t dim;
	double abs_bound;               /* |H x| <= abs_bound max|x| */
	uint32_t task0, ntasks;         /* the instance's tasks in the batch's list */
};
static_assert(sizeof(jn_walk_inst) == 128, "one descriptor is 128 bytes");

struct jn_walk_batch {
	int B;
	jn_walk_inst *h, *d;
	uint32_t *d_task0;              /* B + 1 task offsets */
	uint32_t total;
	unsigned int *d_ctrl;           /* max|x| bits of instance i at 2 i; the task counter at 2 B */
	int num_sms, per_sm[2];         /* resident one-warp CTAs an SM: arithmetic 32, 64 */
	int has32;
};

/* max|x_i| into ctrl[2 i], the FP32 copy of x_i (MODE 32) and the
 * transposed view; x_i = src + i src_ld + (*sel) sel_ld */
template <int MODE>
__global__ void jn_walk_multi_prep_kernel(const jn_walk_inst *__restrict__ I, const double *__restrict__ src,
					  int64_t src_ld, const int *__restrict__ sel, int64_t sel_ld,
					  unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const jn_walk_inst d = I[inst];
	const double *x = src + inst * src_ld + (sel ? (int64_t)(*sel) * sel_ld : 0);
	typedef typename WalkT<MODE>::X X;
	X *xt = (X *)d.xt;
	float m = 0.0f;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.dim; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = x[i];
		if (MODE == 32) d.x32[i] = (float)v;
		if (xt) xt[i] = (X)x[d.perm[i]];
		m = fmaxf(m, (float)fabs(v) * 1.0000002f);     /* round-up margin of the FP32 conversion */
	}
	for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(ctrl + 2 * inst, __float_as_uint(m));
}

/* All instances' tasks in one persistent launch: a warp takes task t of
 * the batch's list from the counter, finds its instance (binary search of
 * the task offsets) and runs it with that instance's plan, elements, x
 * views and accumulator. */
template <int MODE>
__global__ void __launch_bounds__(WALK_THREADS, MODE == 32 ? 32 : 28)
	jn_walk_multi_kernel(const jn_walk_inst *__restrict__ I, const uint32_t *__restrict__ task0, int B, uint32_t total,
			     unsigned int *__restrict__ ctrl, const double *__restrict__ src, int64_t src_ld,
			     const int *__restrict__ sel, int64_t sel_ld, const int *__restrict__ active)
{
	extern __shared__ unsigned long long wslots[];
	const int lane = threadIdx.x & 31;
	unsigned long long *slots = wslots;
	for (int i = lane; i < WALK_SLOTS; i += 32) slots[i] = 0ull;
	__syncwarp();
	const int64_t k = sel ? (int64_t)(*sel) : 0;
	unsigned int t = 0, tn = 0;
	if (lane == 0) t = atomicAdd(ctrl + 2 * B, 1u);
	t = __shfl_sync(0xffffffffu, t, 0);
	for (; t < total; t = __shfl_sync(0xffffffffu, tn, 0)) {
		if (lane == 0) tn = atomicAdd(ctrl + 2 * B, 1u);
		int lo = 0, hi = B;             /* task0[lo] <= t < task0[hi] */
		while (hi - lo > 1) {
			const int mid = (lo + hi) >> 1;
			if (__ldg(task0 + mid) <= t) lo = mid;
			else hi = mid;
		}
		if (active && !active[lo]) continue;
		const jn_walk_inst *d = I + lo;
		int S, sh;
		walk_scales(ctrl[2 * lo], d->abs_bound, 0, MODE, &S, &sh);
		const float scalef = MODE == 32 ? __int_as_float((127 + (S < -126 ? -126 : (S > 127 ? 127 : S))) << 23) : 0.0f;
		const double scale = MODE == 64 ? ldexp(1.0, S) : 0.0;
		typedef typename WalkT<MODE>::C C;
		typedef typename WalkT<MODE>::X X;
		const C *elem;
		const X *x;
		if constexpr (MODE == 32) {
			elem = d->elem32;
			x = d->x32;
		} else {
			elem = d->elem64;
			x = src + lo * src_ld + k * sel_ld;
		}
		const X *xt = (const X *)d->xt;
		const uint4 ta = __ldg(d->tasks + (t - __ldg(task0 + lo)));
		const uint4 pa = __ldg(d->pieces + 2 * ta.x), pb = __ldg(d->pieces + 2 * ta.x + 1);
		const uint32_t U = (ta.w >> 8) & 0xffu;
		if (U == 8)
			walk_task<MODE, 8>(ta, pa, pb, d->lanes, d->walks, d->rows, d->rdst, d->groups, NULL, elem, x, xt, d->gacc,
					   slots, lane, sh, scalef, scale);
		else if (U == 4)
			walk_task<MODE, 4>(ta, pa, pb, d->lanes, d->walks, d->rows, d->rdst, d->groups, NULL, elem, x, xt, d->gacc,
					   slots, lane, sh, scalef, scale);
		else
			walk_task<MODE, 2>(ta, pa, pb, d->lanes, d->walks, d->rows, d->rdst, d->groups, NULL, elem, x, xt, d->gacc,
					   slots, lane, sh, scalef, scale);
	}
}

/* y_i = acc_i 2^-S_i (y + i y_ld); the accumulators are cleared */
template <int MODE>
__global__ void jn_walk_multi_finalize_kernel(const jn_walk_inst *__restrict__ I, double *__restrict__ y, int64_t y_ld,
					      const unsigned int *__restrict__ ctrl, const int *__restrict__ active)
{
	const int inst = blockIdx.y;
	if (active && !active[inst]) return;
	const jn_walk_inst d = I[inst];
	int S, sh;
	walk_scales(ctrl[2 * inst], d.abs_bound, 0, MODE, &S, &sh);
	const double unit = ldexp(1.0, -S);
	double *yy = y + inst * y_ld;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.dim; i += (int64_t)gridDim.x * blockDim.x) {
		yy[i] = (double)(long long)d.gacc[i] * unit;
		d.gacc[i] = 0ull;
	}
}

void jn_walk_batch_free(jn_walk_batch *wb)
{
	if (!wb) return;
	if (wb->h)
		for (int i = 0; i < wb->B; i++) {
			cudaFree((void *)wb->h[i].elem64);
			cudaFree((void *)wb->h[i].elem32);
			cudaFree(wb->h[i].x32);
			cudaFree(wb->h[i].xt);
			cudaFree(wb->h[i].gacc);
		}
	free(wb->h);
	cudaFree(wb->d);
	cudaFree(wb->d_task0);
	cudaFree(wb->d_ctrl);
	free(wb);
}

jn_status jn_walk_batch_create(jn_ctx *const *ctxs, const int *inst_ctx, int B, const double *const *me, int want32,
			       jn_walk_batch **out)
{
	*out = NULL;
	if (B < 1 || B > 65535) return jn_fail(JN_ERR_INVALID, "batch of %d instances", B);
	jn_walk_batch *wb = (jn_walk_batch *)calloc(1, sizeof *wb);
	if (!wb) return jn_fail(JN_ERR_NOMEM, "out of host memory");
	wb->B = B;
	wb->has32 = want32;
	wb->h = (jn_walk_inst *)calloc((size_t)B, sizeof(jn_walk_inst));
	uint32_t *task0 = (uint32_t *)malloc((size_t)(B + 1) * sizeof(uint32_t));
	jn_status s = (!wb->h || !task0) ? jn_fail(JN_ERR_NOMEM, "out of host memory") : JN_OK;
	double *hbuf = NULL;
	int64_t hcap = 0;
	uint64_t total = 0;
	for (int i = 0; i < B && !s; i++) {
		jn_ctx *c = ctxs[inst_ctx[i]];
		if ((s = jn_walk_setup(c))) break;
		const jn_plan_t *p = &c->plan;
		jn_walk_inst *d = &wb->h[i];
		d->tasks = (const uint4 *)c->d_wtasks;
		d->pieces = (const uint4 *)c->d_wpieces;
		d->lanes = c->d_wlanes;
		d->walks = c->d_wwalks;
		d->rows = c->d_wrows;
		d->rdst = c->d_wrdst;
		d->groups = c->d_wgroups;
		d->perm = p->wxt ? c->d_wxperm : NULL;
		d->dim = p->dim;
		d->abs_bound = jn_plan_abs_bound(p, me[i]);
		d->task0 = (uint32_t)total;
		d->ntasks = (uint32_t)p->nwtasks;
		task0[i] = (uint32_t)total;
		total += (uint64_t)p->nwtasks;
		if (total > 0xf0000000ull) { s = jn_fail(JN_ERR_INVALID, "the batch has too many walk tasks"); break; }
		/* the instance's walk element arrays: FP64 built on the host, FP32 converted on the device */
		const int64_t n = p->n_wme;
		if (n > hcap) {
			free(hbuf);
			hcap = n;
			hbuf = (double *)malloc((size_t)hcap * sizeof(double));
			if (!hbuf) { s = jn_fail(JN_ERR_NOMEM, "out of host memory"); break; }
		}
		if (n) jn_walk_elements(p, me[i], hbuf);
		double *e64 = NULL;
		if ((s = wupload(&e64, hbuf, (size_t)n))) break;
		d->elem64 = e64;
		if (want32) {
			float *e32 = NULL;
			if ((s = wupload(&e32, (const void *)NULL, (size_t)n))) break;
			d->elem32 = e32;
			const int g = (int)(n / 256 + 1 < 4096 ? n / 256 + 1 : 4096);
			if (n) jn_walk_f32_kernel<<<g, 256, 0, c->stream>>>(e64, n, e32);
			float *x32 = NULL;
			if ((s = wupload(&x32, (const void *)NULL, (size_t)p->dim))) break;
			d->x32 = x32;
		}
		if (p->wxt) {
			double *xt = NULL;
			if ((s = wupload(&xt, (const void *)NULL, (size_t)p->dim))) break;
			d->xt = xt;
		}
		unsigned long long *g = NULL;
		if ((s = wupload(&g, (const void *)NULL, (size_t)p->dim))) break;
		if (cudaMemset(g, 0, (size_t)(p->dim ? p->dim : 1) * sizeof(unsigned long long)) != cudaSuccess)
			s = jn_fail(JN_ERR_CUDA, "cudaMemset of a batch accumulator");
		d->gacc = g;
		if (!wb->num_sms) {
			wb->num_sms = c->num_sms;
			wb->per_sm[0] = c->walk_per_sm[0];
			wb->per_sm[1] = c->walk_per_sm[1];
		}
	}
	free(hbuf);
	if (!s) {
		task0[B] = (uint32_t)total;
		wb->total = (uint32_t)total;
		if ((s = wupload(&wb->d, wb->h, (size_t)B)) || (s = wupload(&wb->d_task0, task0, (size_t)B + 1)) ||
		    (s = wupload(&wb->d_ctrl, (const void *)NULL, (size_t)2 * B + 1)))
			;
	}
	free(task0);
	if (!s) {
		cudaError_t e = cudaFuncSetAttribute(jn_walk_multi_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
						     (int)WALK_SMEM);
		int per = 0;
		if (e == cudaSuccess) e = cudaFuncSetAttribute(jn_walk_multi_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
							       (int)WALK_SMEM);
		if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, jn_walk_multi_kernel<32>, WALK_THREADS, WALK_SMEM);
		if (e == cudaSuccess) wb->per_sm[0] = per;
		if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, jn_walk_multi_kernel<64>, WALK_THREADS, WALK_SMEM);
		if (e == cudaSuccess) wb->per_sm[1] = per;
		if (e == cudaSuccess) e = cudaDeviceSynchronize();
		if (e != cudaSuccess) s = jn_fail(JN_ERR_CUDA, "batched walk set-up: %s", cudaGetErrorString(e));
		else if (wb->per_sm[0] < 1 || wb->per_sm[1] < 1) s = jn_fail(JN_ERR_CUDA, "the batched walk kernel does not fit on an SM");
	}
	if (s) {
		jn_walk_batch_free(wb);
		return s;
	}
	*out = wb;
	return JN_OK;
}

jn_status jn_walk_batch_enqueue(jn_walk_batch *wb, int mode, const double *src, int64_t src_ld, const int *d_sel,
				int64_t sel_ld, double *y, int64_t y_ld, const int *d_active, int64_t max_dim, cudaStream_t st)
{
	if (mode != 32 && mode != 64) return jn_fail(JN_ERR_INVALID, "batched walk arithmetic %d", mode);
	if (mode == 32 && !wb->has32) return jn_fail(JN_ERR_INVALID, "the batch has no FP32 elements");
	const int B = wb->B;
	int g = (int)((max_dim + 255) / 256);
	if (g > 256) g = 256;
	if (g < 1) g = 1;
	CUDA_TRY(cudaMemsetAsync(wb->d_ctrl, 0, (size_t)(2 * B + 1) * sizeof(unsigned int), st));
	const int grid = wb->num_sms * wb->per_sm[mode == 32 ? 0 : 1];
	if (mode == 32) {
		jn_walk_multi_prep_kernel<32><<<dim3(g, B), 256, 0, st>>>(wb->d, src, src_ld, d_sel, sel_ld, wb->d_ctrl, d_active);
		if (wb->total)
			jn_walk_multi_kernel<32><<<grid, WALK_THREADS, WALK_SMEM, st>>>(wb->d, wb->d_task0, B, wb->total, wb->d_ctrl,
											 src, src_ld, d_sel, sel_ld, d_active);
		jn_walk_multi_finalize_kernel<32><<<dim3(g, B), 256, 0, st>>>(wb->d, y, y_ld, wb->d_ctrl, d_active);
	} else {
		jn_walk_multi_prep_kernel<64><<<dim3(g, B), 256, 0, st>>>(wb->d, src, src_ld, d_sel, sel_ld, wb->d_ctrl, d_active);
		if (wb->total)
			jn_walk_multi_kernel<64><<<grid, WALK_THREADS, WALK_SMEM, st>>>(wb->d, wb->d_task0, B, wb->total, wb->d_ctrl,
											 src, src_ld, d_sel, sel_ld, d_active);
		jn_walk_multi_finalize_kernel<64><<<dim3(g, B), 256, 0, st>>>(wb->d, y, y_ld, wb->d_ctrl, d_active);
	}
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "batched walk product launch: %s", cudaGetErrorString(e));
	return JN_OK;
}

extern "C" jn_status jn_set_walk_arithmetic(jn_ctx *c, int fp64_fma)
{
	if (!c) return jn_fail(JN_ERR_INVALID, "null argument");
	if (fp64_fma != 0 && fp64_fma != 1) return jn_fail(JN_ERR_INVALID, "walk arithmetic %d: must be 0 (exact integers) or 1 (FP64)", fp64_fma);
	c->walk_fp64 = fp64_fma;
	return JN_OK;
}

extern "C" jn_status jn_walk_stats(jn_ctx *c, double *out)
{
	if (!c || !out) return jn_fail(JN_ERR_INVALID, "null argument");
	jn_status s = jn_walk_setup(c);
	if (s) return s;
	const jn_plan_t *p = &c->plan;
	out[0] = (double)p->nwtasks;
	out[1] = (double)p->nwpieces;
	out[2] = (double)p->n_wgroups;
	out[3] = p->wvisits;
	out[4] = p->wlane_slots;
	out[5] = (double)p->n_wme;
	out[6] = (double)(c->num_sms * c->walk_per_sm[walk_slot(walk_mode(c))]);
	return JN_OK;
}
