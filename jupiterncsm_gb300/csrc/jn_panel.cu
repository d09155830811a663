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
 * coefficient of (proton entry j, neutron entry i) is s_p s_n M[k_n + Nd k_p],
 * stored densely and row-major: the product reads each coefficient once,
 * coalesced, with streaming (evict-first) loads, and the index lists only as
 * 4-byte packed (source, destination) pairs.  A warp task spreads up to 32
 * columns of a panel over its lanes (and 32 / columns rows side by side when
 * a panel is narrow) and walks rows; the x gathers hit L1.  The whole
 * output vector is accumulated in shared memory as 64-bit fixed-point
 * integers (two 32-bit atomics with carry): a lane sums the consecutive rows
 * that land on one output element in T arithmetic and adds the rounded run
 * once; the transposed contribution of an off-diagonal panel is rounded and
 * added per product.  Integer addition is exact and associative, so the
 * result is bit-identical whatever the order in which warps and CTAs run.
 * Persistent CTAs take contiguous runs of tasks that touch few blocks, and at
 * the end add only the touched ranges into the global accumulator.
 */
#include "jn_internal.h"
#include "jn_fixed.cuh"

#define PANEL_THREADS 512
#define PANEL_UNROLL 4

template <typename T> __device__ __forceinline__ T load_stream(const T *p) { return __ldcs(p); }

template <typename T, int KIND, bool DIAG>
__device__ __forceinline__ void panel_task(const uint4 pa, const uint4 pb, const uint4 pc, uint32_t j0, uint32_t j1,
					   int R, int r, int i, unsigned int *__restrict__ lo, unsigned int *__restrict__ hi,
					   const T *__restrict__ x, const T *__restrict__ coef,
					   const uint32_t *__restrict__ meta, const T scale)
{
	const int64_t c_off = (int64_t)pa.x | ((int64_t)pa.y << 32);
	const uint32_t row_meta = pa.z, col_meta = pa.w;
	const int out_off = (int)pb.x, in_off = (int)pb.y, Nn_out = (int)pb.z, Nn_in = (int)pb.w;
	const int ncols = (int)pc.x;
	int Ni, No;
	T ccol = 1;
	if (KIND == JN_KIND_P) {
		Ni = No = i;
	} else {
		const uint32_t m = __ldg(meta + col_meta + i);
		Ni = (int)(m & 0xffffu);
		No = (int)(m >> 16);
	}
	if (KIND == JN_KIND_N) ccol = __ldg(coef + c_off + i);
	const T *__restrict__ xin = x + in_off + Ni;
	const T *__restrict__ xout = x + out_off + No;
	const int yin = in_off + Ni, yout = out_off + No;
	const T *__restrict__ crow = coef + c_off + (KIND == JN_KIND_NP ? i : 0);
	int cur = -1;
	T run = 0;
	for (uint32_t j = j0 + r; j < j1; j += PANEL_UNROLL * R) {
		uint32_t mr[PANEL_UNROLL];
		T cv[PANEL_UNROLL];
		/* issue the row entries and coefficients of the next rows first */
#pragma unroll
		for (int u = 0; u < PANEL_UNROLL; u++) {
			const uint32_t jj = j + u * R;
			mr[u] = jj | (jj << 16);
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
			const int Pi = (int)(mr[u] & 0xffffu), Po = (int)(mr[u] >> 16);
			const T xi = __ldg(xin + Pi * Nn_in);
			if (Po != cur) {
				if (cur >= 0) add_fixed(lo, hi, yout + cur * Nn_out, to_fixed<T>(run * scale));
				cur = Po;
				run = 0;
			}
			run = fma(cv[u], xi, run);
			if (!DIAG) {
				const T xo = __ldg(xout + Po * Nn_out);
				add_fixed(lo, hi, yin + Pi * Nn_in, to_fixed<T>(cv[u] * xo * scale));
			}
		}
	}
	if (cur >= 0) add_fixed(lo, hi, yout + cur * Nn_out, to_fixed<T>(run * scale));
}

template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS) jn_panel_kernel(const uint4 *__restrict__ panels,
								 const uint4 *__restrict__ tasks,
								 const uint32_t *__restrict__ cta_ptr,
								 const uint2 *__restrict__ flush,
								 const uint32_t *__restrict__ flush_ptr,
								 const uint32_t *__restrict__ meta, const T *__restrict__ coef,
								 const T *__restrict__ x, unsigned long long *__restrict__ gacc,
								 const unsigned int *__restrict__ xmax_bits, double abs_bound,
								 int dim)
{
	extern __shared__ unsigned int sacc[];
	__shared__ unsigned int next_task;
	unsigned int *lo = sacc, *hi = sacc + dim;
	const int lane = threadIdx.x & 31;
	const uint32_t f0 = flush_ptr[blockIdx.x], f1 = flush_ptr[blockIdx.x + 1];
	/* clear the ranges this CTA touches */
	for (uint32_t f = f0; f < f1; f++) {
		const uint2 rg = flush[f];
		for (uint32_t e = threadIdx.x; e < rg.y; e += blockDim.x) {
			lo[rg.x + e] = 0u;
			hi[rg.x + e] = 0u;
		}
	}
	if (threadIdx.x == 0) next_task = 0;
	__syncthreads();
	const int S = fixed_exponent(*xmax_bits, abs_bound);
	const T scale = (T)ldexp(1.0, S);
	const uint32_t t0 = cta_ptr[blockIdx.x], nt = cta_ptr[blockIdx.x + 1] - t0;
	for (;;) {
		uint32_t k = 0;
		if (lane == 0) k = atomicAdd(&next_task, 1u);
		k = __shfl_sync(0xffffffffu, k, 0);
		if (k >= nt) break;
		const uint4 tk = __ldg(tasks + t0 + k);
		const uint4 pa = __ldg(panels + 3 * tk.x), pb = __ldg(panels + 3 * tk.x + 1), pc = __ldg(panels + 3 * tk.x + 2);
		const int lg = (int)(tk.w >> 24), R = 32 >> lg, r = lane >> lg;
		const int i = (int)(tk.w & 0xffffffu) + (lane & ((1 << lg) - 1));
		if (i >= (int)pc.x) continue;
		const int kind = (int)pc.y & 7;
		const bool diag = (pc.y & JN_PANEL_DIAG) != 0;
		if (kind == JN_KIND_NP) {
			if (diag) panel_task<T, JN_KIND_NP, true>(pa, pb, pc, tk.y, tk.z, R, r, i, lo, hi, x, coef, meta, scale);
			else panel_task<T, JN_KIND_NP, false>(pa, pb, pc, tk.y, tk.z, R, r, i, lo, hi, x, coef, meta, scale);
		} else if (kind == JN_KIND_N) {
			if (diag) panel_task<T, JN_KIND_N, true>(pa, pb, pc, tk.y, tk.z, R, r, i, lo, hi, x, coef, meta, scale);
			else panel_task<T, JN_KIND_N, false>(pa, pb, pc, tk.y, tk.z, R, r, i, lo, hi, x, coef, meta, scale);
		} else {
			if (diag) panel_task<T, JN_KIND_P, true>(pa, pb, pc, tk.y, tk.z, R, r, i, lo, hi, x, coef, meta, scale);
			else panel_task<T, JN_KIND_P, false>(pa, pb, pc, tk.y, tk.z, R, r, i, lo, hi, x, coef, meta, scale);
		}
	}
	__syncthreads();
	for (uint32_t f = f0; f < f1; f++) {
		const uint2 rg = flush[f];
		for (uint32_t e = threadIdx.x; e < rg.y; e += blockDim.x) {
			const unsigned long long v = (unsigned long long)lo[rg.x + e] | ((unsigned long long)hi[rg.x + e] << 32);
			if (v) atomicAdd(gacc + rg.x + e, v);
		}
	}
}

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
	cudaFree(c->d_pflush_ptr); cudaFree(c->d_pmeta); cudaFree(c->d_coef64); cudaFree(c->d_coef32);
	c->d_panels = NULL; c->d_ptasks = NULL; c->d_pcta = NULL; c->d_pflush = NULL;
	c->d_pflush_ptr = NULL; c->d_pmeta = NULL; c->d_coef64 = NULL; c->d_coef32 = NULL;
	c->panel_grid = 0;
}

jn_status jn_panels_setup(jn_ctx *c)
{
	jn_plan_t *p = &c->plan;
	if (p->dim > JN_PANEL_MAX_DIM) return jn_fail(JN_ERR_INVALID, "dimension %lld is above the panel engine's %d",
						       (long long)p->dim, JN_PANEL_MAX_DIM);
	if (c->panel_grid) return JN_OK;
	const size_t smem = (size_t)(p->dim ? p->dim : 1) * 2 * sizeof(unsigned int);
	int per_f = 0, per_d = 0;
	CUDA_TRY(cudaFuncSetAttribute(jn_panel_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	CUDA_TRY(cudaFuncSetAttribute(jn_panel_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_f, jn_panel_kernel<float>, PANEL_THREADS, smem));
	CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_d, jn_panel_kernel<double>, PANEL_THREADS, smem));
	int per = per_f < per_d ? per_f : per_d;
	if (per < 1) return jn_fail(JN_ERR_INVALID, "the panel kernel does not fit on an SM with %zu bytes of accumulator", smem);
	char err[512] = { 0 };
	if (jn_panels_build(p, c->num_sms * per, err, sizeof err)) return jn_fail(JN_ERR_NOMEM, "panel plan: %s", err);
	jn_status s;
	if ((s = upload_n(&c->d_panels, p->panels, (size_t)p->npanels)) ||
	    (s = upload_n(&c->d_ptasks, p->ptasks, (size_t)p->nptasks * 4)) ||
	    (s = upload_n(&c->d_pcta, p->pcta, (size_t)p->pgrid + 1)) ||
	    (s = upload_n(&c->d_pflush_ptr, p->pflush_ptr, (size_t)p->pgrid + 1)) ||
	    (s = upload_n(&c->d_pflush, p->pflush, (size_t)p->npflush * 2)) ||
	    (s = upload_n(&c->d_pmeta, p->pmeta, (size_t)p->n_pmeta))) {
		jn_panels_release(c);
		return s;
	}
	c->panel_grid = p->pgrid;
	return JN_OK;
}

/* coefficients of the context's matrix elements in the precision of the
 * context (built on first use and after the matrix elements change) */
static jn_status ensure_coefficients(jn_ctx *c, int f32)
{
	const jn_plan_t *p = &c->plan;
	if (f32 ? c->d_coef32 != NULL : c->d_coef64 != NULL) return JN_OK;
	const size_t n = (size_t)(p->n_coef ? p->n_coef : 1);
	void *h = malloc(n * (f32 ? sizeof(float) : sizeof(double)));
	if (!h) return jn_fail(JN_ERR_NOMEM, "out of host memory for %zu panel coefficients", n);
	jn_panels_coefficients(p, p->me, f32 ? NULL : (double *)h, f32 ? (float *)h : NULL);
	jn_status s = f32 ? upload_n(&c->d_coef32, h, (size_t)p->n_coef) : upload_n(&c->d_coef64, h, (size_t)p->n_coef);
	free(h);
	return s;
}

void jn_panels_invalidate(jn_ctx *c)
{
	cudaFree(c->d_coef64);
	cudaFree(c->d_coef32);
	c->d_coef64 = NULL;
	c->d_coef32 = NULL;
}

jn_status jn_enqueue_panels(jn_ctx *c, const double *d_x, double *d_y, int accumulate, cudaStream_t st, cudaEvent_t pre,
			    cudaEvent_t mid)
{
	const jn_plan_t *p = &c->plan;
	const int f32 = c->precision == 32;
	jn_status s = jn_panels_setup(c);
	if (!s) s = ensure_coefficients(c, f32);
	if (!s && f32 && !c->d_x32) s = upload_n(&c->d_x32, NULL, (size_t)p->dim);
	if (s) return s;
	unsigned int *ctrl = c->d_xmax;
	CUDA_TRY(cudaMemsetAsync(ctrl, 0, 2 * sizeof(unsigned int), st));
	jn_launch_prep(d_x, f32 ? c->d_x32 : NULL, p->dim, ctrl, st);
	if (pre) cudaEventRecord(pre, st);
	const size_t smem = (size_t)(p->dim ? p->dim : 1) * 2 * sizeof(unsigned int);
	if (p->nptasks) {
		if (f32)
			jn_panel_kernel<float><<<c->panel_grid, PANEL_THREADS, smem, st>>>(
				(const uint4 *)c->d_panels, (const uint4 *)c->d_ptasks, c->d_pcta, (const uint2 *)c->d_pflush,
				c->d_pflush_ptr, c->d_pmeta, c->d_coef32, c->d_x32, c->d_gacc, ctrl, p->abs_bound, (int)p->dim);
		else
			jn_panel_kernel<double><<<c->panel_grid, PANEL_THREADS, smem, st>>>(
				(const uint4 *)c->d_panels, (const uint4 *)c->d_ptasks, c->d_pcta, (const uint2 *)c->d_pflush,
				c->d_pflush_ptr, c->d_pmeta, c->d_coef64, d_x, c->d_gacc, ctrl, p->abs_bound, (int)p->dim);
	}
	if (mid) cudaEventRecord(mid, st);
	jn_launch_finalize(c->d_gacc, d_y, p->dim, ctrl, p->abs_bound, accumulate, st);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "panel product launch: %s", cudaGetErrorString(e));
	return JN_OK;
}
