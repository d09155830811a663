/*
 * jn_lanczos.cu — the Lanczos eigensolver of Bacchus on the GPU, in FP64.
 *
 * Reference: src/Bacchus/lanczos/lanczos.c.  One iteration
 * (lanczos_iteration, :74-153) is
 *     w = H v_k;  alpha_k = <v_k|w>;  w -= alpha_k v_k + beta_{k-1} v_{k-1};
 *     beta_k = |w|;  v_{k+1} = w / beta_k
 * followed by reorthogonalisation (orthogonalize_krylow_basis, :155-169) and
 * the eigen-decomposition of the tridiagonal matrix (diagonalize, :171-253;
 * dsteqr in src/Bacchus/diagonalization/diagonalization.c:16-68).
 *
 * Two modes:
 *   JN_LANCZOS_REFERENCE  the reference's choices: start vector e_0
 *                         (lanczos.c:60-72), reorthogonalisation of
 *                         v_{k+1} against v_0..v_{k-3} only, without
 *                         renormalising (lanczos.c:155-169,
 *                         vector.c:461-476), convergence when the target
 *                         (ground-state) Ritz value moves by less than the
 *                         tolerance (lanczos.c:199-235).
 *   JN_LANCZOS_FULL       full reorthogonalisation (classical Gram-Schmidt,
 *                         applied twice) and convergence when the error
 *                         bound min(r, r^2/gap) of each of the lowest `nev`
 *                         Ritz values is below the tolerance, r being the
 *                         residual norm beta_k |s_{k,i}|.
 *
 * The Krylov basis stays in HBM.  Every reduction is a two-pass fixed-order
 * reduction, so two runs give bit-identical alpha/beta.  The tridiagonal
 * eigenvalues are computed on the GPU by Sturm-sequence bisection (one
 * thread per eigenvalue) and the eigenvectors by inverse iteration on the
 * tridiagonal matrix; the final Ritz vectors are refined by FP64 products
 * (Rayleigh quotient and residual norm).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <time.h>

#include <vector>

#include "jn_internal.h"
#include "jn_tridiag.cuh"

#define RED_BLOCKS 304      /* 2 x 152 SMs */
#define RED_THREADS 256

struct jn_lanczos_state {
	int64_t D;
	int mmax;               /* allocated Krylov dimension (vectors mmax+1) */
	int k;                  /* Lanczos steps done */
	int nev;
	double *d_V;            /* (mmax+1) x D */
	double *d_w;
	double *d_alpha, *d_beta;
	double *d_part;         /* RED_BLOCKS x (mmax+2) partials */
	double *d_h;            /* mmax+2 coefficients */
	double *d_scalar;       /* 4 scalars */
	double *d_theta;        /* Ritz values (ascending), mmax */
	double *d_Z;            /* nev_cap x mmax tridiagonal eigenvectors */
	double *d_ritz;         /* nev x D Ritz vectors */
	double *h_alpha, *h_beta;
	double *h_theta;
	double *h_zlast;        /* bottom components */
	int nev_cap;
	int have_ritz;
	double *h_rq, *h_res;   /* refined Rayleigh quotients and residual norms */
};

void jn_lanczos_release(jn_ctx *c)
{
	struct jn_lanczos_state *s = c->lz;
	if (!s) return;
	cudaFree(s->d_V); cudaFree(s->d_w); cudaFree(s->d_alpha); cudaFree(s->d_beta); cudaFree(s->d_part);
	cudaFree(s->d_h); cudaFree(s->d_scalar); cudaFree(s->d_theta); cudaFree(s->d_Z); cudaFree(s->d_ritz);
	free(s->h_alpha); free(s->h_beta); free(s->h_theta); free(s->h_zlast); free(s->h_rq); free(s->h_res);
	free(s);
	c->lz = NULL;
}

/* ------------------------------------------------------------------ */
/* BLAS-1/2 kernels with fixed reduction order                         */
/* ------------------------------------------------------------------ */

/* part[b*ncol + j] = sum over this block's slice of V[j] . w, j < nvec:
 * warp j % (warps) owns vector j and reduces it with shuffles in a fixed
 * order, so the vectors run side by side with no CTA-wide barrier */
__global__ void __launch_bounds__(RED_THREADS) k_gemv_t(const double *__restrict__ V, int64_t D, int nvec,
							 const double *__restrict__ w, double *__restrict__ part, int ncol)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
	const int64_t chunk = (D + gridDim.x - 1) / gridDim.x;
	const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(D, i0 + chunk);
	for (int j = warp; j < nvec; j += nwarps) {
		const double *v = V + (int64_t)j * D;
		double s = 0.0;
		for (int64_t i = i0 + lane; i < i1; i += 32) s = fma(v[i], w[i], s);
		for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
		if (lane == 0) part[(int64_t)blockIdx.x * ncol + j] = s;
	}
}

/* out[j] = sum_b part[b*ncol + j], one warp per j: lane l sums blocks
 * l, l + 32, ... in order, then the lanes' sums are added by a fixed
 * shuffle tree (the partials' loads are in flight together) */
__global__ void k_finish(const double *__restrict__ part, int nblk, int ncol, int nvec, double *__restrict__ out)
{
	const int j = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
	if (j >= nvec) return;          /* warp-uniform */
	double s = 0.0;
	for (int b = lane; b < nblk; b += 32) s += part[(int64_t)b * ncol + j];
	for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if (lane == 0) out[j] = s;
}

/* w -= sum_j V[j] h[j] (j < nvec) */
__global__ void k_gemv_n_sub(const double *__restrict__ V, int64_t D, int nvec, const double *__restrict__ h,
			     double *__restrict__ w)
{
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int j = 0; j < nvec; j++) s = fma(V[(int64_t)j * D + i], h[j], s);
		w[i] -= s;
	}
}

/* out = sum_j V[j] z[j] */
__global__ void k_gemv_n(const double *__restrict__ V, int64_t D, int nvec, const double *__restrict__ z,
			 double *__restrict__ out)
{
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int j = 0; j < nvec; j++) s = fma(V[(int64_t)j * D + i], z[j], s);
		out[i] = s;
	}
}

/* w -= a*v + b*u (reads a = *pa, b = *pb on the device; u may be NULL) */
__global__ void k_three_term(double *__restrict__ w, const double *__restrict__ v, const double *__restrict__ u,
			     const double *pa, const double *pb, int64_t D)
{
	const double a = *pa, b = pb ? *pb : 0.0;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
		double r = w[i] - a * v[i];
		if (u) r -= b * u[i];
		w[i] = r;
	}
}

/* dst = src / sqrt(*nrm2) ; beta_out = sqrt(*nrm2) */
__global__ void k_normalize(double *__restrict__ dst, const double *__restrict__ src, const double *nrm2,
			    double *beta_out, int64_t D)
{
	const double b = sqrt(*nrm2);
	if (blockIdx.x == 0 && threadIdx.x == 0 && beta_out) *beta_out = b;
	const double inv = 1.0 / b;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x)
		dst[i] = src[i] * inv;
}

__global__ void k_scale_copy(double *__restrict__ dst, const double *__restrict__ src, double s, int64_t D)
{
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x)
		dst[i] = src[i] * s;
}

__global__ void k_axpy_neg(double *__restrict__ y, const double *__restrict__ x, const double *pa, int64_t D)
{
	const double a = *pa;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x)
		y[i] -= a * x[i];
}

/* ------------------------------------------------------------------ */
/* tridiagonal eigenproblem                                            */
/* ------------------------------------------------------------------ */
/* theta[i] for i = blockIdx.x < want: the i-th smallest eigenvalue, by warp multisection */
__global__ void k_tri_bisect(const double *__restrict__ a, const double *__restrict__ b, int n, int want,
			     double *__restrict__ theta)
{
	const int i = blockIdx.x;
	if (i >= want) return;
	const double v = jn_tri_multisect_warp(a, b, n, i);
	if (threadIdx.x == 0) theta[i] = v;
}

/* eigenvector of T for theta[i] by inverse iteration; Z row i holds the n components */
__global__ void k_tri_vectors(const double *__restrict__ a, const double *__restrict__ b, int n, int want,
			      const double *__restrict__ theta, double *__restrict__ Z, int ldz, double *__restrict__ work,
			      int ldw)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= want) return;
	jn_tri_vector_one(a, b, n, theta[i], Z + (int64_t)i * ldz, work + (int64_t)i * ldw);
}

/* modified Gram-Schmidt among the `want` tridiagonal eigenvectors (one CTA) */
__global__ void k_tri_mgs(double *__restrict__ Z, int ldz, int n, int want)
{
	__shared__ double sh[RED_THREADS];
	jn_tri_mgs(Z, ldz, n, want, sh);
}

/* ------------------------------------------------------------------ */
/* host driver                                                         */
/* ------------------------------------------------------------------ */
static double seconds_now(void)
{
	struct timespec t;
	clock_gettime(CLOCK_MONOTONIC, &t);
	return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static int grid_for(int64_t D) { int64_t g = (D + 255) / 256; return (int)(g < 4096 ? (g > 0 ? g : 1) : 4096); }

/* res = <x|y> into device scalar */
static void dot_dev(jn_ctx *c, const double *x, const double *y, double *res)
{
	struct jn_lanczos_state *s = c->lz;
	k_gemv_t<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(x, s->D, 1, y, s->d_part, 1);
	k_finish<<<1, 32, 0, c->stream>>>(s->d_part, RED_BLOCKS, 1, 1, res);
}

/* w -= V[0..nvec) (V[0..nvec)^T w) */
static void cgs_pass(jn_ctx *c, int nvec)
{
	struct jn_lanczos_state *s = c->lz;
	if (nvec <= 0) return;
	int ncol = s->mmax + 2;
	k_gemv_t<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(s->d_V, s->D, nvec, s->d_w, s->d_part, ncol);
	k_finish<<<(nvec + 3) / 4, 128, 0, c->stream>>>(s->d_part, RED_BLOCKS, ncol, nvec, s->d_h);
	k_gemv_n_sub<<<grid_for(s->D), 256, 0, c->stream>>>(s->d_V, s->D, nvec, s->d_h, s->d_w);
}

static jn_status ensure_state(jn_ctx *c, int mmax, int nev)
{
	struct jn_lanczos_state *s = c->lz;
	int64_t D = c->plan.dim;
	if (s && s->mmax >= mmax && s->nev_cap >= nev) return JN_OK;
	jn_lanczos_release(c);
	s = (struct jn_lanczos_state *)calloc(1, sizeof *s);
	c->lz = s;
	s->D = D; s->mmax = mmax; s->nev_cap = nev;
	size_t ncol = (size_t)mmax + 2;
	cudaError_t e = cudaSuccess;
#define DALLOC(ptr, n) if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), (size_t)(n) * sizeof(double))
	DALLOC(s->d_V, (size_t)(mmax + 1) * D);
	DALLOC(s->d_w, D);
	DALLOC(s->d_alpha, mmax + 1);
	DALLOC(s->d_beta, mmax + 1);
	DALLOC(s->d_part, RED_BLOCKS * ncol);
	DALLOC(s->d_h, ncol);
	DALLOC(s->d_scalar, 8);
	DALLOC(s->d_theta, mmax + 1);
	DALLOC(s->d_Z, (size_t)nev * (mmax + 1) + (size_t)nev * 5 * (mmax + 1));
	DALLOC(s->d_ritz, (size_t)nev * D);
#undef DALLOC
	if (e != cudaSuccess) {
		jn_lanczos_release(c);
		return jn_fail(JN_ERR_NOMEM, "Lanczos workspace (%d vectors of %lld): %s", mmax + 1, (long long)D,
			       cudaGetErrorString(e));
	}
	s->h_alpha = (double *)calloc(mmax + 1, sizeof(double));
	s->h_beta = (double *)calloc(mmax + 1, sizeof(double));
	s->h_theta = (double *)calloc(mmax + 1, sizeof(double));
	s->h_zlast = (double *)calloc(nev + 1, sizeof(double));
	s->h_rq = (double *)calloc(nev + 1, sizeof(double));
	s->h_res = (double *)calloc(nev + 1, sizeof(double));
	return JN_OK;
}

/* Ritz values of T_n (ascending) for the lowest `want`, and the tridiagonal
 * eigenvectors when vectors != 0; results copied to the host arrays. */
static jn_status tri_eig(jn_ctx *c, int n, int want, int vectors)
{
	struct jn_lanczos_state *s = c->lz;
	if (want > n) want = n;
	k_tri_bisect<<<want, 32, 0, c->stream>>>(s->d_alpha, s->d_beta, n, want, s->d_theta);
	if (vectors) {
		int ldz = s->mmax + 1;
		double *work = s->d_Z + (size_t)s->nev_cap * ldz;
		int w2 = want < s->nev_cap ? want : s->nev_cap;
		k_tri_vectors<<<(w2 + 31) / 32, 32, 0, c->stream>>>(s->d_alpha, s->d_beta, n, w2, s->d_theta, s->d_Z, ldz,
								    work, 5 * ldz);
		k_tri_mgs<<<1, RED_THREADS, 0, c->stream>>>(s->d_Z, ldz, n, w2);
		for (int i = 0; i < w2; i++)
			CUDA_TRY(cudaMemcpyAsync(s->h_zlast + i, s->d_Z + (size_t)i * ldz + n - 1, sizeof(double),
						 cudaMemcpyDeviceToHost, c->stream));
	}
	CUDA_TRY(cudaMemcpyAsync(s->h_theta, s->d_theta, want * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	CUDA_TRY(cudaStreamSynchronize(c->stream));
	CUDA_TRY(cudaGetLastError());
	return JN_OK;
}

extern "C" jn_status jn_lanczos(jn_ctx *c, const jn_lanczos_options *opt, jn_lanczos_result *res)
{
	if (!c || !opt || !res) return jn_fail(JN_ERR_INVALID, "null argument");
	const int64_t D = c->plan.dim;
	int m = opt->max_iterations > 0 ? opt->max_iterations : 200;
	if ((int64_t)m > D) m = (int)D;               /* lanczos.c:181-185 */
	int nev = opt->num_eigenvalues > 0 ? opt->num_eigenvalues : 10;
	if (nev > JN_MAX_REPORTED) nev = JN_MAX_REPORTED;
	if (nev > m) nev = m;
	const int reference_mode = opt->mode == JN_LANCZOS_REFERENCE;
	const int check_every = opt->check_every > 0 ? opt->check_every : 1;
	jn_status st = ensure_state(c, m, nev < 1 ? 1 : nev);
	if (st) return st;
	struct jn_lanczos_state *s = c->lz;
	s->nev = nev;
	s->have_ritz = 0;
	cudaStream_t q = c->stream;
	const int g = grid_for(D);
	double *V = s->d_V;

	/* v_0 */
	if (opt->start_vector) {
		CUDA_TRY(cudaMemcpyAsync(s->d_w, opt->start_vector, D * sizeof(double), cudaMemcpyHostToDevice, q));
		dot_dev(c, s->d_w, s->d_w, s->d_scalar);
		k_normalize<<<g, 256, 0, q>>>(V, s->d_w, s->d_scalar, NULL, D);
	} else {
		CUDA_TRY(cudaMemsetAsync(V, 0, D * sizeof(double), q));
		double one = 1.0;
		CUDA_TRY(cudaMemcpyAsync(V, &one, sizeof(double), cudaMemcpyHostToDevice, q));
		CUDA_TRY(cudaStreamSynchronize(q));
	}

	double prev = 0.0;
	int k, converged = 0;
	/* the eigenvector criterion keeps the previous step's vector (and the current one after it) */
	const int by_vector = reference_mode && opt->criterion == JN_CONVERGE_EIGENVECTORS;
	std::vector<double> zbuf(by_vector ? 2 * (size_t)(m + 1) : 0, 0.0);
	double *zprev = zbuf.data();
	res->iterations = 0;
	res->iteration_seconds = res->refinement_seconds = 0.0;
	const double t_loop = seconds_now();
	for (k = 0; k < m; k++) {
		double *vk = V + (int64_t)k * D, *vk1 = V + (int64_t)(k + 1) * D;
		st = jn_launch_matvec(c, vk, s->d_w, 0, q);
		if (st) return st;
		dot_dev(c, vk, s->d_w, s->d_alpha + k);
		k_three_term<<<g, 256, 0, q>>>(s->d_w, vk, k ? V + (int64_t)(k - 1) * D : NULL, s->d_alpha + k,
					       k ? s->d_beta + k - 1 : NULL, D);
		if (!reference_mode) {
			cgs_pass(c, k + 1);
			cgs_pass(c, k + 1);
		}
		dot_dev(c, s->d_w, s->d_w, s->d_scalar);
		k_normalize<<<g, 256, 0, q>>>(vk1, s->d_w, s->d_scalar, s->d_beta + k, D);
		if (reference_mode && k > 2) {
			/* MGS of v_{k+1} against v_0..v_{k-3}, no renormalisation (vector.c:461-476) */
			for (int j = 0; j + 2 < k; j++) {
				dot_dev(c, vk1, V + (int64_t)j * D, s->d_scalar + 1);
				k_axpy_neg<<<g, 256, 0, q>>>(vk1, V + (int64_t)j * D, s->d_scalar + 1, D);
			}
		}
		CUDA_TRY(cudaGetLastError());
		const int n = k + 1;
		if ((n % check_every) && n < m) continue;
		CUDA_TRY(cudaMemcpyAsync(s->h_alpha, s->d_alpha, n * sizeof(double), cudaMemcpyDeviceToHost, q));
		CUDA_TRY(cudaMemcpyAsync(s->h_beta, s->d_beta, n * sizeof(double), cudaMemcpyDeviceToHost, q));
		if (reference_mode) {
			st = tri_eig(c, n, 1, by_vector);
			if (st) return st;
			double diff;
			if (by_vector) {
				/* the lowest eigenvector of T_n against the previous step's (lanczos.c:210-215, 276-287) */
				CUDA_TRY(cudaMemcpy(zprev + (m + 1), s->d_Z, n * sizeof(double), cudaMemcpyDeviceToHost));
				double *z = zprev + (m + 1);
				if (z[0] < 0.0)
					for (int i = 0; i < n; i++) z[i] = -z[i];
				double d2 = z[n - 1] * z[n - 1];
				for (int i = 0; i + 1 < n; i++) d2 += (z[i] - zprev[i]) * (z[i] - zprev[i]);
				diff = sqrt(d2);
				memcpy(zprev, z, n * sizeof(double));
			} else {
				diff = fabs(s->h_theta[0] - prev);
			}
			prev = s->h_theta[0];
			if (opt->verbose)
				printf("Lanczos iteration %d: lowest Ritz value %.17lg, difference %lg\n", n, s->h_theta[0], diff);
			if (diff < opt->tolerance) { converged = 1; k++; break; }
		} else {
			int want = nev < n ? nev : n;
			st = tri_eig(c, n, want + (want < n ? 1 : 0), 1);
			if (st) return st;
			int ok = n >= nev;
			double beta = s->h_beta[n - 1];
			for (int i = 0; i < want && ok; i++) {
				double r = fabs(beta * s->h_zlast[i]);
				double gap = 1e300;
				if (i > 0) gap = fmin(gap, s->h_theta[i] - s->h_theta[i - 1]);
				if (i + 1 < want + (want < n ? 1 : 0)) gap = fmin(gap, s->h_theta[i + 1] - s->h_theta[i]);
				double bound = fmin(r, r * r / fmax(gap, 1e-300));
				if (!(bound < opt->tolerance)) ok = 0;
			}
			if (opt->verbose)
				printf("Lanczos iteration %d: lowest Ritz value %.17lg, beta %lg\n", n, s->h_theta[0], beta);
			if (ok || beta == 0.0) { converged = 1; k++; break; }
		}
	}
	s->k = k;
	res->iterations = k;
	res->converged = converged;
	const double t_final = seconds_now();      /* the loop ends on a convergence check, which synchronises */
	res->iteration_seconds = t_final - t_loop;
	/* final decomposition of T_k: all Ritz values, vectors of the lowest nev */
	CUDA_TRY(cudaMemcpyAsync(s->h_alpha, s->d_alpha, k * sizeof(double), cudaMemcpyDeviceToHost, q));
	CUDA_TRY(cudaMemcpyAsync(s->h_beta, s->d_beta, k * sizeof(double), cudaMemcpyDeviceToHost, q));
	int want = nev < k ? nev : k;
	st = tri_eig(c, k, k, 0);
	if (st) return st;
	res->num_ritz_values = k;
	st = tri_eig(c, k, want, 1);
	if (st) return st;
	/* Ritz vectors x_i = sum_j z_i[j] v_j and their FP64 refinement */
	int ldz = s->mmax + 1;
	for (int i = 0; i < want; i++)
		k_gemv_n<<<g, 256, 0, q>>>(V, D, k, s->d_Z + (size_t)i * ldz, s->d_ritz + (size_t)i * D);
	s->have_ritz = 1;
	/* the refinement's products are FP64-grade whatever the iteration's precision */
	const int prec0 = c->precision, engine0 = c->engine;
	c->precision = 64;
	c->engine = c->engine_of[0];
	for (int i = 0; i < want; i++) {
		double *xi = s->d_ritz + (size_t)i * D;
		st = jn_launch_matvec(c, xi, s->d_w, 0, q);
		if (st) { c->precision = prec0; c->engine = engine0; return st; }
		dot_dev(c, xi, s->d_w, s->d_scalar + 0);
		dot_dev(c, xi, xi, s->d_scalar + 1);
		double h2[2];
		CUDA_TRY(cudaMemcpyAsync(h2, s->d_scalar, 2 * sizeof(double), cudaMemcpyDeviceToHost, q));
		CUDA_TRY(cudaStreamSynchronize(q));
		double rq = h2[0] / h2[1];
		s->h_rq[i] = rq;
		/* r = H x - rq x */
		CUDA_TRY(cudaMemcpyAsync(s->d_scalar + 2, &rq, sizeof(double), cudaMemcpyHostToDevice, q));
		k_axpy_neg<<<g, 256, 0, q>>>(s->d_w, xi, s->d_scalar + 2, D);
		dot_dev(c, s->d_w, s->d_w, s->d_scalar + 3);
		double r2;
		CUDA_TRY(cudaMemcpyAsync(&r2, s->d_scalar + 3, sizeof(double), cudaMemcpyDeviceToHost, q));
		CUDA_TRY(cudaStreamSynchronize(q));
		s->h_res[i] = sqrt(r2 / h2[1]);
	}
	c->precision = prec0;
	c->engine = engine0;
	CUDA_TRY(cudaGetLastError());
	res->refinement_seconds = seconds_now() - t_final;
	res->num_eigenvalues = want;
	for (int i = 0; i < want && i < JN_MAX_REPORTED; i++) {
		res->eigenvalues[i] = s->h_rq[i];
		res->ritz_values[i] = s->h_theta[i];
		res->residual_norms[i] = s->h_res[i];
	}
	return converged ? JN_OK : (opt->mode == JN_LANCZOS_REFERENCE ? JN_OK : jn_fail(JN_ERR_NOT_CONVERGED,
		"Lanczos did not converge in %d iterations", k));
}

extern "C" jn_status jn_lanczos_ritz_values(jn_ctx *c, double *out, int capacity, int *count)
{
	if (!c || !c->lz || !out) return jn_fail(JN_ERR_INVALID, "no Lanczos solve on this context");
	struct jn_lanczos_state *s = c->lz;
	jn_status st = tri_eig(c, s->k, s->k, 0);
	if (st) return st;
	int n = s->k < capacity ? s->k : capacity;
	memcpy(out, s->h_theta, n * sizeof(double));
	if (count) *count = s->k;
	return JN_OK;
}

extern "C" jn_status jn_lanczos_eigenvector(jn_ctx *c, int i, double *host_out)
{
	if (!c || !c->lz || !c->lz->have_ritz || !host_out) return jn_fail(JN_ERR_INVALID, "no Ritz vectors on this context");
	struct jn_lanczos_state *s = c->lz;
	if (i < 0 || i >= s->nev || i >= s->k) return jn_fail(JN_ERR_INVALID, "eigenvector index out of range");
	CUDA_TRY(cudaMemcpyAsync(host_out, s->d_ritz + (size_t)i * s->D, s->D * sizeof(double), cudaMemcpyDeviceToHost,
				 c->stream));
	CUDA_TRY(cudaStreamSynchronize(c->stream));
	return JN_OK;
}

extern "C" jn_status jn_lanczos_save_eigenvectors(jn_ctx *c, const char *directory, int count)
{
	if (!c || !directory) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_plan_t *p = &c->plan;
	double *buf = (double *)malloc((p->dim ? p->dim : 1) * sizeof(double));
	jn_status st = JN_OK;
	mkdir(directory, 0755);
	for (int i = 0; i < count && !st; i++) {
		st = jn_lanczos_eigenvector(c, i, buf);
		if (st) break;
		char dir[8192];
		snprintf(dir, sizeof dir, "%s/eigenvector_%d", directory, i + 1);   /* bacchus.c:68-87 */
		mkdir(dir, 0755);
		for (int b = 0; b < p->nblocks && !st; b++) {
			char path[8300];
			snprintf(path, sizeof path, "%s/vec_%d", dir, b + 1);            /* vector.c:538-555 */
			FILE *f = fopen(path, "wb");
			if (!f) { st = jn_fail(JN_ERR_IO, "Could not open %s", path); break; }
			size_t n = (size_t)(p->blocks[b].Np * p->blocks[b].Nn);
			if (fwrite(buf + p->blocks[b].offset, sizeof(double), n, f) != n) st = jn_fail(JN_ERR_IO, "write %s", path);
			fclose(f);
		}
	}
	free(buf);
	return st;
}

extern "C" void jn_print_eigensystem(const double *ev, int n)
{
	printf("eigensystem:\n{\n");
	printf("\tnum_eigenvalues = %d;\n", n);
	printf("\teigenvalues = ( ");
	for (int i = 0; i < n; i++) printf("%.17lg%s ", ev[i], i == n - 1 ? "" : ",");
	printf(");\n}\n");
	fflush(stdout);
}
