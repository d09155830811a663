/*
 * jn_batch.cu — many Hamiltonians of one basis solved together: batched,
 * mixed-precision Lanczos with a captured CUDA graph per step.
 *
 * The instances share the context's index lists and differ only in their
 * matrix elements (H(c) = H0 + sum_i c_i H_i keeps the sparsity of the
 * lists).  Every kernel runs all instances at once, instance = blockIdx.y;
 * the step index k is read from device memory, so one captured graph of a
 * Lanczos step is replayed for every step.  An instance that has converged
 * is frozen (its kernels return at once) while the others go on.
 *
 * Arithmetic (precision 32): the products use FP32 copies of the matrix
 * elements and of v_k with exact fixed-point sums (the block-tile engine);
 * the three-term recurrence, full reorthogonalisation (classical
 * Gram-Schmidt, twice), the tridiagonal eigenproblem and the final
 * refinement are FP64.  Refinement: the lowest r Ritz vectors X of each
 * instance are multiplied by the FP64 Hamiltonian, and the r x r pencil
 * (X^T H X, X^T X) is solved in FP64 (Rayleigh-Ritz), which removes the
 * error of the FP32 operator to second order.  Precision 64 runs the same
 * solver with FP64 products.
 *
 * Reference: one instance of this is Bacchus' Lanczos
 * (src/Bacchus/lanczos/lanczos.c:74-253) with full reorthogonalisation.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jn_internal.h"
#include "jn_tridiag.cuh"

#include <functional>

#define BT 256          /* threads of the vector kernels */
#define BNB 16          /* reduction CTAs per instance */

/* ------------------------------------------------------------------ */
/* batched vector kernels (instance = blockIdx.y, k = *d_k)            */
/* ------------------------------------------------------------------ */
#define SKIP_INACTIVE() \
	const int inst = blockIdx.y; \
	if (active && !active[inst]) return
/* the dimension of an instance: D (the vectors' stride) unless each instance has its own */
#define DIM_OF(inst) (dims ? dims[inst] : D)

__device__ __forceinline__ void slice(int64_t D, int64_t *i0, int64_t *i1)
{
	const int64_t chunk = (D + gridDim.x - 1) / gridDim.x;
	*i0 = (int64_t)blockIdx.x * chunk;
	*i1 = min(D, *i0 + chunk);
}

/* part[inst][blk] = x . y over this CTA's slice; x = X + inst*x_ld (+ k*D when xk) */
__global__ void __launch_bounds__(BT) kb_dot(const double *__restrict__ X, int64_t x_ld, int xk,
					      const double *__restrict__ Y, int64_t y_ld, int yk, const int *__restrict__ d_k,
					      int64_t D, const int64_t *__restrict__ dims, double *__restrict__ part,
					      const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int64_t n = DIM_OF(inst);
	__shared__ double sh[BT];
	const int k = *d_k;
	const double *x = X + inst * x_ld + (xk ? (int64_t)k * D : 0);
	const double *y = Y + inst * y_ld + (yk ? (int64_t)k * D : 0);
	int64_t i0, i1;
	slice(n, &i0, &i1);
	double s = 0.0;
	for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) s = fma(x[i], y[i], s);
	s = jn_block_sum(s, sh);
	if (threadIdx.x == 0) part[(int64_t)inst * gridDim.x + blockIdx.x] = s;
}

/* out[inst*out_ld + (k when outk)] = sum of the CTA partials in order */
__global__ void kb_finish_dot(const double *__restrict__ part, int nblk, double *__restrict__ out, int64_t out_ld,
			      int outk, const int *__restrict__ d_k, const int *__restrict__ active)
{
	SKIP_INACTIVE();
	if (threadIdx.x) return;
	double s = 0.0;
	for (int b = 0; b < nblk; b++) s += part[(int64_t)inst * nblk + b];
	out[inst * out_ld + (outk ? *d_k : 0)] = s;
}

/* w -= alpha_k v_k + beta_{k-1} v_{k-1} */
__global__ void kb_three_term(double *__restrict__ W, const double *__restrict__ V, int64_t ldV,
			      const double *__restrict__ alpha, const double *__restrict__ beta, int64_t ldab,
			      const int *__restrict__ d_k, int64_t D, const int64_t *__restrict__ dims,
			      const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int64_t n = DIM_OF(inst);
	const int k = *d_k;
	const double a = alpha[inst * ldab + k], b = k > 0 ? beta[inst * ldab + k - 1] : 0.0;
	const double *v = V + inst * ldV + (int64_t)k * D, *u = k > 0 ? v - D : v;
	double *w = W + inst * D;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		double r = w[i] - a * v[i];
		if (k > 0) r -= b * u[i];
		w[i] = r;
	}
}

/* part[inst][blk][j] = V_j . w over the slice, j <= k: warp j % 8 owns
 * vector j and reduces it with shuffles in a fixed order, so no CTA-wide
 * barrier is taken per vector */
__global__ void __launch_bounds__(BT) kb_gemv_t(const double *__restrict__ V, int64_t ldV, const double *__restrict__ W,
						 const int *__restrict__ d_k, int64_t D, const int64_t *__restrict__ dims,
						 double *__restrict__ part, int ncol, const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int nvec = *d_k + 1;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
	const double *w = W + inst * D;
	int64_t i0, i1;
	slice(DIM_OF(inst), &i0, &i1);
	for (int j = warp; j < nvec; j += nwarps) {
		const double *v = V + inst * ldV + (int64_t)j * D;
		double s = 0.0;
		for (int64_t i = i0 + lane; i < i1; i += 32) s = fma(v[i], w[i], s);
		for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
		if (lane == 0) part[((int64_t)inst * gridDim.x + blockIdx.x) * ncol + j] = s;
	}
}

__global__ void kb_finish(const double *__restrict__ part, int nblk, int ncol, const int *__restrict__ d_k,
			  double *__restrict__ h, const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j > *d_k) return;
	double s = 0.0;
	for (int b = 0; b < nblk; b++) s += part[((int64_t)inst * nblk + b) * ncol + j];
	h[(int64_t)inst * ncol + j] = s;
}

/* w -= sum_{j<=k} V_j h_j */
__global__ void kb_gemv_n_sub(const double *__restrict__ V, int64_t ldV, const double *__restrict__ h, int ncol,
			      const int *__restrict__ d_k, int64_t D, const int64_t *__restrict__ dims, double *__restrict__ W,
			      const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int64_t n = DIM_OF(inst);
	const int nvec = *d_k + 1;
	const double *hh = h + (int64_t)inst * ncol, *v = V + inst * ldV;
	double *w = W + inst * D;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int j = 0; j < nvec; j++) s = fma(v[(int64_t)j * D + i], hh[j], s);
		w[i] -= s;
	}
}

/* v_{k+1} = w / |w|, beta_k = |w| (|w|^2 in nrm2[inst]) */
__global__ void kb_normalize(double *__restrict__ V, int64_t ldV, const double *__restrict__ W,
			     const double *__restrict__ nrm2, double *__restrict__ beta, int64_t ldab,
			     const int *__restrict__ d_k, int64_t D, const int64_t *__restrict__ dims,
			     const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int64_t n = DIM_OF(inst);
	const int k = *d_k;
	const double b = sqrt(nrm2[inst]);
	if (blockIdx.x == 0 && threadIdx.x == 0) beta[inst * ldab + k] = b;
	const double inv = b > 0.0 ? 1.0 / b : 0.0;
	double *v = V + inst * ldV + (int64_t)(k + 1) * D;
	const double *w = W + inst * D;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		v[i] = w[i] * inv;
}

/* v_0 /= |v_0| (|v_0|^2 in nrm2[inst]) */
__global__ void kb_scale_start(double *__restrict__ V, int64_t ldV, const double *__restrict__ nrm2, int64_t D,
			       const int64_t *__restrict__ dims)
{
	const int inst = blockIdx.y;
	const int64_t n = DIM_OF(inst);
	const double inv = 1.0 / sqrt(nrm2[inst]);
	double *v = V + inst * ldV;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		v[i] *= inv;
}

__global__ void kb_advance(int *d_k) { if (threadIdx.x == 0 && blockIdx.x == 0) *d_k += 1; }

/* ------------------------------------------------------------------ */
/* batched tridiagonal work (n per instance)                            */
/* ------------------------------------------------------------------ */
/* one warp per eigenvalue i = blockIdx.x (multisection) */
__global__ void kb_tri_bisect(const double *__restrict__ alpha, const double *__restrict__ beta, int64_t ldab,
			      const int *__restrict__ n_arr, int want, double *__restrict__ theta, int ldt,
			      const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int i = blockIdx.x;
	const int n = n_arr[inst];
	if (i >= want || i >= n) return;
	const double v = jn_tri_multisect_warp(alpha + inst * ldab, beta + inst * ldab, n, i);
	if (threadIdx.x == 0) theta[(int64_t)inst * ldt + i] = v;
}

__global__ void kb_tri_vectors(const double *__restrict__ alpha, const double *__restrict__ beta, int64_t ldab,
			       const int *__restrict__ n_arr, int want, const double *__restrict__ theta, int ldt,
			       double *__restrict__ Z, int ldz, double *__restrict__ work, double *__restrict__ zlast,
			       const int *__restrict__ active)
{
	SKIP_INACTIVE();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int n = n_arr[inst];
	if (i >= want || i >= n) return;
	double *z = Z + ((int64_t)inst * want + i) * ldz;
	jn_tri_vector_one(alpha + inst * ldab, beta + inst * ldab, n, theta[(int64_t)inst * ldt + i], z,
			  work + ((int64_t)inst * want + i) * 5 * ldz);
	if (zlast) zlast[(int64_t)inst * ldt + i] = z[n - 1];
}

__global__ void kb_tri_mgs(double *__restrict__ Z, int ldz, const int *__restrict__ n_arr, int want,
			   const int *__restrict__ active)
{
	SKIP_INACTIVE();
	__shared__ double sh[BT];
	const int n = n_arr[inst];
	jn_tri_mgs(Z + (int64_t)inst * want * ldz, ldz, n, want < n ? want : n, sh);
}

/* converged[inst] = every one of the nev lowest Ritz values has
 * min(r, r^2/gap) < tol, r = |beta_{n-1} z_i[n-1]| (the criterion of the
 * single solve's full mode); theta holds nev+1 values when n > nev */
__global__ void kb_converged(const double *__restrict__ theta, const double *__restrict__ zlast, int ldt,
			     const double *__restrict__ beta, int64_t ldab, const int *__restrict__ n_arr, int nev,
			     double tol, int *__restrict__ flag, const int *__restrict__ active, int B)
{
	const int inst = blockIdx.x * blockDim.x + threadIdx.x;
	if (inst >= B) return;
	if (active && !active[inst]) { flag[inst] = 0; return; }
	const int n = n_arr[inst];
	const double b = beta[inst * ldab + n - 1];
	int ok = n >= nev;
	const int have = nev < n ? nev + 1 : n;
	const double *th = theta + (int64_t)inst * ldt;
	for (int i = 0; i < nev && i < n && ok; i++) {
		const double r = fabs(b * zlast[(int64_t)inst * ldt + i]);
		double gap = 1e300;
		if (i > 0) gap = fmin(gap, th[i] - th[i - 1]);
		if (i + 1 < have) gap = fmin(gap, th[i + 1] - th[i]);
		const double bound = fmin(r, r * r / fmax(gap, 1e-300));
		if (!(bound < tol)) ok = 0;
	}
	flag[inst] = ok || b == 0.0;
}

/* X[inst][j] = sum_{l < n} V[inst][l] Z[inst][j][l], j < r */
__global__ void kb_ritz(const double *__restrict__ V, int64_t ldV, const double *__restrict__ Z, int ldz,
			const int *__restrict__ n_arr, int r, int64_t D, const int64_t *__restrict__ dims,
			double *__restrict__ X)
{
	const int inst = blockIdx.y;
	const int n = n_arr[inst];
	const int64_t dim = DIM_OF(inst);
	const double *v = V + inst * ldV;
	const double *z = Z + (int64_t)inst * r * ldz;
	double *x = X + (int64_t)inst * r * D;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
		for (int j = 0; j < r; j++) {
			double s = 0.0;
			if (j < n)
				for (int l = 0; l < n; l++) s = fma(v[(int64_t)l * D + i], z[(int64_t)j * ldz + l], s);
			x[(int64_t)j * D + i] = s;
		}
}

/* G[inst][i][j] = A[inst][i] . Bm[inst][j]; one CTA per (i, j, inst) */
__global__ void __launch_bounds__(BT) kb_gram(const double *__restrict__ A, const double *__restrict__ Bm, int r,
					       int64_t D, const int64_t *__restrict__ dims, double *__restrict__ G)
{
	__shared__ double sh[BT];
	const int inst = blockIdx.y, i = blockIdx.x / r, j = blockIdx.x % r;
	const int64_t n = DIM_OF(inst);
	const double *a = A + ((int64_t)inst * r + i) * D, *b = Bm + ((int64_t)inst * r + j) * D;
	double s = 0.0;
	for (int64_t t = threadIdx.x; t < n; t += blockDim.x) s = fma(a[t], b[t], s);
	s = jn_block_sum(s, sh);
	if (threadIdx.x == 0) G[((int64_t)inst * r + i) * r + j] = s;
}

/* out[inst][e] = sum_j X[inst][j] C[inst][e][j], e < nv: the refined vectors */
__global__ void kb_combine(const double *__restrict__ X, const double *__restrict__ C, int r, int nv, int64_t D,
			   const int64_t *__restrict__ dims, double *__restrict__ out)
{
	const int inst = blockIdx.y;
	const int64_t n = DIM_OF(inst);
	const double *x = X + (int64_t)inst * r * D;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		for (int e = 0; e < nv; e++) {
			const double *c = C + ((int64_t)inst * r + e) * r;
			double s = 0.0;
			for (int j = 0; j < r; j++) s = fma(x[(int64_t)j * D + i], c[j], s);
			out[((int64_t)inst * nv + e) * D + i] = s;
		}
}

/* ------------------------------------------------------------------ */
/* host: the r x r generalized symmetric eigenproblem A c = l G c       */
/* ------------------------------------------------------------------ */
/* Cholesky G = L L^T in place (lower); returns 0 or -1 when not positive */
static int cholesky(double *G, int r)
{
	for (int j = 0; j < r; j++) {
		double d = G[j * r + j];
		for (int k = 0; k < j; k++) d -= G[j * r + k] * G[j * r + k];
		if (!(d > 0)) return -1;
		d = sqrt(d);
		G[j * r + j] = d;
		for (int i = j + 1; i < r; i++) {
			double s = G[i * r + j];
			for (int k = 0; k < j; k++) s -= G[i * r + k] * G[j * r + k];
			G[i * r + j] = s / d;
		}
	}
	return 0;
}

/* cyclic Jacobi: S (r x r symmetric) -> eigenvalues w (ascending) and eigenvectors Q (columns) */
static void jacobi_eigen(double *S, int r, double *w, double *Q)
{
	for (int i = 0; i < r * r; i++) Q[i] = 0.0;
	for (int i = 0; i < r; i++) Q[i * r + i] = 1.0;
	for (int sweep = 0; sweep < 100; sweep++) {
		double off = 0.0;
		for (int p = 0; p < r; p++)
			for (int q = p + 1; q < r; q++) off += S[p * r + q] * S[p * r + q];
		if (off < 1e-300) break;
		for (int p = 0; p < r; p++)
			for (int q = p + 1; q < r; q++) {
				const double apq = S[p * r + q];
				if (apq == 0.0) continue;
				const double theta = (S[q * r + q] - S[p * r + p]) / (2.0 * apq);
				const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
				const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
				for (int k = 0; k < r; k++) {
					const double skp = S[k * r + p], skq = S[k * r + q];
					S[k * r + p] = c * skp - s * skq;
					S[k * r + q] = s * skp + c * skq;
				}
				for (int k = 0; k < r; k++) {
					const double spk = S[p * r + k], sqk = S[q * r + k];
					S[p * r + k] = c * spk - s * sqk;
					S[q * r + k] = s * spk + c * sqk;
				}
				for (int k = 0; k < r; k++) {
					const double qkp = Q[k * r + p], qkq = Q[k * r + q];
					Q[k * r + p] = c * qkp - s * qkq;
					Q[k * r + q] = s * qkp + c * qkq;
				}
			}
	}
	/* sort ascending */
	for (int i = 0; i < r; i++) w[i] = S[i * r + i];
	for (int i = 0; i < r; i++) {
		int m = i;
		for (int j = i + 1; j < r; j++) if (w[j] < w[m]) m = j;
		if (m != i) {
			double t = w[i]; w[i] = w[m]; w[m] = t;
			for (int k = 0; k < r; k++) { t = Q[k * r + i]; Q[k * r + i] = Q[k * r + m]; Q[k * r + m] = t; }
		}
	}
}

/* refined values lam[0..r), residual norms res[] and the coefficients of
 * the refined vectors (row e of cv, row length ldc, when cv is not NULL),
 * from G1 = X^T X, G2 = X^T H X, G3 = (HX)^T HX */
static int rayleigh_ritz(const double *G1, const double *G2, const double *G3, int r, double *lam, double *res,
			 double *cv, int ldc)
{
	double *L = (double *)malloc(sizeof(double) * r * r), *S = (double *)malloc(sizeof(double) * r * r);
	double *Q = (double *)malloc(sizeof(double) * r * r), *T = (double *)malloc(sizeof(double) * r * r);
	double *c = (double *)malloc(sizeof(double) * r);
	memcpy(L, G1, sizeof(double) * r * r);
	int rc = cholesky(L, r);
	if (!rc) {
		/* T = L^-1 G2, S = T L^-T */
		for (int j = 0; j < r; j++)
			for (int i = 0; i < r; i++) {
				double s = G2[i * r + j];
				for (int k = 0; k < i; k++) s -= L[i * r + k] * T[k * r + j];
				T[i * r + j] = s / L[i * r + i];
			}
		for (int i = 0; i < r; i++)
			for (int j = 0; j < r; j++) {
				double s = T[i * r + j];
				for (int k = 0; k < j; k++) s -= S[i * r + k] * L[j * r + k];
				S[i * r + j] = s / L[j * r + j];
			}
		for (int i = 0; i < r; i++)
			for (int j = i + 1; j < r; j++) S[i * r + j] = S[j * r + i] = 0.5 * (S[i * r + j] + S[j * r + i]);
		jacobi_eigen(S, r, lam, Q);
		for (int e = 0; e < r; e++) {
			/* c = L^-T q_e */
			for (int i = r - 1; i >= 0; i--) {
				double s = Q[i * r + e];
				for (int k = i + 1; k < r; k++) s -= L[k * r + i] * c[k];
				c[i] = s / L[i * r + i];
			}
			double h2 = 0, hx = 0, xx = 0;
			for (int i = 0; i < r; i++)
				for (int j = 0; j < r; j++) {
					h2 += c[i] * G3[i * r + j] * c[j];
					hx += c[i] * G2[i * r + j] * c[j];
					xx += c[i] * G1[i * r + j] * c[j];
				}
			double r2 = h2 - 2.0 * lam[e] * hx + lam[e] * lam[e] * xx;
			res[e] = sqrt(fmax(r2, 0.0) / fmax(xx, 1e-300));
			if (cv) memcpy(cv + (size_t)e * ldc, c, sizeof(double) * r);
		}
	}
	free(L); free(S); free(Q); free(T); free(c);
	return rc;
}

/* ------------------------------------------------------------------ */
/* the solver                                                           */
/* ------------------------------------------------------------------ */
/* The instances of one batched solve, their layout and their products.
 * Instance i has dimension dims[i] <= Dp; its vectors are stored Dp apart. */
struct batch_job {
	int B;
	int64_t Dp;
	const int64_t *dims;
	/* W_i = H_i v_k for every active instance, in the solve's arithmetic (k read on the device) */
	std::function<jn_status(const double *V, int64_t ldV, const int *d_k, double *W, const int *d_active, cudaStream_t)>
		product;
	/* HX_i = H_i X_i in FP64-grade arithmetic for every instance (X_i = X + i ld); scratch: B x Dp */
	std::function<jn_status(const double *X, int64_t ld, double *HX, double *scratch, cudaStream_t)> product64;
	const double *const *start_vectors;     /* B entries, or NULL */
	double *const *eigenvectors;            /* B entries, or NULL */
	jn_batch_result **res;                  /* B results */
};

struct bstate {
	double *V, *W, *alpha, *beta, *part, *h, *scal, *theta, *zlast, *Z, *work, *X, *HX, *G, *C, *GS;
	int64_t *dims;
	int *k, *active, *flag, *narr;
};

static void bstate_free(struct bstate *s)
{
	void *p[] = { s->V, s->W, s->alpha, s->beta, s->part, s->h, s->scal, s->theta, s->zlast, s->Z, s->work, s->X,
		      s->HX, s->G, s->C, s->GS, s->dims, s->k, s->active, s->flag, s->narr };
	for (size_t i = 0; i < sizeof p / sizeof p[0]; i++) cudaFree(p[i]);
}

#define BALLOC(ptr, count)                                                                                    \
	do {                                                                                                  \
		if (!st && cudaMalloc((void **)&(ptr), (size_t)(count) * sizeof(*(ptr)) + 64) != cudaSuccess)   \
			st = jn_fail(JN_ERR_NOMEM, "batched Lanczos: device allocation of %s failed", #ptr);   \
	} while (0)

/* the shared options of a batched solve */
static jn_status batch_check_options(const jn_batch_options *o)
{
	if (o->precision != 32 && o->precision != 64) return jn_fail(JN_ERR_INVALID, "precision must be 32 or 64");
	if (o->num_eigenvectors < 0 || o->num_eigenvectors > (o->num_eigenvalues > 0 ? o->num_eigenvalues : 10) ||
	    o->num_eigenvectors > JN_MAX_REPORTED)
		return jn_fail(JN_ERR_INVALID, "num_eigenvectors must be in 0..num_eigenvalues");
	return JN_OK;
}

/* Lanczos with full reorthogonalisation for every instance of the job, one
 * captured graph per step; then the FP64 Rayleigh-Ritz refinement. */
static jn_status batch_solve(cudaStream_t q, const jn_batch_options *o, const batch_job &job)
{
	const int B = job.B;
	const int64_t Dp = job.Dp;
	int m = o->max_iterations > 0 ? o->max_iterations : 200;
	if (m > Dp) m = (int)Dp;
	int nev = o->num_eigenvalues > 0 ? o->num_eigenvalues : 10;
	if (nev > JN_MAX_REPORTED) nev = JN_MAX_REPORTED;
	if (nev > m) nev = m;
	const int extra = o->refine_extra >= 0 ? o->refine_extra : 4;
	int r = nev + extra;
	if (r > m) r = m;
	const int check_every = o->check_every > 0 ? o->check_every : 10;
	const int nvo = o->num_eigenvectors;
	const int want = nev + 1 < m ? nev + 1 : m;
	const int ldz = m + 1;
	const int ncol = m + 2;
	const int64_t ldV = (int64_t)(m + 1) * Dp, ldab = m + 1;
	/* an instance stops at the dimension of its Krylov space */
	int *lim = (int *)malloc(B * sizeof(int));
	for (int i = 0; i < B; i++) lim[i] = job.dims[i] < m ? (int)job.dims[i] : m;
	jn_status st = JN_OK;
	struct bstate s;
	memset(&s, 0, sizeof s);
	BALLOC(s.V, (size_t)B * ldV);
	BALLOC(s.W, (size_t)B * Dp);
	BALLOC(s.alpha, (size_t)B * ldab);
	BALLOC(s.beta, (size_t)B * ldab);
	BALLOC(s.part, (size_t)B * BNB * ncol);
	BALLOC(s.h, (size_t)B * ncol);
	BALLOC(s.scal, (size_t)B);
	BALLOC(s.theta, (size_t)B * (r + 1));
	BALLOC(s.zlast, (size_t)B * (r + 1));
	const int zrows = r > want ? r : want;  /* vectors per instance: r at the end, want in checks */
	BALLOC(s.Z, (size_t)B * zrows * ldz);
	BALLOC(s.work, (size_t)B * zrows * 5 * ldz);
	BALLOC(s.dims, B);
	BALLOC(s.k, 1);
	BALLOC(s.active, B);
	BALLOC(s.flag, B);
	BALLOC(s.narr, B);
	if (st) { bstate_free(&s); free(lim); return st; }
	if (cudaMemcpy(s.dims, job.dims, B * sizeof(int64_t), cudaMemcpyHostToDevice) != cudaSuccess)
		st = jn_fail(JN_ERR_CUDA, "upload of the instances' dimensions");

	/* start vectors: given, or one seeded pseudo-random vector of the instance's dimension */
	double *hv = (double *)malloc(Dp * sizeof(double));
	for (int i = 0; i < B && !st; i++) {
		const double *sv = job.start_vectors ? job.start_vectors[i] : NULL;
		if (!sv) {
			jn_default_start_vector(job.dims[i], hv);
			sv = hv;
		}
		if (cudaMemcpy(s.V + (size_t)i * ldV, sv, job.dims[i] * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "upload of start vectors");
	}
	free(hv);
	int *hact = (int *)malloc(B * sizeof(int)), *hn = (int *)malloc(B * sizeof(int)), *hflag = (int *)malloc(B * sizeof(int));
	for (int i = 0; i < B; i++) { hact[i] = 1; hn[i] = 0; }
	cudaGraphExec_t gexec = NULL;
	cudaGraph_t graph = NULL;
	int k = 0, nactive = B;
	const int vg = (int)((Dp + BT - 1) / BT < 64 ? (Dp + BT - 1) / BT : 64);
	const dim3 gv(vg > 0 ? vg : 1, B), gr(BNB, B), g1(1, B);
	const int64_t *dims = s.dims;
	if (!st) {
		cudaMemsetAsync(s.k, 0, sizeof(int), q);
		cudaMemcpyAsync(s.active, hact, B * sizeof(int), cudaMemcpyHostToDevice, q);
		/* v_0 normalised */
		kb_dot<<<gr, BT, 0, q>>>(s.V, ldV, 0, s.V, ldV, 0, s.k, Dp, dims, s.part, NULL);
		kb_finish_dot<<<g1, 32, 0, q>>>(s.part, BNB, s.scal, 1, 0, s.k, NULL);
		kb_scale_start<<<gv, BT, 0, q>>>(s.V, ldV, s.scal, Dp, dims);
		if (cudaGetLastError() != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "batched Lanczos start");
	}

	/* one Lanczos step for every active instance, k read on the device */
	auto step = [&](cudaStream_t qs) -> jn_status {
		jn_status e = job.product(s.V, ldV, s.k, s.W, s.active, qs);
		if (e) return e;
		kb_dot<<<gr, BT, 0, qs>>>(s.V, ldV, 1, s.W, Dp, 0, s.k, Dp, dims, s.part, s.active);
		kb_finish_dot<<<g1, 32, 0, qs>>>(s.part, BNB, s.alpha, ldab, 1, s.k, s.active);
		kb_three_term<<<gv, BT, 0, qs>>>(s.W, s.V, ldV, s.alpha, s.beta, ldab, s.k, Dp, dims, s.active);
		for (int pass = 0; pass < 2; pass++) {
			kb_gemv_t<<<gr, BT, 0, qs>>>(s.V, ldV, s.W, s.k, Dp, dims, s.part, ncol, s.active);
			kb_finish<<<dim3((ncol + 127) / 128, B), 128, 0, qs>>>(s.part, BNB, ncol, s.k, s.h, s.active);
			kb_gemv_n_sub<<<gv, BT, 0, qs>>>(s.V, ldV, s.h, ncol, s.k, Dp, dims, s.W, s.active);
		}
		kb_dot<<<gr, BT, 0, qs>>>(s.W, Dp, 0, s.W, Dp, 0, s.k, Dp, dims, s.part, s.active);
		kb_finish_dot<<<g1, 32, 0, qs>>>(s.part, BNB, s.scal, 1, 0, s.k, s.active);
		kb_normalize<<<gv, BT, 0, qs>>>(s.V, ldV, s.W, s.scal, s.beta, ldab, s.k, Dp, dims, s.active);
		kb_advance<<<1, 32, 0, qs>>>(s.k);
		return cudaGetLastError() == cudaSuccess ? JN_OK : jn_fail(JN_ERR_CUDA, "batched Lanczos step launch");
	};

	if (!st && o->use_graph) {
		if (cudaStreamBeginCapture(q, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "stream capture");
		jn_status e = st ? st : step(q);
		cudaError_t ce = cudaStreamEndCapture(q, &graph);
		if (!st && (e || ce != cudaSuccess)) st = e ? e : jn_fail(JN_ERR_CUDA, "end capture: %s", cudaGetErrorString(ce));
		if (!st && cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "graph instantiation");
	}

	while (!st && nactive > 0 && k < m) {
		if (gexec) {
			if (cudaGraphLaunch(gexec, q) != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "graph launch");
		} else {
			st = step(q);
		}
		k++;
		if (st) break;
		int at_limit = 0;
		for (int i = 0; i < B; i++) at_limit |= hact[i] && k >= lim[i];
		if (k % check_every && k < m && !at_limit) continue;
		/* convergence of every active instance at n = k */
		for (int i = 0; i < B; i++) hn[i] = hact[i] ? k : hn[i];
		cudaMemcpyAsync(s.narr, hn, B * sizeof(int), cudaMemcpyHostToDevice, q);
		const int wk = want < k ? want : k;
		kb_tri_bisect<<<dim3(wk, B), 32, 0, q>>>(s.alpha, s.beta, ldab, s.narr, wk, s.theta, r + 1, s.active);
		kb_tri_vectors<<<dim3((wk + 31) / 32, B), 32, 0, q>>>(s.alpha, s.beta, ldab, s.narr, wk, s.theta, r + 1, s.Z,
									ldz, s.work, s.zlast, s.active);
		kb_converged<<<(B + 127) / 128, 128, 0, q>>>(s.theta, s.zlast, r + 1, s.beta, ldab, s.narr, nev, o->tolerance,
							     s.flag, s.active, B);
		if (cudaMemcpyAsync(hflag, s.flag, B * sizeof(int), cudaMemcpyDeviceToHost, q) != cudaSuccess ||
		    cudaStreamSynchronize(q) != cudaSuccess) {
			st = jn_fail(JN_ERR_CUDA, "convergence check: %s", cudaGetErrorString(cudaGetLastError()));
			break;
		}
		for (int i = 0; i < B; i++)
			if (hact[i] && (hflag[i] || k >= lim[i])) {
				hact[i] = 0;
				hn[i] = k;
				job.res[i]->converged = hflag[i];
				job.res[i]->iterations = k;
				nactive--;
			}
		cudaMemcpyAsync(s.active, hact, B * sizeof(int), cudaMemcpyHostToDevice, q);
	}
	if (gexec) cudaGraphExecDestroy(gexec);
	if (graph) cudaGraphDestroy(graph);

	/* Ritz vectors of the final T of each instance, FP64 products, Rayleigh-Ritz */
	if (!st) {
		BALLOC(s.X, (size_t)B * r * Dp);
		BALLOC(s.HX, (size_t)B * r * Dp);
		BALLOC(s.G, (size_t)B * 3 * r * r);
		BALLOC(s.C, (size_t)B * r * r);
		if (nvo) BALLOC(s.GS, (size_t)B * nvo * Dp);
	}
	double *hG = NULL;
	if (!st) {
		for (int i = 0; i < B; i++) hact[i] = 1;
		cudaMemcpyAsync(s.narr, hn, B * sizeof(int), cudaMemcpyHostToDevice, q);
		cudaMemcpyAsync(s.active, hact, B * sizeof(int), cudaMemcpyHostToDevice, q);
		kb_tri_bisect<<<dim3(r, B), 32, 0, q>>>(s.alpha, s.beta, ldab, s.narr, r, s.theta, r + 1, NULL);
		kb_tri_vectors<<<dim3((r + 31) / 32, B), 32, 0, q>>>(s.alpha, s.beta, ldab, s.narr, r, s.theta, r + 1, s.Z, ldz,
								     s.work, NULL, NULL);
		kb_tri_mgs<<<g1, BT, 0, q>>>(s.Z, ldz, s.narr, r, NULL);
		kb_ritz<<<gv, BT, 0, q>>>(s.V, ldV, s.Z, ldz, s.narr, r, Dp, dims, s.X);
		/* H X in FP64-grade arithmetic, one batched product per Ritz index */
		for (int j = 0; j < r && !st; j++)
			st = job.product64(s.X + (size_t)j * Dp, (int64_t)r * Dp, s.HX + (size_t)j * Dp, s.W, q);
	}
	if (!st) {
		kb_gram<<<dim3(r * r, B), BT, 0, q>>>(s.X, s.X, r, Dp, dims, s.G);
		kb_gram<<<dim3(r * r, B), BT, 0, q>>>(s.X, s.HX, r, Dp, dims, s.G + (size_t)B * r * r);
		kb_gram<<<dim3(r * r, B), BT, 0, q>>>(s.HX, s.HX, r, Dp, dims, s.G + (size_t)2 * B * r * r);
		hG = (double *)malloc(sizeof(double) * 3 * B * r * r);
		double *hth = (double *)malloc(sizeof(double) * B * (r + 1));
		if (cudaMemcpyAsync(hG, s.G, sizeof(double) * 3 * B * r * r, cudaMemcpyDeviceToHost, q) != cudaSuccess ||
		    cudaMemcpyAsync(hth, s.theta, sizeof(double) * B * (r + 1), cudaMemcpyDeviceToHost, q) != cudaSuccess ||
		    cudaStreamSynchronize(q) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "refinement: %s", cudaGetErrorString(cudaGetLastError()));
		double *hC = (double *)calloc((size_t)B * r * r, sizeof(double));
		double *lam = (double *)malloc(sizeof(double) * r), *rn = (double *)malloc(sizeof(double) * r);
		for (int i = 0; i < B && !st; i++) {
			const int ri = hn[i] < r ? hn[i] : r;
			double *G1 = (double *)malloc(sizeof(double) * ri * ri), *G2 = (double *)malloc(sizeof(double) * ri * ri),
			       *G3 = (double *)malloc(sizeof(double) * ri * ri);
			for (int a = 0; a < ri; a++)
				for (int b2 = 0; b2 < ri; b2++) {
					G1[a * ri + b2] = hG[((size_t)i * r + a) * r + b2];
					G2[a * ri + b2] = 0.5 * (hG[(size_t)B * r * r + ((size_t)i * r + a) * r + b2] +
								 hG[(size_t)B * r * r + ((size_t)i * r + b2) * r + a]);
					G3[a * ri + b2] = hG[(size_t)2 * B * r * r + ((size_t)i * r + a) * r + b2];
				}
			if (rayleigh_ritz(G1, G2, G3, ri, lam, rn, hC + (size_t)i * r * r, r))
				st = jn_fail(JN_ERR_NOT_CONVERGED, "instance %d: Ritz vectors are not independent", i);
			jn_batch_result *R = job.res[i];
			R->num_eigenvalues = nev < ri ? nev : ri;
			for (int e = 0; e < R->num_eigenvalues; e++) {
				R->eigenvalues[e] = lam[e];
				R->residual_norms[e] = rn[e];
				R->ritz_values[e] = hth[(size_t)i * (r + 1) + e];
			}
			free(G1); free(G2); free(G3);
		}
		if (!st && nvo) {
			cudaMemcpyAsync(s.C, hC, sizeof(double) * B * r * r, cudaMemcpyHostToDevice, q);
			kb_combine<<<gv, BT, 0, q>>>(s.X, s.C, r, nvo, Dp, dims, s.GS);
			for (int i = 0; i < B && !st; i++)
				for (int e = 0; e < nvo && !st && job.eigenvectors && job.eigenvectors[i]; e++)
					if (cudaMemcpyAsync(job.eigenvectors[i] + (size_t)e * job.dims[i], s.GS + ((size_t)i * nvo + e) * Dp,
							    (size_t)job.dims[i] * sizeof(double), cudaMemcpyDeviceToHost, q) != cudaSuccess)
						st = jn_fail(JN_ERR_CUDA, "eigenvector copy");
			if (!st && cudaStreamSynchronize(q) != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "eigenvector copy");
		}
		free(hC); free(lam); free(rn); free(hth);
	}
	free(hG);
	free(hact); free(hn); free(hflag); free(lim);
	bstate_free(&s);
	if (!st && cudaGetLastError() != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "batched Lanczos");
	return st;
}

extern "C" jn_status jn_lanczos_batch(jn_ctx *c, const jn_batch_options *o, jn_batch_result *res)
{
	if (!c || !o || !res || !o->matrix_elements) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_plan_t *p = &c->plan;
	const int B = o->num_instances;
	const int64_t D = p->dim, nme = p->n_me;
	if (B < 1 || B > 4096) return jn_fail(JN_ERR_INVALID, "num_instances must be in 1..4096");
	if (D < 1) return jn_fail(JN_ERR_INVALID, "empty basis");
	if (p->btiles_off)
		return jn_fail(JN_ERR_INVALID, "the batched solver's FP64 refinement needs the block-tile engine: %s", p->btiles_why);
	jn_status st = batch_check_options(o);
	if (st) return st;
	if (o->num_eigenvectors && !o->eigenvectors)
		return jn_fail(JN_ERR_INVALID, "num_eigenvectors must be in 0..num_eigenvalues with an output array");
	const int f32 = o->precision == 32;
	cudaStream_t q = c->stream;
	/* the products' state: matrix elements, converted x, accumulators */
	double *me64 = NULL, *x64 = NULL;
	float *me32 = NULL, *x32 = NULL;
	unsigned long long *gacc = NULL, *pcmax = NULL;
	unsigned int *ctrl = NULL;
	int *pcoef = NULL, *pxbuf = NULL;
	BALLOC(me64, (size_t)B * nme);
	/* 32-bit products on the panel engine where it is this context's engine */
	const int panels = f32 && c->engine_of[1] == 4 && jn_panels_setup(c) == JN_OK && jn_panels_fit(c, 1);
	if (f32 && !panels) { BALLOC(me32, (size_t)B * nme); BALLOC(x32, (size_t)B * D); }
	else BALLOC(x64, (size_t)B * D);
	BALLOC(gacc, (size_t)B * D);
	BALLOC(ctrl, (size_t)2 * B);
	if (panels) {
		BALLOC(pcoef, (size_t)B * (p->n_coef ? p->n_coef : 1));
		BALLOC(pxbuf, (size_t)B * 2 * D);
		BALLOC(pcmax, B);
	}
	/* matrix elements: FP64 for refinement, FP32 copies with the reference's
	   |M| < 1e-12 skip of single-species blocks (matrix_vector_multiplication.c:52-53) */
	double maxme = 0.0;
	float *h32 = !st && f32 && !panels ? (float *)malloc(nme * sizeof(float)) : NULL;
	for (int i = 0; i < B && !st; i++) {
		const double *me = o->matrix_elements[i];
		if (!me) { st = jn_fail(JN_ERR_INVALID, "matrix_elements[%d] is NULL", i); break; }
		for (int64_t e = 0; e < nme; e++) maxme = fmax(maxme, fabs(me[e]));
		if (cudaMemcpyAsync(me64 + (size_t)i * nme, me, nme * sizeof(double), cudaMemcpyHostToDevice, q) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "upload of matrix elements");
		if (h32 && !st) {
			for (int b = 0; b < p->nmes; b++) {
				const jn_me_t *M = &p->mes[b];
				for (int64_t e = 0; e < M->len; e++) {
					const double v = me[M->offset + e];
					h32[M->offset + e] = (M->single && fabs(v) < 1e-12) ? 0.0f : (float)v;
				}
			}
			if (cudaMemcpy(me32 + (size_t)i * nme, h32, nme * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
				st = jn_fail(JN_ERR_CUDA, "upload of FP32 matrix elements");
		}
	}
	free(h32);
	if (!st) st = cudaMemsetAsync(gacc, 0, (size_t)B * D * sizeof(unsigned long long), q) == cudaSuccess
			      ? JN_OK : jn_fail(JN_ERR_CUDA, "accumulator clear");
	/* fixed-point scale bound valid for every instance */
	const double abs_bound = jn_plan_abs_bound(p, NULL) * maxme;
	if (!st && panels) st = jn_panels_batched_coefficients(c, B, me64, nme, pcoef, pcmax, q);
	/* each instance gets about (resident CTAs) / B persistent CTAs */
	jn_panel_partition part;
	memset(&part, 0, sizeof part);
	if (!st && panels) {
		int g = c->num_sms * c->panel_per_sm[1] / B;
		st = jn_panels_partition_upload(c, g < 8 ? 8 : g, &part);
	}
	int64_t *dims = (int64_t *)malloc(B * sizeof(int64_t));
	jn_batch_result **rp = (jn_batch_result **)malloc(B * sizeof(jn_batch_result *));
	for (int i = 0; i < B; i++) { dims[i] = D; rp[i] = res + i; }
	if (!st) {
		batch_job job;
		job.B = B;
		job.Dp = D;
		job.dims = dims;
		job.product = [&](const double *V, int64_t ldV, const int *d_k, double *W, const int *act, cudaStream_t qs) {
			return panels ? jn_enqueue_panels_batched(c, B, pcoef, pcmax, V, ldV, d_k, D, W, D, pxbuf, gacc, ctrl, act,
								  &part, qs)
				      : jn_enqueue_batched(c, B, f32, f32 ? (const void *)me32 : (const void *)me64, nme, V, ldV,
							   d_k, D, W, D, x64, x32, gacc, ctrl, act, abs_bound, qs);
		};
		job.product64 = [&](const double *X, int64_t ld, double *HX, double *scratch, cudaStream_t qs) {
			return jn_enqueue_batched(c, B, 0, me64, nme, X, ld, NULL, 0, HX, ld, scratch, NULL, gacc, ctrl, NULL,
						  abs_bound, qs);
		};
		job.start_vectors = o->start_vectors;
		job.eigenvectors = o->eigenvectors;
		job.res = rp;
		st = batch_solve(q, o, job);
	}
	free(dims); free(rp);
	void *bufs[] = { me64, x64, me32, x32, gacc, pcmax, ctrl, pcoef, pxbuf };
	for (size_t i = 0; i < sizeof bufs / sizeof bufs[0]; i++) cudaFree(bufs[i]);
	jn_panels_partition_free(&part);
	return st;
}

extern "C" jn_status jn_lanczos_batch_bases(jn_ctx *const *ctxs, int num_bases, const jn_batch_options *options,
					    jn_batch_result *const *results)
{
	if (!ctxs || !options || !results || num_bases < 1) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_batch_options *o = &options[0];
	jn_status st = batch_check_options(o);
	if (st) return st;
	int B = 0;
	int64_t Dp = 0;
	for (int b = 0; b < num_bases; b++) {
		const jn_batch_options *ob = &options[b];
		if (!ctxs[b] || !results[b] || !ob->matrix_elements) return jn_fail(JN_ERR_INVALID, "null argument for basis %d", b);
		if (ctxs[b]->plan.btiles_off)
			return jn_fail(JN_ERR_INVALID, "basis %d: the batched solver's FP64 refinement needs the block-tile engine: %s", b,
				       ctxs[b]->plan.btiles_why);
		if (ob->num_instances < 1) return jn_fail(JN_ERR_INVALID, "basis %d: num_instances must be >= 1", b);
		if (ob->max_iterations != o->max_iterations || ob->num_eigenvalues != o->num_eigenvalues ||
		    ob->tolerance != o->tolerance || ob->precision != o->precision || ob->check_every != o->check_every ||
		    ob->use_graph != o->use_graph || ob->refine_extra != o->refine_extra ||
		    ob->num_eigenvectors != o->num_eigenvectors)
			return jn_fail(JN_ERR_INVALID, "basis %d: the solver options differ from basis 0's", b);
		if (ob->num_eigenvectors && !ob->eigenvectors)
			return jn_fail(JN_ERR_INVALID, "basis %d: num_eigenvectors without an output array", b);
		if (ctxs[b]->plan.dim < 1) return jn_fail(JN_ERR_INVALID, "basis %d: empty basis", b);
		for (int j = 0; j < ob->num_instances; j++)
			if (!ob->matrix_elements[j]) return jn_fail(JN_ERR_INVALID, "basis %d: matrix_elements[%d] is NULL", b, j);
		B += ob->num_instances;
		if (ctxs[b]->plan.dim > Dp) Dp = ctxs[b]->plan.dim;
	}
	if (B > 4096) return jn_fail(JN_ERR_INVALID, "more than 4096 instances");
	cudaStream_t q = ctxs[0]->stream;
	/* the instances, basis by basis */
	int *ictx = (int *)malloc(B * sizeof(int)), *count = (int *)malloc(num_bases * sizeof(int));
	int *first = (int *)malloc(num_bases * sizeof(int));
	int64_t *dims = (int64_t *)malloc(B * sizeof(int64_t));
	const double **me = (const double **)malloc(B * sizeof(double *));
	const double **sv = (const double **)malloc(B * sizeof(double *));
	double **ev = (double **)malloc(B * sizeof(double *));
	jn_batch_result **rp = (jn_batch_result **)malloc(B * sizeof(jn_batch_result *));
	for (int b = 0, i = 0; b < num_bases; b++) {
		count[b] = options[b].num_instances;
		first[b] = i;
		for (int j = 0; j < count[b]; j++, i++) {
			ictx[i] = b;
			dims[i] = ctxs[b]->plan.dim;
			me[i] = options[b].matrix_elements[j];
			sv[i] = options[b].start_vectors ? options[b].start_vectors[j] : NULL;
			ev[i] = options[b].eigenvectors ? options[b].eigenvectors[j] : NULL;
			rp[i] = results[b] + j;
		}
	}
	/* per basis: FP64 matrix elements on the device, the refinement's accumulators, the scale bound */
	double **me64 = (double **)calloc(num_bases, sizeof(double *));
	unsigned long long **gacc = (unsigned long long **)calloc(num_bases, sizeof(void *));
	unsigned int **ctrl = (unsigned int **)calloc(num_bases, sizeof(void *));
	double *bound = (double *)calloc(num_bases, sizeof(double));
	for (int b = 0; b < num_bases && !st; b++) {
		const jn_plan_t *p = &ctxs[b]->plan;
		const int64_t nme = p->n_me;
		BALLOC(me64[b], (size_t)count[b] * nme);
		BALLOC(gacc[b], (size_t)count[b] * p->dim);
		BALLOC(ctrl[b], (size_t)2 * count[b]);
		double maxme = 0.0;
		for (int j = 0; j < count[b] && !st; j++) {
			const double *m = me[first[b] + j];
			for (int64_t e = 0; e < nme; e++) maxme = fmax(maxme, fabs(m[e]));
			if (cudaMemcpy(me64[b] + (size_t)j * nme, m, nme * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
				st = jn_fail(JN_ERR_CUDA, "upload of matrix elements");
		}
		if (!st && cudaMemset(gacc[b], 0, (size_t)count[b] * p->dim * sizeof(unsigned long long)) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "accumulator clear");
		bound[b] = jn_plan_abs_bound(p, NULL) * maxme;
	}
	/* the iteration products: one launch for every instance of every basis, on
	   the panel engine where every basis runs it (32-bit products), else on the
	   walk engine */
	struct jn_panel_batch *pb = NULL;
	struct jn_walk_batch *wb = NULL;
	if (!st) {
		if (o->precision == 32 && jn_panel_batch_possible(ctxs, num_bases))
			st = jn_panel_batch_create(ctxs, num_bases, count, me64, &pb);
		else
			st = jn_walk_batch_create(ctxs, ictx, B, me, o->precision == 32, &wb);
	}
	if (!st) {
		const int mode = o->precision == 32 ? 32 : 64;
		batch_job job;
		job.B = B;
		job.Dp = Dp;
		job.dims = dims;
		job.product = [&](const double *V, int64_t ldV, const int *d_k, double *W, const int *act, cudaStream_t qs) {
			return pb ? jn_panel_batch_enqueue(pb, V, ldV, d_k, Dp, W, Dp, act, Dp, qs)
				  : jn_walk_batch_enqueue(wb, mode, V, ldV, d_k, Dp, W, Dp, act, Dp, qs);
		};
		/* refinement, basis by basis, on the block-tile engine in FP64 */
		job.product64 = [&](const double *X, int64_t ld, double *HX, double *scratch, cudaStream_t qs) {
			for (int b = 0; b < num_bases; b++) {
				jn_ctx *c = ctxs[b];
				const size_t i0 = (size_t)first[b];
				jn_status e = jn_enqueue_batched(c, count[b], 0, me64[b], c->plan.n_me, X + i0 * ld, ld, NULL, 0,
								 HX + i0 * ld, ld, scratch + i0 * Dp, NULL, gacc[b], ctrl[b], NULL,
								 bound[b], qs);
				if (e) return e;
			}
			return JN_OK;
		};
		job.start_vectors = sv;
		job.eigenvectors = ev;
		job.res = rp;
		st = batch_solve(q, o, job);
	}
	jn_panel_batch_free(pb);
	jn_walk_batch_free(wb);
	for (int b = 0; b < num_bases; b++) {
		cudaFree(me64[b]);
		cudaFree(gacc[b]);
		cudaFree(ctrl[b]);
	}
	free(me64); free(gacc); free(ctrl); free(bound);
	free(ictx); free(count); free(first); free(dims); free(me); free(sv); free(ev); free(rp);
	return st;
}

/* ------------------------------------------------------------------ */
/* matrix-element sets on the context's lists                           */
/* ------------------------------------------------------------------ */
extern "C" size_t jn_me_count(const jn_ctx *c) { return c ? (size_t)c->plan.n_me : 0; }

extern "C" jn_status jn_read_matrix_elements(const jn_ctx *c, const char *dir, double *out)
{
	if (!c || !dir || !out) return jn_fail(JN_ERR_INVALID, "null argument");
	char err[1024] = "";
	if (jn_plan_read_me(&c->plan, dir, out, err, sizeof err))
		return jn_fail(strstr(err, "Could not open") ? JN_ERR_IO : JN_ERR_FORMAT, "%s", err);
	return JN_OK;
}

extern "C" jn_status jn_set_matrix_elements(jn_ctx *c, const double *me)
{
	if (!c || !me) return jn_fail(JN_ERR_INVALID, "null argument");
	jn_plan_t *p = &c->plan;
	memcpy(p->me, me, (size_t)p->n_me * sizeof(double));
	p->abs_bound = jn_plan_abs_bound(p, p->me);
	CUDA_TRY(cudaMemcpy(c->d_me, p->me, (size_t)p->n_me * sizeof(double), cudaMemcpyHostToDevice));
	jn_panels_invalidate(c);
	jn_walk_invalidate(c);
	if (c->d_me32) {
		float *h = (float *)malloc((p->n_me ? p->n_me : 1) * sizeof(float));
		if (!h) return jn_fail(JN_ERR_NOMEM, "out of host memory");
		for (int b = 0; b < p->nmes; b++) {
			const jn_me_t *M = &p->mes[b];
			for (int64_t e = 0; e < M->len; e++) {
				const double v = p->me[M->offset + e];
				h[M->offset + e] = (M->single && fabs(v) < 1e-12) ? 0.0f : (float)v;
			}
		}
		cudaError_t e = cudaMemcpy(c->d_me32, h, (size_t)p->n_me * sizeof(float), cudaMemcpyHostToDevice);
		free(h);
		if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "FP32 matrix elements: %s", cudaGetErrorString(e));
	}
	return JN_OK;
}
