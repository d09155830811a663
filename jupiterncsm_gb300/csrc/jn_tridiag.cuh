/*
 * jn_tridiag.cuh — device routines for the symmetric tridiagonal
 * eigenproblem of Lanczos (diagonal a[0..n), off-diagonal b[0..n-1)),
 * shared by the single solve (jn_lanczos.cu) and the batched solve
 * (jn_batch.cu).  They replace LAPACK dsteqr in the reference
 * (src/Bacchus/diagonalization/diagonalization.c:16-68).
 */
#ifndef JN_TRIDIAG_CUH
#define JN_TRIDIAG_CUH

#include <stdint.h>

/* number of eigenvalues below x (Sturm sequence) */
__device__ __forceinline__ int jn_sturm_count(const double *a, const double *b, int n, double x)
{
	int c = 0;
	double q = a[0] - x;
	if (q < 0) c++;
	for (int i = 1; i < n; i++) {
		double qq = q == 0.0 ? 1e-300 : q;
		q = a[i] - x - b[i - 1] * b[i - 1] / qq;
		if (q < 0) c++;
	}
	return c;
}

/* the i-th smallest eigenvalue by multisection, one warp per eigenvalue:
 * each round the 32 lanes evaluate the Sturm count at 32 points of the
 * bracket, which shrinks 32-fold, so about 11 rounds reach full precision
 * where bisection needs about 52 sequential steps.  Every lane returns the
 * same value. */
__device__ __forceinline__ double jn_tri_multisect_warp(const double *a, const double *b, int n, int i)
{
	const int lane = threadIdx.x & 31;
	double lo = 1e300, hi = -1e300;
	for (int j = lane; j < n; j += 32) {
		double r = (j > 0 ? fabs(b[j - 1]) : 0.0) + (j < n - 1 ? fabs(b[j]) : 0.0);
		lo = fmin(lo, a[j] - r);
		hi = fmax(hi, a[j] + r);
	}
	for (int o = 16; o; o >>= 1) {
		lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
		hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
	}
	const double span = fmax(fabs(lo), fabs(hi));
	lo -= 1e-12 * span + 1e-300;
	hi += 1e-12 * span + 1e-300;
	for (int round = 0; round < 64; round++) {
		const double w = (hi - lo) * (1.0 / 32.0);
		const double x = lane == 31 ? hi : lo + (double)(lane + 1) * w;
		const unsigned int above = __ballot_sync(0xffffffffu, jn_sturm_count(a, b, n, x) > i);
		const int f = above ? __ffs(above) - 1 : 31;
		const double nlo = f == 0 ? lo : __shfl_sync(0xffffffffu, x, f - 1);
		const double nhi = __shfl_sync(0xffffffffu, x, f);
		if (!(nlo > lo || nhi < hi)) break;     /* the bracket no longer shrinks: converged */
		lo = nlo;
		hi = nhi;
	}
	return 0.5 * (lo + hi);
}

/* eigenvector z[0..n) for the eigenvalue sh by inverse iteration with the
 * LU factorisation (partial pivoting) of T - sh I, as dgttrf/dgtts2 do;
 * normalised, z[0] >= 0 as diagonalization.c:55-58 makes it.
 * work: 5 n doubles. */
__device__ __forceinline__ void jn_tri_vector_one(const double *a, const double *b, int n, double sh, double *z,
						  double *work)
{
	double *d = work, *u1 = d + n, *u2 = u1 + n, *l = u2 + n, *pv = l + n;
	double span = 0.0;
	for (int j = 0; j < n; j++) span = fmax(span, fabs(a[j]) + (j < n - 1 ? fabs(b[j]) : 0.0));
	const double eps = 2.2e-16 * fmax(span, 1e-300);
	double dd = a[0] - sh, e = n > 1 ? b[0] : 0.0;
	for (int j = 0; j < n - 1; j++) {
		double sub = b[j];
		double nd = a[j + 1] - sh, ne = (j + 1 < n - 1) ? b[j + 1] : 0.0;
		if (fabs(dd) >= fabs(sub)) {
			pv[j] = 0.0;
			if (dd == 0.0) dd = eps;
			double m = sub / dd;
			l[j] = m;
			d[j] = dd; u1[j] = e; u2[j] = 0.0;
			dd = nd - m * e;
			e = ne;
		} else {
			pv[j] = 1.0;
			double m = dd / sub;
			l[j] = m;
			d[j] = sub; u1[j] = nd; u2[j] = ne;
			dd = e - m * nd;
			e = -m * ne;
		}
	}
	if (dd == 0.0) dd = eps;
	d[n - 1] = dd; u1[n - 1] = 0.0; u2[n - 1] = 0.0;
	for (int j = 0; j < n; j++) z[j] = 1.0;
	for (int iter = 0; iter < 3; iter++) {
		for (int j = 0; j < n - 1; j++) {
			if (pv[j] != 0.0) { double t = z[j]; z[j] = z[j + 1]; z[j + 1] = t - l[j] * z[j]; }
			else z[j + 1] -= l[j] * z[j];
		}
		for (int j = n - 1; j >= 0; j--) {
			double s = z[j];
			if (j + 1 < n) s -= u1[j] * z[j + 1];
			if (j + 2 < n) s -= u2[j] * z[j + 2];
			z[j] = s / (fabs(d[j]) < eps ? (d[j] < 0 ? -eps : eps) : d[j]);
		}
		double nrm = 0.0;
		for (int j = 0; j < n; j++) nrm = fma(z[j], z[j], nrm);
		nrm = sqrt(nrm);
		for (int j = 0; j < n; j++) z[j] /= nrm;
	}
	if (z[0] < 0)
		for (int j = 0; j < n; j++) z[j] = -z[j];
}

/* fixed-order sum over the CTA (blockDim.x a power of two, sh of blockDim.x) */
__device__ __forceinline__ double jn_block_sum(double v, double *sh)
{
	const int t = threadIdx.x;
	sh[t] = v;
	__syncthreads();
	for (int s = blockDim.x / 2; s > 0; s >>= 1) {
		if (t < s) sh[t] += sh[t + s];
		__syncthreads();
	}
	double r = sh[0];
	__syncthreads();
	return r;
}

/* modified Gram-Schmidt among `want` vectors of length n (rows of Z), by one
 * CTA: repairs inverse-iteration vectors of close eigenvalues */
__device__ __forceinline__ void jn_tri_mgs(double *Z, int ldz, int n, int want, double *sh)
{
	for (int i = 0; i < want; i++) {
		double *zi = Z + (int64_t)i * ldz;
		for (int j = 0; j < i; j++) {
			const double *zj = Z + (int64_t)j * ldz;
			double s = 0.0;
			for (int t = threadIdx.x; t < n; t += blockDim.x) s = fma(zi[t], zj[t], s);
			s = jn_block_sum(s, sh);
			for (int t = threadIdx.x; t < n; t += blockDim.x) zi[t] -= s * zj[t];
			__syncthreads();
		}
		double s = 0.0;
		for (int t = threadIdx.x; t < n; t += blockDim.x) s = fma(zi[t], zi[t], s);
		s = jn_block_sum(s, sh);
		double inv = 1.0 / sqrt(s);
		for (int t = threadIdx.x; t < n; t += blockDim.x) zi[t] *= inv;
		__syncthreads();
		if (threadIdx.x == 0) sh[0] = zi[0] < 0 ? -1.0 : 1.0;
		__syncthreads();
		double sg = sh[0];
		__syncthreads();
		for (int t = threadIdx.x; t < n; t += blockDim.x) zi[t] *= sg;
		__syncthreads();
	}
}

#endif
