/*
 * jn_mlp.cu — the learned warm start: a small MLP, trained and run with
 * hand-written kernels, that maps the couplings c of H(c) = H0 + sum c_i H_i
 * to coefficients over a reduced basis of snapshot eigenvectors.  The
 * expanded vector is the Lanczos start vector.  No counterpart in the
 * reference.
 *
 * Network (FP32): x (n_in) -> h1 = gelu(W1 x + b1) (H) -> h2 = gelu(W2 h1 + b2)
 * (H) -> y = W3 h2 + b3 (n_out), gelu(a) = a/2 (1 + erf(a/sqrt 2)).
 * Loss: sum over samples and outputs of (y - t)^2 / (2 N).  Parameters are
 * one flat array [W1 (H x n_in), b1, W2 (H x H), b2, W3 (n_out x H), b3],
 * row-major with the output index first.  Gradients are summed over samples
 * in sample order (no atomics), so training is deterministic.  Adam updates
 * the parameters.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "jn_internal.h"
#include "jn_tridiag.cuh"

struct jn_mlp {
	int nin, nh, nout;
	int64_t np;                     /* parameters */
	float *d_p, *d_g, *d_m, *d_v;   /* parameters, gradient, Adam moments */
	int64_t t;                      /* Adam steps taken */
	int cap;                        /* samples the activation buffers hold */
	float *d_x, *d_t, *d_a1, *d_h1, *d_a2, *d_h2, *d_y, *d_d1, *d_d2, *d_d3, *d_loss;
	cudaStream_t stream;
};

struct mlp_off {
	int64_t w1, b1, w2, b2, w3, b3;
};

__host__ __device__ static inline mlp_off offsets(int nin, int nh, int nout)
{
	mlp_off o;
	o.w1 = 0;
	o.b1 = o.w1 + (int64_t)nh * nin;
	o.w2 = o.b1 + nh;
	o.b2 = o.w2 + (int64_t)nh * nh;
	o.w3 = o.b2 + nh;
	o.b3 = o.w3 + (int64_t)nout * nh;
	return o;
}

__device__ __forceinline__ float gelu(float a) { return 0.5f * a * (1.0f + erff(a * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float a)
{
	return 0.5f * (1.0f + erff(a * 0.70710678118654752f)) + a * 0.39894228040143268f * expf(-0.5f * a * a);
}

/* one CTA per sample, blockDim >= max(nh, nout) */
__global__ void mlp_forward(const float *__restrict__ P, int nin, int nh, int nout, int n, const float *__restrict__ X,
			    float *__restrict__ A1, float *__restrict__ H1, float *__restrict__ A2, float *__restrict__ H2,
			    float *__restrict__ Y)
{
	extern __shared__ float sm[];
	float *x = sm, *h1 = x + nin, *h2 = h1 + nh;
	const int s = blockIdx.x, j = threadIdx.x;
	if (s >= n) return;
	const mlp_off o = offsets(nin, nh, nout);
	for (int i = j; i < nin; i += blockDim.x) x[i] = X[(int64_t)s * nin + i];
	__syncthreads();
	if (j < nh) {
		float a = P[o.b1 + j];
		for (int i = 0; i < nin; i++) a = fmaf(P[o.w1 + (int64_t)j * nin + i], x[i], a);
		A1[(int64_t)s * nh + j] = a;
		h1[j] = H1[(int64_t)s * nh + j] = gelu(a);
	}
	__syncthreads();
	if (j < nh) {
		float a = P[o.b2 + j];
		for (int k = 0; k < nh; k++) a = fmaf(P[o.w2 + (int64_t)j * nh + k], h1[k], a);
		A2[(int64_t)s * nh + j] = a;
		h2[j] = H2[(int64_t)s * nh + j] = gelu(a);
	}
	__syncthreads();
	if (j < nout) {
		float a = P[o.b3 + j];
		for (int k = 0; k < nh; k++) a = fmaf(P[o.w3 + (int64_t)j * nh + k], h2[k], a);
		Y[(int64_t)s * nout + j] = a;
	}
}

/* per sample: output error and the back-propagated deltas; loss partial per sample */
__global__ void mlp_deltas(const float *__restrict__ P, int nin, int nh, int nout, int n, const float *__restrict__ T,
			   const float *__restrict__ Y, const float *__restrict__ A1, const float *__restrict__ A2,
			   float *__restrict__ D1, float *__restrict__ D2, float *__restrict__ D3, float *__restrict__ lossp)
{
	extern __shared__ float sm[];
	float *d3 = sm, *d2 = d3 + nout;
	const int s = blockIdx.x, j = threadIdx.x;
	if (s >= n) return;
	const mlp_off o = offsets(nin, nh, nout);
	const float inv = 1.0f / (float)n;
	if (j < nout) {
		const float e = Y[(int64_t)s * nout + j] - T[(int64_t)s * nout + j];
		d3[j] = D3[(int64_t)s * nout + j] = e * inv;
	}
	__syncthreads();
	if (j == 0) {
		float l = 0.0f;
		for (int q = 0; q < nout; q++) {
			const float e = Y[(int64_t)s * nout + q] - T[(int64_t)s * nout + q];
			l = fmaf(e, e, l);
		}
		lossp[s] = 0.5f * l * inv;
	}
	if (j < nh) {
		float g = 0.0f;
		for (int q = 0; q < nout; q++) g = fmaf(P[o.w3 + (int64_t)q * nh + j], d3[q], g);
		d2[j] = D2[(int64_t)s * nh + j] = g * gelu_grad(A2[(int64_t)s * nh + j]);
	}
	__syncthreads();
	if (j < nh) {
		float g = 0.0f;
		for (int k = 0; k < nh; k++) g = fmaf(P[o.w2 + (int64_t)k * nh + j], d2[k], g);
		D1[(int64_t)s * nh + j] = g * gelu_grad(A1[(int64_t)s * nh + j]);
	}
}

/* one thread per parameter: the gradient summed over samples in order */
__global__ void mlp_gradients(int nin, int nh, int nout, int n, const float *__restrict__ X, const float *__restrict__ H1,
			      const float *__restrict__ H2, const float *__restrict__ D1, const float *__restrict__ D2,
			      const float *__restrict__ D3, float *__restrict__ G)
{
	const mlp_off o = offsets(nin, nh, nout);
	const int64_t np = o.b3 + nout;
	const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= np) return;
	const float *delta, *act;
	int dn, an, row, col;
	if (p < o.b1) { delta = D1; dn = nh; act = X; an = nin; row = (int)((p - o.w1) / nin); col = (int)((p - o.w1) % nin); }
	else if (p < o.w2) { delta = D1; dn = nh; act = NULL; an = 0; row = (int)(p - o.b1); col = 0; }
	else if (p < o.b2) { delta = D2; dn = nh; act = H1; an = nh; row = (int)((p - o.w2) / nh); col = (int)((p - o.w2) % nh); }
	else if (p < o.w3) { delta = D2; dn = nh; act = NULL; an = 0; row = (int)(p - o.b2); col = 0; }
	else if (p < o.b3) { delta = D3; dn = nout; act = H2; an = nh; row = (int)((p - o.w3) / nh); col = (int)((p - o.w3) % nh); }
	else { delta = D3; dn = nout; act = NULL; an = 0; row = (int)(p - o.b3); col = 0; }
	float g = 0.0f;
	for (int s = 0; s < n; s++) {
		const float d = delta[(int64_t)s * dn + row];
		g = act ? fmaf(d, act[(int64_t)s * an + col], g) : g + d;
	}
	G[p] = g;
}

__global__ void mlp_loss_sum(const float *__restrict__ lossp, int n, float *__restrict__ out)
{
	if (threadIdx.x || blockIdx.x) return;
	float l = 0.0f;
	for (int s = 0; s < n; s++) l += lossp[s];
	out[n] = l;
}

__global__ void mlp_adam(float *__restrict__ P, const float *__restrict__ G, float *__restrict__ M, float *__restrict__ V,
			 int64_t np, float lr, float b1, float b2, float eps, float c1, float c2)
{
	const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= np) return;
	const float g = G[p];
	const float m = M[p] = b1 * M[p] + (1.0f - b1) * g;
	const float v = V[p] = b2 * V[p] + (1.0f - b2) * g * g;
	P[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

/* ------------------------------------------------------------------ */
static int threads_for(const jn_mlp *m)
{
	int t = m->nh > m->nout ? m->nh : m->nout;
	return (t + 31) / 32 * 32;
}

static jn_status ensure_capacity(jn_mlp *m, int n)
{
	if (n <= m->cap) return JN_OK;
	float **bufs[] = { &m->d_x, &m->d_t, &m->d_a1, &m->d_h1, &m->d_a2, &m->d_h2, &m->d_y, &m->d_d1, &m->d_d2, &m->d_d3,
			   &m->d_loss };
	const int64_t w[] = { m->nin, m->nout, m->nh, m->nh, m->nh, m->nh, m->nout, m->nh, m->nh, m->nout, 1 };
	for (size_t i = 0; i < sizeof bufs / sizeof bufs[0]; i++) {
		cudaFree(*bufs[i]);
		*bufs[i] = NULL;
		if (cudaMalloc((void **)bufs[i], (size_t)(n + 1) * w[i] * sizeof(float)) != cudaSuccess) {
			m->cap = 0;
			return jn_fail(JN_ERR_NOMEM, "MLP activations for %d samples", n);
		}
	}
	m->cap = n;
	return JN_OK;
}

extern "C" void jn_mlp_destroy(jn_mlp *m)
{
	if (!m) return;
	float *p[] = { m->d_p, m->d_g, m->d_m, m->d_v, m->d_x, m->d_t, m->d_a1, m->d_h1, m->d_a2, m->d_h2, m->d_y,
		       m->d_d1, m->d_d2, m->d_d3, m->d_loss };
	for (size_t i = 0; i < sizeof p / sizeof p[0]; i++) cudaFree(p[i]);
	if (m->stream) cudaStreamDestroy(m->stream);
	free(m);
}

extern "C" jn_status jn_mlp_create(int nin, int nh, int nout, uint64_t seed, jn_mlp **out)
{
	if (!out || nin < 1 || nh < 1 || nout < 1 || nh > 1024 || nout > 1024 || nin > 1024)
		return jn_fail(JN_ERR_INVALID, "MLP sizes must be in 1..1024");
	*out = NULL;
	jn_mlp *m = (jn_mlp *)calloc(1, sizeof *m);
	m->nin = nin; m->nh = nh; m->nout = nout;
	const mlp_off o = offsets(nin, nh, nout);
	m->np = o.b3 + nout;
	float *h = (float *)calloc(m->np, sizeof(float));
	/* seeded uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases */
	uint64_t z = seed;
	auto unif = [&z]() {
		z += 0x9E3779B97F4A7C15ull;
		uint64_t v = z;
		v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ull;
		v = (v ^ (v >> 27)) * 0x94D049BB133111EBull;
		v ^= v >> 31;
		return (double)(v >> 11) * 0x1.0p-53 * 2.0 - 1.0;
	};
	for (int64_t i = 0; i < (int64_t)nh * nin; i++) h[o.w1 + i] = (float)(unif() / sqrt((double)nin));
	for (int64_t i = 0; i < (int64_t)nh * nh; i++) h[o.w2 + i] = (float)(unif() / sqrt((double)nh));
	for (int64_t i = 0; i < (int64_t)nout * nh; i++) h[o.w3 + i] = (float)(unif() / sqrt((double)nh));
	jn_status st = JN_OK;
	float **bufs[] = { &m->d_p, &m->d_g, &m->d_m, &m->d_v };
	for (int i = 0; i < 4 && !st; i++)
		if (cudaMalloc((void **)bufs[i], m->np * sizeof(float)) != cudaSuccess ||
		    cudaMemset(*bufs[i], 0, m->np * sizeof(float)) != cudaSuccess)
			st = jn_fail(JN_ERR_NOMEM, "MLP parameters");
	if (!st && cudaMemcpy(m->d_p, h, m->np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
		st = jn_fail(JN_ERR_CUDA, "MLP parameter upload");
	if (!st && cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess)
		st = jn_fail(JN_ERR_CUDA, "MLP stream");
	free(h);
	if (st) { jn_mlp_destroy(m); return st; }
	*out = m;
	return JN_OK;
}

extern "C" size_t jn_mlp_num_params(const jn_mlp *m) { return m ? (size_t)m->np : 0; }

extern "C" jn_status jn_mlp_get_params(const jn_mlp *m, float *params)
{
	if (!m || !params) return jn_fail(JN_ERR_INVALID, "null argument");
	CUDA_TRY(cudaMemcpy(params, m->d_p, m->np * sizeof(float), cudaMemcpyDeviceToHost));
	return JN_OK;
}

extern "C" jn_status jn_mlp_set_params(jn_mlp *m, const float *params)
{
	if (!m || !params) return jn_fail(JN_ERR_INVALID, "null argument");
	CUDA_TRY(cudaMemcpy(m->d_p, params, m->np * sizeof(float), cudaMemcpyHostToDevice));
	return JN_OK;
}

static jn_status forward(jn_mlp *m, int n)
{
	const int th = threads_for(m);
	mlp_forward<<<n, th, (m->nin + 2 * m->nh) * sizeof(float), m->stream>>>(m->d_p, m->nin, m->nh, m->nout, n, m->d_x,
										m->d_a1, m->d_h1, m->d_a2, m->d_h2, m->d_y);
	return cudaGetLastError() == cudaSuccess ? JN_OK : jn_fail(JN_ERR_CUDA, "MLP forward launch");
}

static jn_status backward(jn_mlp *m, int n)
{
	const int th = threads_for(m);
	mlp_deltas<<<n, th, (m->nout + m->nh) * sizeof(float), m->stream>>>(m->d_p, m->nin, m->nh, m->nout, n, m->d_t,
									      m->d_y, m->d_a1, m->d_a2, m->d_d1, m->d_d2,
									      m->d_d3, m->d_loss);
	mlp_loss_sum<<<1, 32, 0, m->stream>>>(m->d_loss, n, m->d_loss);
	mlp_gradients<<<(int)((m->np + 255) / 256), 256, 0, m->stream>>>(m->nin, m->nh, m->nout, n, m->d_x, m->d_h1, m->d_h2,
									  m->d_d1, m->d_d2, m->d_d3, m->d_g);
	return cudaGetLastError() == cudaSuccess ? JN_OK : jn_fail(JN_ERR_CUDA, "MLP backward launch");
}

static jn_status load(jn_mlp *m, const float *x, const float *t, int n)
{
	jn_status s = ensure_capacity(m, n);
	if (s) return s;
	CUDA_TRY(cudaMemcpyAsync(m->d_x, x, (size_t)n * m->nin * sizeof(float), cudaMemcpyHostToDevice, m->stream));
	if (t) CUDA_TRY(cudaMemcpyAsync(m->d_t, t, (size_t)n * m->nout * sizeof(float), cudaMemcpyHostToDevice, m->stream));
	return JN_OK;
}

extern "C" jn_status jn_mlp_loss_and_gradient(jn_mlp *m, const float *x, const float *t, int n, float *loss, float *grad)
{
	if (!m || !x || !t || n < 1) return jn_fail(JN_ERR_INVALID, "bad argument");
	jn_status s = load(m, x, t, n);
	if (!s) s = forward(m, n);
	if (!s) s = backward(m, n);
	if (s) return s;
	if (loss) CUDA_TRY(cudaMemcpyAsync(loss, m->d_loss + n, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
	if (grad) CUDA_TRY(cudaMemcpyAsync(grad, m->d_g, m->np * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
	CUDA_TRY(cudaStreamSynchronize(m->stream));
	return JN_OK;
}

extern "C" jn_status jn_mlp_train(jn_mlp *m, const float *x, const float *t, int n, int steps, float lr, float *final_loss)
{
	if (!m || !x || !t || n < 1 || steps < 0) return jn_fail(JN_ERR_INVALID, "bad argument");
	jn_status s = load(m, x, t, n);
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	for (int it = 0; it < steps && !s; it++) {
		s = forward(m, n);
		if (!s) s = backward(m, n);
		m->t++;
		const float c1 = 1.0f - powf(b1, (float)m->t), c2 = 1.0f - powf(b2, (float)m->t);
		if (!s) mlp_adam<<<(int)((m->np + 255) / 256), 256, 0, m->stream>>>(m->d_p, m->d_g, m->d_m, m->d_v, m->np, lr, b1,
										       b2, eps, c1, c2);
	}
	if (s) return s;
	/* loss of the final parameters */
	s = forward(m, n);
	if (!s) s = backward(m, n);
	if (s) return s;
	if (final_loss) CUDA_TRY(cudaMemcpyAsync(final_loss, m->d_loss + n, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
	CUDA_TRY(cudaStreamSynchronize(m->stream));
	CUDA_TRY(cudaGetLastError());
	return JN_OK;
}

extern "C" jn_status jn_mlp_predict(jn_mlp *m, const float *x, int n, float *y)
{
	if (!m || !x || !y || n < 1) return jn_fail(JN_ERR_INVALID, "bad argument");
	jn_status s = load(m, x, NULL, n);
	if (!s) s = forward(m, n);
	if (s) return s;
	CUDA_TRY(cudaMemcpyAsync(y, m->d_y, (size_t)n * m->nout * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
	CUDA_TRY(cudaStreamSynchronize(m->stream));
	return JN_OK;
}


/* ------------------------------------------------------------------ */
/* warm start: reduced basis of solver snapshots + MLP coordinates      */
/* ------------------------------------------------------------------ */
#define WT 256

/* out[row] = A_row . V_row with A_row = A + row * lda, V_row = V + row * ldv
 * (ldv = 0: one vector for all rows); one CTA per row, fixed order */
__global__ void __launch_bounds__(WT) ws_dots(const double *__restrict__ A, int64_t lda, const double *__restrict__ V,
					      int64_t ldv, int64_t dim, double *__restrict__ out)
{
	__shared__ double sh[WT];
	const double *a = A + (int64_t)blockIdx.x * lda, *v = V + (int64_t)blockIdx.x * ldv;
	double s = 0.0;
	for (int64_t i = threadIdx.x; i < dim; i += WT) s = fma(a[i], v[i], s);
	s = jn_block_sum(s, sh);
	if (threadIdx.x == 0) out[blockIdx.x] = s;
}

/* out = sum_{r < nrows} coef[r] A_r (coef on the device), or out -= it when sub */
__global__ void ws_combine(const double *__restrict__ A, int64_t lda, int nrows, const double *__restrict__ coef,
			   int64_t dim, double *__restrict__ out, int sub)
{
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int r = 0; r < nrows; r++) s = fma(coef[r], A[(int64_t)r * lda + i], s);
		out[i] = sub ? out[i] - s : s;
	}
}

/* row = blockIdx.y: A_row *= 1 / sqrt(nrm2[row]) */
__global__ void ws_scale(double *__restrict__ A, int64_t lda, const double *__restrict__ nrm2, int64_t dim)
{
	double *a = A + (int64_t)blockIdx.y * lda;
	const double inv = 1.0 / sqrt(nrm2[blockIdx.y]);
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
		a[i] *= inv;
}

/* sample s = blockIdx.y: out_s = sum_j coef[s][j] Q_j + noise * r */
__global__ void ws_expand(const double *__restrict__ Q, int k, const double *__restrict__ coef,
			  const double *__restrict__ r, double noise, int64_t dim, double *__restrict__ out)
{
	const int s = blockIdx.y;
	const double *c = coef + (int64_t)s * k;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
		double v = noise * r[i];
		for (int j = 0; j < k; j++) v = fma(c[j], Q[(int64_t)j * dim + i], v);
		out[(int64_t)s * dim + i] = v;
	}
}

struct jn_warm_start {
	int64_t dim;
	int nc, k;
	double noise;
	double *mean, *scale;   /* input standardisation (host, nc) */
	jn_mlp *mlp;
	double *d_Q;            /* reduced basis, k x dim, orthonormal */
	double *d_r;            /* the default start vector, normalised */
};

extern "C" void jn_default_start_vector(int64_t dim, double *out)
{
	/* SplitMix64 stream, uniform in [-0.5, 0.5) */
	uint64_t z = 0x9E3779B97F4A7C15ull;
	for (int64_t e = 0; e < dim; e++) {
		z += 0x9E3779B97F4A7C15ull;
		uint64_t v = z;
		v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ull;
		v = (v ^ (v >> 27)) * 0x94D049BB133111EBull;
		v ^= v >> 31;
		out[e] = (double)(v >> 11) * 0x1.0p-53 - 0.5;
	}
}

extern "C" void jn_warm_start_destroy(jn_warm_start *w)
{
	if (!w) return;
	jn_mlp_destroy(w->mlp);
	cudaFree(w->d_Q);
	cudaFree(w->d_r);
	free(w->mean);
	free(w->scale);
	free(w);
}

static int grid_for(int64_t dim)
{
	int64_t g = (dim + 255) / 256;
	return (int)(g < 1 ? 1 : g > 256 ? 256 : g);
}

extern "C" jn_status jn_warm_start_fit(const jn_warm_start_options *o, int64_t dim, int nc, int S, const double *cpl,
				       int nv, const double *const *eig, jn_warm_start **out, float *final_loss)
{
	if (!o || !cpl || !eig || !out) return jn_fail(JN_ERR_INVALID, "null argument");
	*out = NULL;
	const int hidden = o->hidden > 0 ? o->hidden : 128;
	int k = o->basis_size > 0 ? o->basis_size : 32;
	const int steps = o->train_steps > 0 ? o->train_steps : 3000;
	const float lr = o->learning_rate > 0 ? o->learning_rate : 1e-3f;
	if (dim < 1 || nc < 1 || nc > 1024 || S < 1 || S > 2048 || nv < 1 || o->noise < 0)
		return jn_fail(JN_ERR_INVALID, "warm start: need dim >= 1, 1..1024 couplings, 1..2048 samples, "
					       "num_vectors >= 1, noise >= 0");
	if (k > S) k = S;
	if (k > 1024) k = 1024;
	for (int s = 0; s < S; s++)
		if (!eig[s]) return jn_fail(JN_ERR_INVALID, "eigenvectors[%d] is NULL", s);
	jn_warm_start *w = (jn_warm_start *)calloc(1, sizeof *w);
	w->dim = dim;
	w->nc = nc;
	w->noise = o->noise > 0 ? o->noise : 0.01;
	w->mean = (double *)calloc(nc, sizeof(double));
	w->scale = (double *)calloc(nc, sizeof(double));
	jn_status st = JN_OK;
	double *d_E = NULL, *d_U = NULL, *d_c = NULL, *d_d = NULL;
	double *hr = (double *)malloc(dim * sizeof(double)), *hd = (double *)malloc(S * sizeof(double));
	double *T = (double *)calloc((size_t)S * k, sizeof(double)), *res = (double *)malloc(S * sizeof(double));
	char *used = (char *)calloc(S, 1);
	cudaStream_t q = NULL;
	if (cudaMalloc((void **)&w->d_r, dim * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&w->d_Q, (size_t)k * dim * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&d_E, (size_t)nv * dim * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&d_U, (size_t)S * dim * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&d_c, (size_t)(S > nv ? S : nv) * sizeof(double) + (size_t)k * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&d_d, (size_t)(S > k ? S : k) * sizeof(double)) != cudaSuccess)
		st = jn_fail(JN_ERR_NOMEM, "warm start: device buffers for %d samples of dimension %lld", S, (long long)dim);
	if (!st) st = jn_mlp_create(nc, hidden, k, o->seed, &w->mlp);
	if (!st) q = w->mlp->stream;
	const int g = grid_for(dim);
	/* r / |r| */
	if (!st) {
		jn_default_start_vector(dim, hr);
		double n2 = 0.0;
		for (int64_t i = 0; i < dim; i++) n2 += hr[i] * hr[i];
		const double inv = 1.0 / sqrt(n2);
		for (int64_t i = 0; i < dim; i++) hr[i] *= inv;
		if (cudaMemcpy(w->d_r, hr, dim * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "warm start: upload");
	}
	/* u_s = sum_e v_e (v_e . r), normalised */
	for (int s = 0; s < S && !st; s++) {
		if (cudaMemcpyAsync(d_E, eig[s], (size_t)nv * dim * sizeof(double), cudaMemcpyHostToDevice, q) != cudaSuccess) {
			st = jn_fail(JN_ERR_CUDA, "warm start: upload of snapshot %d", s);
			break;
		}
		ws_dots<<<nv, WT, 0, q>>>(d_E, dim, w->d_r, 0, dim, d_c);
		ws_combine<<<g, 256, 0, q>>>(d_E, dim, nv, d_c, dim, d_U + (size_t)s * dim, 0);
		/* the staging buffer is reused by the next sample's copy */
		if (cudaStreamSynchronize(q) != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "warm start: snapshot %d", s);
	}
	if (!st) {
		ws_dots<<<S, WT, 0, q>>>(d_U, dim, d_U, dim, dim, d_d);
		if (cudaMemcpyAsync(hd, d_d, S * sizeof(double), cudaMemcpyDeviceToHost, q) != cudaSuccess ||
		    cudaStreamSynchronize(q) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "warm start: snapshot norms");
		for (int s = 0; s < S && !st; s++)
			if (!(hd[s] > 0.0) || !isfinite(hd[s]))
				st = jn_fail(JN_ERR_INVALID, "warm start: snapshot %d has no component along the start vector", s);
		if (!st) ws_scale<<<dim3(g, S), 256, 0, q>>>(d_U, dim, d_d, dim);
	}
	/* greedy reduced basis: the snapshot with the largest residual, CGS2 */
	for (int s = 0; s < S; s++) res[s] = 1.0;
	int kk = 0;
	for (int j = 0; j < k && !st; j++) {
		int best = -1;
		for (int s = 0; s < S; s++)
			if (!used[s] && (best < 0 || res[s] > res[best])) best = s;
		if (best < 0 || res[best] < 1e-12) break;  /* residual norm below 1e-6 */
		used[best] = 1;
		double *qj = w->d_Q + (size_t)j * dim;
		cudaMemcpyAsync(qj, d_U + (size_t)best * dim, dim * sizeof(double), cudaMemcpyDeviceToDevice, q);
		for (int pass = 0; pass < 2 && j > 0; pass++) {
			ws_dots<<<j, WT, 0, q>>>(w->d_Q, dim, qj, 0, dim, d_c);
			ws_combine<<<g, 256, 0, q>>>(w->d_Q, dim, j, d_c, dim, qj, 1);
		}
		ws_dots<<<1, WT, 0, q>>>(qj, dim, qj, 0, dim, d_c);
		ws_scale<<<dim3(g, 1), 256, 0, q>>>(qj, dim, d_c, dim);
		ws_dots<<<S, WT, 0, q>>>(d_U, dim, qj, 0, dim, d_d);
		if (cudaMemcpyAsync(hd, d_d, S * sizeof(double), cudaMemcpyDeviceToHost, q) != cudaSuccess ||
		    cudaStreamSynchronize(q) != cudaSuccess) {
			st = jn_fail(JN_ERR_CUDA, "warm start: reduced basis");
			break;
		}
		for (int s = 0; s < S; s++) {
			T[(size_t)s * k + j] = hd[s];
			res[s] -= hd[s] * hd[s];
		}
		kk = j + 1;
	}
	if (!st && kk < 1) st = jn_fail(JN_ERR_INVALID, "warm start: the snapshots span nothing");
	/* a rank-deficient snapshot set gives a smaller basis: rebuild the MLP with kk outputs */
	if (!st && kk < k) {
		jn_mlp_destroy(w->mlp);
		w->mlp = NULL;
		st = jn_mlp_create(nc, hidden, kk, o->seed, &w->mlp);
	}
	w->k = kk;
	/* train on standardised couplings */
	float *X = NULL, *Y = NULL;
	if (!st) {
		for (int i = 0; i < nc; i++) {
			double m = 0.0, v = 0.0;
			for (int s = 0; s < S; s++) m += cpl[(size_t)s * nc + i];
			m /= S;
			for (int s = 0; s < S; s++) v += (cpl[(size_t)s * nc + i] - m) * (cpl[(size_t)s * nc + i] - m);
			v = sqrt(v / S);
			w->mean[i] = m;
			w->scale[i] = v > 1e-12 ? 1.0 / v : 1.0;
		}
		X = (float *)malloc((size_t)S * nc * sizeof(float));
		Y = (float *)malloc((size_t)S * kk * sizeof(float));
		for (int s = 0; s < S; s++) {
			for (int i = 0; i < nc; i++) X[(size_t)s * nc + i] = (float)((cpl[(size_t)s * nc + i] - w->mean[i]) * w->scale[i]);
			for (int j = 0; j < kk; j++) Y[(size_t)s * kk + j] = (float)T[(size_t)s * k + j];
		}
		st = jn_mlp_train(w->mlp, X, Y, S, steps, lr, final_loss);
	}
	free(X); free(Y);
	cudaFree(d_E); cudaFree(d_U); cudaFree(d_c); cudaFree(d_d);
	free(hr); free(hd); free(T); free(res); free(used);
	if (st) {
		jn_warm_start_destroy(w);
		return st;
	}
	*out = w;
	return JN_OK;
}

extern "C" jn_status jn_warm_start_vectors(jn_warm_start *w, int n, const double *cpl, double *const *vec)
{
	if (!w || !cpl || !vec || n < 1) return jn_fail(JN_ERR_INVALID, "bad argument");
	const int nc = w->nc, k = w->k;
	const int64_t dim = w->dim;
	float *X = (float *)malloc((size_t)n * nc * sizeof(float)), *Y = (float *)malloc((size_t)n * k * sizeof(float));
	double *C = (double *)malloc((size_t)n * k * sizeof(double));
	for (int s = 0; s < n; s++)
		for (int i = 0; i < nc; i++) X[(size_t)s * nc + i] = (float)((cpl[(size_t)s * nc + i] - w->mean[i]) * w->scale[i]);
	jn_status st = jn_mlp_predict(w->mlp, X, n, Y);
	/* unit coordinates: |Q y| = |y| for an orthonormal basis */
	for (int s = 0; s < n && !st; s++) {
		double n2 = 0.0;
		for (int j = 0; j < k; j++) n2 += (double)Y[(size_t)s * k + j] * Y[(size_t)s * k + j];
		const double inv = n2 > 0.0 ? 1.0 / sqrt(n2) : 0.0;
		for (int j = 0; j < k; j++) C[(size_t)s * k + j] = Y[(size_t)s * k + j] * inv;
	}
	double *d_C = NULL, *d_o = NULL;
	cudaStream_t q = w->mlp->stream;
	if (!st && (cudaMalloc((void **)&d_C, (size_t)n * k * sizeof(double)) != cudaSuccess ||
		    cudaMalloc((void **)&d_o, (size_t)n * dim * sizeof(double)) != cudaSuccess))
		st = jn_fail(JN_ERR_NOMEM, "warm start: %d vectors of dimension %lld", n, (long long)dim);
	if (!st && cudaMemcpyAsync(d_C, C, (size_t)n * k * sizeof(double), cudaMemcpyHostToDevice, q) != cudaSuccess)
		st = jn_fail(JN_ERR_CUDA, "warm start: upload");
	if (!st) {
		ws_expand<<<dim3(grid_for(dim), n), 256, 0, q>>>(w->d_Q, k, d_C, w->d_r, w->noise, dim, d_o);
		if (cudaGetLastError() != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "warm start: expansion launch");
	}
	for (int s = 0; s < n && !st; s++)
		if (vec[s] && cudaMemcpyAsync(vec[s], d_o + (size_t)s * dim, dim * sizeof(double), cudaMemcpyDeviceToHost, q) !=
				      cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "warm start: copy of vector %d", s);
	if (!st && cudaStreamSynchronize(q) != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "warm start: expansion");
	cudaFree(d_C);
	cudaFree(d_o);
	free(X); free(Y); free(C);
	return st;
}

extern "C" int jn_warm_start_basis_size(const jn_warm_start *w) { return w ? w->k : 0; }

extern "C" jn_status jn_warm_start_basis(const jn_warm_start *w, double *basis)
{
	if (!w || !basis) return jn_fail(JN_ERR_INVALID, "null argument");
	CUDA_TRY(cudaMemcpy(basis, w->d_Q, (size_t)w->k * w->dim * sizeof(double), cudaMemcpyDeviceToHost));
	return JN_OK;
}
