/*
 * jn_transform.cu — the J-scheme -> M-scheme two-body transform on the GPU
 * (Mercury's mercury_J_scheme_to_internal, two-body part) and its C ABI.
 *
 * The host plan (jn_transform.c) reduces the reference's dense
 * S_bra^T V_JT S_ket decoupling to one short sum per matrix element,
 * because every M-scheme pair state overlaps exactly one coupled state per
 * (J, T).  jn_jt_to_m_kernel computes every two-body matrix element of the
 * combination table in one launch: it decodes the element's connection into
 * a (bra, ket) pair of M-scheme pair states and sums
 *     fl(fl(S_ket * V) * S_bra)
 * over (J, T) in the reference's loop order (J ascending, then T), with
 * separately rounded multiplies and adds, which is exactly the arithmetic
 * of transform_matrix and accumulate_matrix
 * (src/Neptune/matrix_transform/matrix_transform.c:30-46, 431-486).
 *
 * Roofline: the kernel writes 8 bytes per element and reads a 4- or
 * 8-byte connection record per element; the expansion tables and the
 * interaction (a few MB) stay in L2.  It is bound by HBM writes and L2
 * gathers, not by arithmetic (at most 2 (2 j_max + 1) multiply pairs per
 * element), so it runs on the FP64 pipe, not on tensor cores.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include "jn_internal.h"
#include "jn_transform.h"

struct jn_transform {
	jn_tplan_t plan;
	int device;
	cudaStream_t stream;
	jn_tblock_t *d_tb;
	jn_mstate_t *d_ms;
	double *d_cs;
	int32_t *d_ca;
	int32_t *d_cket, *d_cbra, *d_csign;
	jn_pconn_t *d_pc;
	jn_nconn_t *d_nc;
	int32_t *d_lut;
	double *d_V;
	int64_t *d_cfg_first;
	int32_t *d_cfg_end;
	double *d_out;
	double *h_out;
	int have_out;
	double plan_seconds;
	int grid;
};

__global__ void __launch_bounds__(256) jn_jt_to_m_kernel(
	const jn_tblock_t *__restrict__ tb, int n2, int64_t nelem, const jn_mstate_t *__restrict__ ms,
	const double *__restrict__ cs, const int32_t *__restrict__ ca, const int32_t *__restrict__ cket,
	const int32_t *__restrict__ cbra, const int32_t *__restrict__ csign, const jn_pconn_t *__restrict__ pc,
	const jn_nconn_t *__restrict__ nc, const int32_t *__restrict__ lut, const double *__restrict__ V,
	int64_t nconfig, const int64_t *__restrict__ cfg_first, const int32_t *__restrict__ cfg_end,
	double *__restrict__ out)
{
	for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nelem;
	     e += (int64_t)gridDim.x * blockDim.x) {
		/* the block holding element e (blocks are stored in output order) */
		int lo = 0, hi = n2 - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (tb[mid].out <= e) lo = mid; else hi = mid - 1;
		}
		const jn_tblock_t b = tb[lo];
		const int64_t i = e - b.out;
		int32_t ket, bra;
		int neg;
		if (b.kind == 0) {
			ket = cket[b.conn + i];
			bra = cbra[b.conn + i];
			neg = csign[b.conn + i] < 0;
		} else {
			const int64_t kp = i / b.nn, kn = i - kp * b.nn;
			const jn_pconn_t p = pc[b.conn + kp];
			const jn_nconn_t n = nc[b.nconn + kn];
			int32_t k = lut[p.ket_lut + (int64_t)p.p_ann * p.ket_nn + n.n_ann];
			int32_t r = lut[p.bra_lut + (int64_t)p.p_cre * p.bra_nn + n.n_cre];
			neg = 0;
			if (k < 0) { k = -k - 1; neg ^= 1; }
			if (r < 0) { r = -r - 1; neg ^= 1; }
			ket = k;
			bra = r;
		}
		const jn_mstate_t K = ms[ket], B = ms[bra];
		const int jlo = max((int)K.jlo, (int)B.jlo);
		const int jhi = min((int)K.jlo + (int)K.nj, (int)B.jlo + (int)B.nj) - 1;
		const double *Vt = V + (int64_t)b.tz * nconfig;
		double acc = 0.0;
		for (int J = jlo; J <= jhi; J++) {
			const int ik = K.coef + 2 * (J - K.jlo), ib = B.coef + 2 * (J - B.jlo);
#pragma unroll
			for (int T = 0; T < 2; T++) {
				const int32_t ak = ca[ik + T], ab = ca[ib + T];
				if (ak < 0 || ab < 0) continue;
				const int a0 = min(ak, ab), a1 = max(ak, ab);
				const double v = a1 < cfg_end[a0] ? Vt[cfg_first[a0] + (a1 - a0)] : 0.0;
				acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(cs[ik + T], v), cs[ib + T]));
			}
		}
		out[e] = neg ? -acc : acc;
	}
}

template <typename T>
static jn_status up(T **d, const T *h, size_t n)
{
	*d = NULL;
	cudaError_t e = cudaMalloc((void **)d, (n ? n : 1) * sizeof(T));
	if (e == cudaSuccess && n && h) e = cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return jn_fail(JN_ERR_NOMEM, "transform upload of %zu bytes: %s", n * sizeof(T), cudaGetErrorString(e));
	return JN_OK;
}

extern "C" void jn_transform_close(jn_transform *t)
{
	if (!t) return;
	cudaFree(t->d_tb); cudaFree(t->d_ms); cudaFree(t->d_cs); cudaFree(t->d_ca); cudaFree(t->d_cket);
	cudaFree(t->d_cbra); cudaFree(t->d_csign); cudaFree(t->d_pc); cudaFree(t->d_nc); cudaFree(t->d_lut);
	cudaFree(t->d_V); cudaFree(t->d_cfg_first); cudaFree(t->d_cfg_end); cudaFree(t->d_out);
	if (t->stream) cudaStreamDestroy(t->stream);
	free(t->h_out);
	jn_tplan_free(&t->plan);
	free(t);
}

extern "C" jn_status jn_transform_open(const char *comb, const char *lists_dir, int Z, int N, int e1, int e2,
				       const char *antoine, int include_kinetic, jn_transform **out)
{
	if (!comb || !lists_dir || !antoine || !out) return jn_fail(JN_ERR_INVALID, "null argument");
	*out = NULL;
	jn_transform *t = (jn_transform *)calloc(1, sizeof *t);
	if (!t) return jn_fail(JN_ERR_NOMEM, "out of memory");
	struct timespec a, b;
	clock_gettime(CLOCK_MONOTONIC, &a);
	char err[1024] = "";
	if (jn_tplan_build(&t->plan, comb, lists_dir, Z, N, e1, e2, antoine, include_kinetic, err, sizeof err)) {
		free(t);
		return jn_fail(strstr(err, "Could not open") ? JN_ERR_IO : JN_ERR_FORMAT, "%s", err);
	}
	clock_gettime(CLOCK_MONOTONIC, &b);
	t->plan_seconds = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
	const jn_tplan_t *p = &t->plan;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		jn_transform_close(t);
		return jn_fail(JN_ERR_CUDA, "no CUDA device");
	}
	cudaGetDevice(&t->device);
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t->device);
	jn_status s = JN_OK;
	if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) s = jn_fail(JN_ERR_CUDA, "stream");
	if (!s) s = up(&t->d_tb, p->tb, p->n2);
	if (!s) s = up(&t->d_ms, p->ms, p->nms);
	if (!s) s = up(&t->d_cs, p->coef_s, p->ncoef);
	if (!s) s = up(&t->d_ca, p->coef_a, p->ncoef);
	if (!s) s = up(&t->d_cket, p->conn_ket, p->nconn1);
	if (!s) s = up(&t->d_cbra, p->conn_bra, p->nconn1);
	if (!s) s = up(&t->d_csign, p->conn_sign, p->nconn1);
	if (!s) s = up(&t->d_pc, p->pc, p->npc);
	if (!s) s = up(&t->d_nc, p->nc, p->nnc);
	if (!s) s = up(&t->d_lut, p->lut, p->nlut);
	if (!s) s = up(&t->d_V, p->V, (size_t)3 * p->jt.nconfig);
	if (!s) s = up(&t->d_cfg_first, p->jt.cfg_first, (size_t)p->jt.n);
	if (!s) s = up(&t->d_cfg_end, (const int32_t *)p->jt.cfg_end, (size_t)p->jt.n);
	if (!s) s = up(&t->d_out, (const double *)NULL, (size_t)p->nelem);
	if (s) { jn_transform_close(t); return s; }
	int64_t g = (p->nelem + 255) / 256;
	int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
	t->grid = (int)(g < 1 ? 1 : (g > cap ? cap : g));
	*out = t;
	return JN_OK;
}

static jn_status enqueue(jn_transform *t, cudaStream_t st)
{
	const jn_tplan_t *p = &t->plan;
	if (p->nelem)
		jn_jt_to_m_kernel<<<t->grid, 256, 0, st>>>(t->d_tb, p->n2, p->nelem, t->d_ms, t->d_cs, t->d_ca, t->d_cket,
							  t->d_cbra, t->d_csign, t->d_pc, t->d_nc, t->d_lut, t->d_V,
							  p->jt.nconfig, t->d_cfg_first, t->d_cfg_end, t->d_out);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "transform kernel launch: %s", cudaGetErrorString(e));
	t->have_out = 0;
	return JN_OK;
}

extern "C" jn_status jn_transform_run(jn_transform *t, void *stream)
{
	if (!t) return jn_fail(JN_ERR_INVALID, "null argument");
	return enqueue(t, stream ? (cudaStream_t)stream : t->stream);
}

extern "C" jn_status jn_transform_profile(jn_transform *t, float *ms)
{
	if (!t || !ms) return jn_fail(JN_ERR_INVALID, "null argument");
	cudaEvent_t a, b;
	CUDA_TRY(cudaEventCreate(&a));
	CUDA_TRY(cudaEventCreate(&b));
	CUDA_TRY(cudaEventRecord(a, t->stream));
	jn_status s = enqueue(t, t->stream);
	if (s) return s;
	CUDA_TRY(cudaEventRecord(b, t->stream));
	CUDA_TRY(cudaEventSynchronize(b));
	CUDA_TRY(cudaEventElapsedTime(ms, a, b));
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	return JN_OK;
}

static jn_status fetch(jn_transform *t)
{
	const jn_tplan_t *p = &t->plan;
	if (t->have_out) return JN_OK;
	CUDA_TRY(cudaStreamSynchronize(t->stream));
	if (!t->h_out) t->h_out = (double *)malloc((p->nelem ? p->nelem : 1) * sizeof(double));
	if (!t->h_out) return jn_fail(JN_ERR_NOMEM, "out of memory");
	CUDA_TRY(cudaMemcpy(t->h_out, t->d_out, p->nelem * sizeof(double), cudaMemcpyDeviceToHost));
	t->have_out = 1;
	return JN_OK;
}

extern "C" jn_status jn_transform_elements(jn_transform *t, int block_id, double *host_out, size_t capacity,
					   size_t *count)
{
	if (!t || !count) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_tplan_t *p = &t->plan;
	for (int i = 0; i < p->n1; i++)
		if (p->info[p->z1_info[i]].id == block_id) {
			*count = (size_t)p->z1_count[i];
			if (host_out && capacity < *count) return jn_fail(JN_ERR_INVALID, "capacity %zu < %zu", capacity, *count);
			if (host_out) memset(host_out, 0, *count * sizeof(double));
			return JN_OK;
		}
	for (int i = 0; i < p->n2; i++)
		if (p->info[p->tb_info[i]].id == block_id) {
			*count = (size_t)p->tb[i].count;
			if (!host_out) return JN_OK;
			if (capacity < *count) return jn_fail(JN_ERR_INVALID, "capacity %zu < %zu", capacity, *count);
			jn_status s = fetch(t);
			if (s) return s;
			memcpy(host_out, t->h_out + p->tb[i].out, *count * sizeof(double));
			return JN_OK;
		}
	return jn_fail(JN_ERR_INVALID, "block %d is not a one- or two-body matrix-element block", block_id);
}

/* <dir>/<id>_matrix_elements: size_t n_dim, size_t p_dim, double[]
 * (src/Mercury/mercury_matrix_block/mercury_matrix_block.c:106-179) */
static jn_status write_block(const char *dir, const jn_meblock_info_t *b, const double *x, int64_t n)
{
	char path[8192];
	snprintf(path, sizeof path, "%s/%d_matrix_elements", dir, b->id);
	FILE *f = fopen(path, "wb");
	if (!f) return jn_fail(JN_ERR_IO, "Could not open file %s for writing", path);
	size_t hdr[2] = { (size_t)b->Nn, (size_t)b->Np };
	int bad = fwrite(hdr, sizeof(size_t), 2, f) != 2;
	if (!bad && n) bad = fwrite(x, sizeof(double), (size_t)n, f) != (size_t)n;
	if (fclose(f) || bad) return jn_fail(JN_ERR_IO, "Could not write %s", path);
	return JN_OK;
}

extern "C" jn_status jn_transform_write(jn_transform *t, const char *dir)
{
	if (!t || !dir) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_tplan_t *p = &t->plan;
	mkdir(dir, 0755);
	jn_status s = enqueue(t, t->stream);
	if (!s) s = fetch(t);
	for (int i = 0; i < p->n2 && !s; i++) s = write_block(dir, &p->info[p->tb_info[i]], t->h_out + p->tb[i].out, p->tb[i].count);
	if (!s && p->n1) {
		int64_t mx = 0;
		for (int i = 0; i < p->n1; i++) mx = p->z1_count[i] > mx ? p->z1_count[i] : mx;
		double *z = (double *)calloc(mx ? mx : 1, sizeof(double));
		for (int i = 0; i < p->n1 && !s; i++) s = write_block(dir, &p->info[p->z1_info[i]], z, p->z1_count[i]);
		free(z);
	}
	return s;
}

extern "C" jn_status jn_transform_get_stats(const jn_transform *t, jn_transform_stats *st)
{
	if (!t || !st) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_tplan_t *p = &t->plan;
	memset(st, 0, sizeof *st);
	st->num_two_body_blocks = p->n2;
	st->num_one_body_blocks = p->n1;
	st->num_elements = (size_t)p->nelem;
	st->num_pair_states = (size_t)p->nms;
	st->num_configurations = (size_t)p->jt.nconfig;
	st->dense_flops = p->dense_flops;
	/* compulsory traffic of one launch: elements written, connection records,
	   pair states with their expansions, interaction and configuration index */
	st->algorithmic_bytes = 8.0 * p->nelem + 12.0 * p->nconn1 + sizeof(jn_pconn_t) * (double)p->npc +
				sizeof(jn_nconn_t) * (double)p->nnc + 4.0 * p->nlut + sizeof(jn_mstate_t) * (double)p->nms +
				12.0 * p->ncoef + 24.0 * p->jt.nconfig + 12.0 * p->jt.n + sizeof(jn_tblock_t) * (double)p->n2;
	st->plan_seconds = t->plan_seconds;
	return JN_OK;
}

extern "C" jn_status jn_transform_2nf(const char *comb, const char *lists_dir, const char *output_dir, int Z, int N,
				      int e1, int e2, const char *antoine, int include_kinetic)
{
	jn_transform *t = NULL;
	jn_status s = jn_transform_open(comb, lists_dir, Z, N, e1, e2, antoine, include_kinetic, &t);
	if (s) return s;
	s = jn_transform_write(t, output_dir);
	jn_transform_close(t);
	return s;
}

extern "C" double jn_clebsch_gordan(int j1, int j2, int j3, int m1, int m2, int m3)
{
	return jn_cg(j1, j2, j3, m1, m2, m3);
}
