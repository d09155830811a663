/*
 * jn_transform3.cu — the J-scheme -> M-scheme three-body transform on the
 * GPU (Mercury's mercury_J_scheme_to_internal, three-body part) and its
 * C ABI.
 *
 * The host plan (jn_transform3.c) replaces the reference's dense
 * D_M = sum_J S_bra^T V_J S_ket per total-M block
 * (src/Neptune/block_transform/block_transform.c:147-356,
 * src/Neptune/matrix_transform/matrix_transform.c:431-486) by short
 * expansions of every M-scheme state.  Every three-body matrix element of
 * the combination table is the element of D_M of a (bra, ket) pair of
 * M-scheme states, evaluated as the reference's loops do: J_abc ascending,
 * then for each bra coupled state the sum over the ket's coupled states,
 *     d += (sum_a' fl(S_ket V[a][a'])) S_bra,   acc += d,
 * with separately rounded multiplies and adds.  The inner sums depend on
 * the energy block, the ket state, the slot and the bra's row a only, so
 * two launches share them across every bra of a ket:
 *   jn_jjj_inner_kernel  T = V(eb, J) s_ket over every row, once for each
 *                        (energy block, ket) pair the elements use and each
 *                        slot of the ket;
 *   jn_jjj_to_m_kernel   each element: d += fl(T[a] S_bra), acc += d, the
 *                        same operations in the same order.
 * On 6Li Nmax 4 this is 2.2x fewer FP64 multiply-adds than summing each
 * inner sum on the spot.
 *
 * Roofline: GB300's FP64 pipe (each multiply and add is its own FP64
 * instruction, as the reference rounds them); FP64 has no fast tensor-core
 * form on GB300, and the per-element form needs no GEMM.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include "jn_internal.h"
#include "jn_transform3.h"

struct jn_transform3 {
	jn_t3plan_t plan;
	int device;
	cudaStream_t stream;
	jn_t3block_t *d_tb;
	int32_t *d_chunk;               /* per 2^T3_CHUNK_SHIFT elements: the block of the first */
	jn_m3state_t *d_ms;
	jn_m3term_t *d_term;
	int64_t *d_voff;
	int32_t *d_vld;
	double *d_V;
	int32_t *d_cket, *d_cbra, *d_csign;
	jn_p3conn_t *d_pc;
	jn_nconn_t *d_nc;
	int32_t *d_lut;
	int32_t *d_epair;
	int64_t *d_pseg;
	jn_t3seg_t *d_seg;
	double *d_T;                    /* the shared inner sums */
	double *d_out;
	double *h_out;
	int have_out;
	double plan_seconds;
	int grid;
};

#define T3_CHUNK_SHIFT 6

/* Phase 1: the inner sums of every (energy block, ket) pair and slot, one
 * warp per segment, lanes over the rows of V:
 *     T[toff + v] = sum_r fl(S_r V[v][v_r])   (r over the ket's terms of the slot, in order) */
__global__ void __launch_bounds__(256) jn_jjj_inner_kernel(const jn_t3seg_t *__restrict__ seg, int64_t nseg,
							  const jn_m3term_t *__restrict__ term, const int64_t *__restrict__ voff,
							  const int32_t *__restrict__ vld, int nslots, const double *__restrict__ V,
							  double *__restrict__ T)
{
	const int lane = threadIdx.x & 31;
	const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
	for (int64_t g = w0; g < nseg; g += nw) {
		const jn_t3seg_t sg = seg[g];
		if (sg.toff < 0) continue;
		const int64_t vi = (int64_t)sg.eb * nslots + sg.slot;
		const double *Vs = V + voff[vi];
		const int64_t ld = vld[vi];
		for (int v = lane; v < sg.rows; v += 32) {
			const double *row = Vs + (int64_t)v * ld;
			double inner = 0.0;
			for (int r = sg.term0; r < sg.term0 + sg.nterm; r++) {
				const jn_m3term_t tk = term[r];
				inner = __dadd_rn(inner, __dmul_rn(tk.s, row[tk.v]));
			}
			T[sg.toff + v] = inner;
		}
	}
}

/* Phase 2: every element from the inner sums of its (energy block, ket)
 * pair: J_abc ascending, for each slot the bra's coupled states in order,
 *     d += fl(T[v_bra] S_bra),   acc += d,
 * the same separately rounded operations, in the same order, as summing
 * each inner sum on the spot. */
__global__ void __launch_bounds__(256) jn_jjj_to_m_kernel(
	const jn_t3block_t *__restrict__ tb, const int32_t *__restrict__ chunk_block, int n3, int64_t nelem, const jn_m3state_t *__restrict__ ms,
	const jn_m3term_t *__restrict__ term, const int32_t *__restrict__ elem_pair, const int64_t *__restrict__ pair_seg,
	const jn_t3seg_t *__restrict__ seg, const double *__restrict__ T, const int32_t *__restrict__ cket,
	const int32_t *__restrict__ cbra, const int32_t *__restrict__ csign, const jn_p3conn_t *__restrict__ pc,
	const jn_nconn_t *__restrict__ nc, const int32_t *__restrict__ lut, double *__restrict__ out)
{
	for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nelem;
	     e += (int64_t)gridDim.x * blockDim.x) {
		/* the block holding element e: from the block of its chunk's first
		   element, forward over the blocks that start inside the chunk */
		int lo = chunk_block[e >> T3_CHUNK_SHIFT];
		while (lo + 1 < n3 && tb[lo + 1].out <= e) lo++;
		const jn_t3block_t b = tb[lo];
		const int64_t i = e - b.out;
		int32_t ket, bra;
		int neg;
		if (b.kind == 0) {
			ket = cket[b.conn + i];
			bra = cbra[b.conn + i];
			neg = csign[b.conn + i] < 0;
		} else {
			const int64_t kp = i / b.nn, kn = i - kp * b.nn;
			const jn_p3conn_t p = pc[b.conn + kp];
			const jn_nconn_t n = nc[b.nconn + kn];
			int32_t k = lut[p.ket_lut + (int64_t)p.p_ann * p.ket_nn + n.n_ann];
			int32_t r = lut[p.bra_lut + (int64_t)p.p_cre * p.bra_nn + n.n_cre];
			neg = 0;
			if (k < 0) { k = -k - 1; neg ^= 1; }
			if (r < 0) { r = -r - 1; neg ^= 1; }
			ket = k;
			bra = r;
		}
		const jn_m3state_t K = ms[ket], B = ms[bra];
		const int jlo = max((int)K.jlo, (int)B.jlo), jhi = min((int)K.jhi, (int)B.jhi);
		const int32_t pr = elem_pair[e];
		int64_t j = pair_seg[pr];
		const int64_t j1 = pair_seg[pr + 1];
		int ib = B.ent;
		const int eb = B.ent + B.nent;
		double acc = 0.0;
		while (j < j1 && ib < eb) {
			const jn_t3seg_t sg = seg[j];
			const int sb = term[ib].slot;
			if (sg.slot < sb) { j++; continue; }
			int gb = ib;
			while (gb < eb && term[gb].slot == sb) gb++;
			if (sb < sg.slot) { ib = gb; continue; }
			if (sb >= jlo && sb <= jhi && sg.toff >= 0) {
				const double *Tr = T + sg.toff;
				double d = 0.0;
				for (int q = ib; q < gb; q++) {
					const jn_m3term_t tbq = term[q];
					d = __dadd_rn(d, __dmul_rn(Tr[tbq.v], tbq.s));
				}
				acc = __dadd_rn(acc, d);
			}
			j++;
			ib = gb;
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

extern "C" void jn_transform3_close(jn_transform3 *t)
{
	if (!t) return;
	cudaFree(t->d_tb); cudaFree(t->d_chunk); cudaFree(t->d_ms); cudaFree(t->d_term); cudaFree(t->d_voff); cudaFree(t->d_vld);
	cudaFree(t->d_V); cudaFree(t->d_cket); cudaFree(t->d_cbra); cudaFree(t->d_csign); cudaFree(t->d_pc);
	cudaFree(t->d_nc); cudaFree(t->d_lut); cudaFree(t->d_out);
	cudaFree(t->d_epair); cudaFree(t->d_pseg); cudaFree(t->d_seg); cudaFree(t->d_T);
	if (t->stream) cudaStreamDestroy(t->stream);
	free(t->h_out);
	jn_t3plan_free(&t->plan);
	free(t);
}

extern "C" jn_status jn_transform3_open(const char *comb, const char *lists_dir, int Z, int N, int emax,
					const char *jscheme_dir, jn_transform3 **out)
{
	if (!comb || !lists_dir || !jscheme_dir || !out) return jn_fail(JN_ERR_INVALID, "null argument");
	*out = NULL;
	jn_transform3 *t = (jn_transform3 *)calloc(1, sizeof *t);
	if (!t) return jn_fail(JN_ERR_NOMEM, "out of memory");
	struct timespec a, b;
	clock_gettime(CLOCK_MONOTONIC, &a);
	char err[1024] = "";
	if (jn_t3plan_build(&t->plan, comb, lists_dir, Z, N, emax, jscheme_dir, err, sizeof err)) {
		free(t);
		return jn_fail(strstr(err, "Could not open") ? JN_ERR_IO : JN_ERR_FORMAT, "%s", err);
	}
	if (jn_t3plan_shared(&t->plan, err, sizeof err)) {
		jn_t3plan_free(&t->plan);
		free(t);
		return jn_fail(JN_ERR_NOMEM, "%s", err);
	}
	clock_gettime(CLOCK_MONOTONIC, &b);
	t->plan_seconds = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
	const jn_t3plan_t *p = &t->plan;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		jn_transform3_close(t);
		return jn_fail(JN_ERR_CUDA, "no CUDA device");
	}
	cudaGetDevice(&t->device);
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t->device);
	jn_status s = JN_OK;
	if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) s = jn_fail(JN_ERR_CUDA, "stream");
	if (!s) s = up(&t->d_tb, p->tb, p->n3);
	if (!s) {
		const int64_t nch = ((p->nelem ? p->nelem : 1) + (1 << T3_CHUNK_SHIFT) - 1) >> T3_CHUNK_SHIFT;
		int32_t *cb = (int32_t *)malloc(nch * sizeof(int32_t));
		if (!cb) s = jn_fail(JN_ERR_NOMEM, "out of memory");
		for (int64_t c = 0, b = 0; !s && c < nch; c++) {
			const int64_t e = c << T3_CHUNK_SHIFT;
			while (b + 1 < p->n3 && p->tb[b + 1].out <= e) b++;
			cb[c] = (int32_t)b;
		}
		if (!s) s = up(&t->d_chunk, cb, (size_t)nch);
		free(cb);
	}
	if (!s) s = up(&t->d_ms, p->ms, p->nms);
	if (!s) s = up(&t->d_term, p->term, p->nterm);
	if (!s) s = up(&t->d_voff, p->voff, (size_t)p->neb * p->nslots);
	if (!s) s = up(&t->d_vld, p->vld, (size_t)p->neb * p->nslots);
	if (!s) s = up(&t->d_V, p->V, p->nv);
	if (!s) s = up(&t->d_cket, p->conn_ket, p->nconn0);
	if (!s) s = up(&t->d_cbra, p->conn_bra, p->nconn0);
	if (!s) s = up(&t->d_csign, p->conn_sign, p->nconn0);
	if (!s) s = up(&t->d_pc, p->pc, p->npc);
	if (!s) s = up(&t->d_nc, p->nc, p->nnc);
	if (!s) s = up(&t->d_lut, p->lut, p->nlut);
	if (!s) s = up(&t->d_out, (const double *)NULL, (size_t)p->nelem);
	if (!s) s = up(&t->d_epair, p->elem_pair, (size_t)p->nelem);
	if (!s) s = up(&t->d_pseg, p->pair_seg, (size_t)p->npairs + 1);
	if (!s) s = up(&t->d_seg, p->seg, (size_t)p->nseg);
	if (!s) s = up(&t->d_T, (const double *)NULL, (size_t)p->nT);
	if (s) { jn_transform3_close(t); return s; }
	int64_t g = (p->nelem + 255) / 256;
	int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
	t->grid = (int)(g < 1 ? 1 : (g > cap ? cap : g));
	*out = t;
	return JN_OK;
}

static jn_status enqueue(jn_transform3 *t, cudaStream_t st)
{
	const jn_t3plan_t *p = &t->plan;
	if (p->nseg) {
		int64_t g = (p->nseg * 32 + 255) / 256;
		if (g > (int64_t)t->grid * 4) g = (int64_t)t->grid * 4;
		jn_jjj_inner_kernel<<<(int)(g < 1 ? 1 : g), 256, 0, st>>>(t->d_seg, p->nseg, t->d_term, t->d_voff, t->d_vld,
									  p->nslots, t->d_V, t->d_T);
	}
	if (p->nelem)
		jn_jjj_to_m_kernel<<<t->grid, 256, 0, st>>>(t->d_tb, t->d_chunk, p->n3, p->nelem, t->d_ms, t->d_term, t->d_epair,
							   t->d_pseg, t->d_seg, t->d_T, t->d_cket, t->d_cbra, t->d_csign,
							   t->d_pc, t->d_nc, t->d_lut, t->d_out);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "three-body transform launch: %s", cudaGetErrorString(e));
	t->have_out = 0;
	return JN_OK;
}

extern "C" jn_status jn_transform3_run(jn_transform3 *t, void *stream)
{
	if (!t) return jn_fail(JN_ERR_INVALID, "null argument");
	return enqueue(t, stream ? (cudaStream_t)stream : t->stream);
}

extern "C" jn_status jn_transform3_profile(jn_transform3 *t, float *ms)
{
	if (!t || !ms) return jn_fail(JN_ERR_INVALID, "null argument");
	cudaEvent_t a, b;
	CUDA_TRY(cudaEventCreate(&a));
	CUDA_TRY(cudaEventCreate(&b));
	CUDA_TRY(cudaEventRecord(a, t->stream));
	jn_status s = enqueue(t, t->stream);
	if (!s) {
		CUDA_TRY(cudaEventRecord(b, t->stream));
		CUDA_TRY(cudaEventSynchronize(b));
		CUDA_TRY(cudaEventElapsedTime(ms, a, b));
	}
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	return s;
}

static jn_status fetch(jn_transform3 *t)
{
	const jn_t3plan_t *p = &t->plan;
	if (t->have_out) return JN_OK;
	CUDA_TRY(cudaStreamSynchronize(t->stream));
	if (!t->h_out) t->h_out = (double *)malloc((p->nelem ? p->nelem : 1) * sizeof(double));
	if (!t->h_out) return jn_fail(JN_ERR_NOMEM, "out of memory");
	CUDA_TRY(cudaMemcpy(t->h_out, t->d_out, p->nelem * sizeof(double), cudaMemcpyDeviceToHost));
	t->have_out = 1;
	return JN_OK;
}

extern "C" jn_status jn_transform3_elements(jn_transform3 *t, int block_id, double *host_out, size_t capacity,
					    size_t *count)
{
	if (!t || !count) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_t3plan_t *p = &t->plan;
	for (int i = 0; i < p->n3; i++)
		if (p->info[p->tb_info[i]].id == block_id) {
			*count = (size_t)p->tb[i].count;
			if (!host_out) return JN_OK;
			if (capacity < *count) return jn_fail(JN_ERR_INVALID, "capacity %zu < %zu", capacity, *count);
			jn_status s = fetch(t);
			if (s) return s;
			memcpy(host_out, t->h_out + p->tb[i].out, *count * sizeof(double));
			return JN_OK;
		}
	return jn_fail(JN_ERR_INVALID, "block %d is not a three-body matrix-element block", block_id);
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

extern "C" jn_status jn_transform3_write(jn_transform3 *t, const char *dir)
{
	if (!t || !dir) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_t3plan_t *p = &t->plan;
	mkdir(dir, 0755);
	jn_status s = enqueue(t, t->stream);
	if (!s) s = fetch(t);
	for (int i = 0; i < p->n3 && !s; i++) s = write_block(dir, &p->info[p->tb_info[i]], t->h_out + p->tb[i].out, p->tb[i].count);
	return s;
}

extern "C" jn_status jn_transform3_get_stats(const jn_transform3 *t, jn_transform3_stats *st)
{
	if (!t || !st) return jn_fail(JN_ERR_INVALID, "null argument");
	const jn_t3plan_t *p = &t->plan;
	memset(st, 0, sizeof *st);
	st->num_three_body_blocks = p->n3;
	st->num_elements = (size_t)p->nelem;
	st->num_states = (size_t)p->nms;
	st->num_terms = (size_t)p->nterm;
	st->num_coupled_states = (size_t)p->coupled_states;
	st->num_m_blocks = (size_t)p->mblocks;
	st->file_states = (size_t)p->file_states;
	st->file_elements = (size_t)p->file_elements;
	st->v_entries = (size_t)p->nv;
	st->dense_flops = p->dense_flops;
	/* compulsory traffic of one launch: elements written, connection records,
	   LUT, state records with their terms, V and its tables, block records */
	st->algorithmic_bytes = 8.0 * p->nelem + 12.0 * p->nconn0 + sizeof(jn_p3conn_t) * (double)p->npc +
				sizeof(jn_nconn_t) * (double)p->nnc + 4.0 * p->nlut + sizeof(jn_m3state_t) * (double)p->nms +
				sizeof(jn_m3term_t) * (double)p->nterm + 8.0 * p->nv + 12.0 * (double)p->neb * p->nslots +
				sizeof(jn_t3block_t) * (double)p->n3;
	st->plan_seconds = t->plan_seconds;
	return JN_OK;
}

extern "C" jn_status jn_transform_3nf(const char *comb, const char *lists_dir, const char *output_dir, int Z, int N,
				      int emax, const char *jscheme_dir)
{
	jn_transform3 *t = NULL;
	jn_status s = jn_transform3_open(comb, lists_dir, Z, N, emax, jscheme_dir, &t);
	if (s) return s;
	s = jn_transform3_write(t, output_dir);
	jn_transform3_close(t);
	return s;
}
