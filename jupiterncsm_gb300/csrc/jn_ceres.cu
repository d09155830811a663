/*
 * jn_ceres.cu — subspace matrices of training vectors (the reference's
 * Ceres, src/Ceres/programs/ceres.c:17-80): the norm matrix
 * N_ij = <v_i|v_j> (src/Ceres/norm_matrix/norm_matrix.c:4-28) and the
 * projected operator O_ij = <v_j|H v_i>
 * (src/Ceres/subspace_operator/subspace_operator.c:7-61), both symmetric
 * with the upper triangle computed, written as .npy files
 * (src/Ceres/numpy_matrix/numpy_matrix.c:7-35).
 *
 * GB300 organisation: the training vectors are uploaded once, the products
 * H v_i run on the context's engine, and each matrix element is one CTA's
 * fixed-order dot product, so the matrices repeat bit for bit.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jn_internal.h"
#include "jn_tridiag.cuh"

#define CT 256

/* element (i, j) = blockIdx.{x, y}, j >= i: a_i . b_j (b_j = a_j for the norm matrix) */
__global__ void __launch_bounds__(CT) jn_subspace_gram(const double *__restrict__ A, const double *__restrict__ Bm,
						       int64_t D, int n, double *__restrict__ out)
{
	__shared__ double sh[CT];
	const int i = blockIdx.x, j = blockIdx.y;
	if (j < i) return;
	const double *a = A + (int64_t)i * D, *b = Bm + (int64_t)j * D;
	double s = 0.0;
	for (int64_t e = threadIdx.x; e < D; e += CT) s = fma(a[e], b[e], s);
	s = jn_block_sum(s, sh);
	if (threadIdx.x == 0) {
		out[(int64_t)i * n + j] = s;
		out[(int64_t)j * n + i] = s;
	}
}

extern "C" jn_status jn_subspace_matrices(jn_ctx *c, int n, const double *const *vectors, double *norm, double *op)
{
	if (!c || n < 1 || !vectors || (!norm && !op)) return jn_fail(JN_ERR_INVALID, "bad argument");
	if (n > 4096) return jn_fail(JN_ERR_INVALID, "%d training vectors: at most 4096", n);
	for (int i = 0; i < n; i++)
		if (!vectors[i]) return jn_fail(JN_ERR_INVALID, "vectors[%d] is NULL", i);
	const int64_t D = c->plan.dim;
	double *dV = NULL, *dHV = NULL, *dM = NULL;
	jn_status st = JN_OK;
	cudaStream_t q = c->stream;
	if (cudaMalloc((void **)&dV, (size_t)n * D * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&dHV, (size_t)n * D * sizeof(double)) != cudaSuccess ||
	    cudaMalloc((void **)&dM, (size_t)2 * n * n * sizeof(double)) != cudaSuccess)
		st = jn_fail(JN_ERR_NOMEM, "%d training vectors of dimension %lld do not fit", n, (long long)D);
	for (int i = 0; i < n && !st; i++)
		if (cudaMemcpyAsync(dV + (size_t)i * D, vectors[i], D * sizeof(double), cudaMemcpyHostToDevice, q) != cudaSuccess)
			st = jn_fail(JN_ERR_CUDA, "upload of training vector %d", i);
	for (int i = 0; i < n && !st && op; i++)
		st = jn_launch_matvec(c, dV + (size_t)i * D, dHV + (size_t)i * D, 0, q);
	if (!st) {
		if (norm) jn_subspace_gram<<<dim3(n, n), CT, 0, q>>>(dV, dV, D, n, dM);
		if (op) jn_subspace_gram<<<dim3(n, n), CT, 0, q>>>(dHV, dV, D, n, dM + (size_t)n * n);
		if (cudaGetLastError() != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "subspace matrices launch");
	}
	if (!st && norm && cudaMemcpyAsync(norm, dM, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, q) != cudaSuccess)
		st = jn_fail(JN_ERR_CUDA, "norm matrix copy");
	if (!st && op &&
	    cudaMemcpyAsync(op, dM + (size_t)n * n, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, q) != cudaSuccess)
		st = jn_fail(JN_ERR_CUDA, "operator matrix copy");
	if (!st && cudaStreamSynchronize(q) != cudaSuccess) st = jn_fail(JN_ERR_CUDA, "subspace matrices");
	cudaFree(dV);
	cudaFree(dHV);
	cudaFree(dM);
	return st;
}

/* the reference's .npy layout: version 1.0, the dictionary padded with
 * spaces by 64 - (length mod 8) bytes and ended by a newline.  The reference
 * stores the header length as the constant 118, right only while the header
 * fits 128 bytes (matrices below 100 x 100); the length written here is the
 * actual one, so larger matrices load too and smaller ones are byte-identical. */
static jn_status save_npy(const char *path, const double *m, int n)
{
	FILE *f = fopen(path, "wb");
	if (!f) return jn_fail(JN_ERR_IO, "Could not open file \"%s\" for writing", path);
	char header[512];
	size_t len = (size_t)snprintf(header, sizeof header,
				      "\x93NUMPY\x01%c__{'descr': '<f8', 'fortran_order': False, 'shape': (%d, %d), }", 0, n, n);
	const size_t pad = 64 - len % 8;
	memset(header + len, ' ', pad);
	len += pad;
	header[len - 1] = 0x0a;
	header[8] = (char)((len - 10) & 0xff);
	header[9] = (char)((len - 10) >> 8);
	jn_status st = JN_OK;
	if (fwrite(header, 1, len, f) != len || fwrite(m, sizeof(double), (size_t)n * n, f) != (size_t)n * n)
		st = jn_fail(JN_ERR_IO, "Could not write %s", path);
	fclose(f);
	return st;
}

extern "C" jn_status jn_ceres_files(jn_ctx *c, int n, const char *const *vector_dirs, const char *norm_matrix_path,
				    const char *subspace_operator_path)
{
	if (!c || n < 1 || !vector_dirs || (!norm_matrix_path && !subspace_operator_path))
		return jn_fail(JN_ERR_INVALID, "bad argument");
	const jn_plan_t *p = &c->plan;
	const int64_t D = p->dim;
	double *V = (double *)malloc((size_t)n * D * sizeof(double));
	double **rows = (double **)malloc((size_t)n * sizeof(double *));
	double *N = (double *)malloc((size_t)n * n * sizeof(double)), *O = (double *)malloc((size_t)n * n * sizeof(double));
	jn_status st = V && rows && N && O ? JN_OK : jn_fail(JN_ERR_NOMEM, "out of host memory");
	/* training vectors as Bacchus stores them: <dir>/vec_<block id> (src/Bacchus/vector/vector.c:538-555) */
	for (int i = 0; i < n && !st; i++) {
		rows[i] = V + (size_t)i * D;
		for (int b = 0; b < p->nblocks && !st; b++) {
			const jn_block_t *B = &p->blocks[b];
			char path[8192];
			snprintf(path, sizeof path, "%s/vec_%d", vector_dirs[i], B->id);
			FILE *f = fopen(path, "rb");
			const size_t len = (size_t)(B->Np * B->Nn);
			if (!f) { st = jn_fail(JN_ERR_IO, "Could not open vector block file %s", path); break; }
			if (fread(rows[i] + B->offset, sizeof(double), len, f) != len)
				st = jn_fail(JN_ERR_IO, "Could not read elements of block %d in %s", B->id, vector_dirs[i]);
			fclose(f);
		}
	}
	if (!st) st = jn_subspace_matrices(c, n, rows, norm_matrix_path ? N : NULL, subspace_operator_path ? O : NULL);
	if (!st && norm_matrix_path) st = save_npy(norm_matrix_path, N, n);
	if (!st && subspace_operator_path) st = save_npy(subspace_operator_path, O, n);
	free(V); free(rows); free(N); free(O);
	return st;
}
