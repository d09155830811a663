/*
 * transform_emulator.c — test helper: a CPU model of jn_jt_to_m_kernel.
 *
 * It builds the product's transform plan (jn_transform.c) and evaluates
 * every two-body matrix element with the kernel's arithmetic: separately
 * rounded multiplies and adds (compile with -ffp-contract=off), J ascending
 * then T, sign applied last.  The tests compare it with the reference's own
 * transform (oracle/_ref/ref_mercury) without a GPU, and the GPU tests
 * compare the kernel with it bit for bit.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../jupiterncsm_gb300/csrc/jn_transform.h"

static char g_err[1024];
const char *temu_error(void) { return g_err; }

typedef struct {
	jn_tplan_t plan;
	double *out;
} temu_t;

static double element(const jn_tplan_t *p, int blk, int64_t i)
{
	const jn_tblock_t *b = &p->tb[blk];
	int32_t ket, bra;
	int neg;
	if (b->kind == 0) {
		ket = p->conn_ket[b->conn + i];
		bra = p->conn_bra[b->conn + i];
		neg = p->conn_sign[b->conn + i] < 0;
	} else {
		int64_t kp = i / b->nn, kn = i - kp * b->nn;
		const jn_pconn_t *c = &p->pc[b->conn + kp];
		const jn_nconn_t *n = &p->nc[b->nconn + kn];
		int32_t k = p->lut[c->ket_lut + (int64_t)c->p_ann * c->ket_nn + n->n_ann];
		int32_t r = p->lut[c->bra_lut + (int64_t)c->p_cre * c->bra_nn + n->n_cre];
		neg = 0;
		if (k < 0) { k = -k - 1; neg ^= 1; }
		if (r < 0) { r = -r - 1; neg ^= 1; }
		ket = k; bra = r;
	}
	const jn_mstate_t *K = &p->ms[ket], *B = &p->ms[bra];
	int jlo = K->jlo > B->jlo ? K->jlo : B->jlo;
	int khi = K->jlo + K->nj, bhi = B->jlo + B->nj;
	int jhi = (khi < bhi ? khi : bhi) - 1;
	const double *Vt = p->V + (int64_t)b->tz * p->jt.nconfig;
	double acc = 0.0;
	for (int J = jlo; J <= jhi; J++) {
		int ik = K->coef + 2 * (J - K->jlo), ib = B->coef + 2 * (J - B->jlo);
		for (int T = 0; T < 2; T++) {
			int32_t ak = p->coef_a[ik + T], ab = p->coef_a[ib + T];
			if (ak < 0 || ab < 0) continue;
			int a0 = ak < ab ? ak : ab, a1 = ak < ab ? ab : ak;
			double v = a1 < p->jt.cfg_end[a0] ? Vt[p->jt.cfg_first[a0] + (a1 - a0)] : 0.0;
			double x = p->coef_s[ik + T] * v;
			x = x * p->coef_s[ib + T];
			acc = acc + x;
		}
	}
	return neg ? -acc : acc;
}

void *temu_open(const char *comb, const char *lists, int Z, int N, int e1, int e2, const char *antoine, int kinetic)
{
	temu_t *t = (temu_t *)calloc(1, sizeof *t);
	if (jn_tplan_build(&t->plan, comb, lists, Z, N, e1, e2, antoine, kinetic, g_err, sizeof g_err)) {
		free(t);
		return NULL;
	}
	const jn_tplan_t *p = &t->plan;
	t->out = (double *)malloc((p->nelem ? p->nelem : 1) * sizeof(double));
	for (int b = 0; b < p->n2; b++)
		for (int64_t i = 0; i < p->tb[b].count; i++) t->out[p->tb[b].out + i] = element(p, b, i);
	return t;
}

/* elements of block `id` (count only when out is NULL); -1 if absent */
int64_t temu_block(void *h, int id, double *out)
{
	temu_t *t = (temu_t *)h;
	const jn_tplan_t *p = &t->plan;
	for (int b = 0; b < p->n2; b++)
		if (p->info[p->tb_info[b]].id == id) {
			if (out) memcpy(out, t->out + p->tb[b].out, p->tb[b].count * sizeof(double));
			return p->tb[b].count;
		}
	for (int b = 0; b < p->n1; b++)
		if (p->info[p->z1_info[b]].id == id) {
			if (out) memset(out, 0, p->z1_count[b] * sizeof(double));
			return p->z1_count[b];
		}
	return -1;
}

/* ids of the one- and two-body blocks; returns their number */
int temu_ids(void *h, int *ids, int cap)
{
	temu_t *t = (temu_t *)h;
	const jn_tplan_t *p = &t->plan;
	int n = 0;
	for (int b = 0; b < p->n2; b++) { if (n < cap) ids[n] = p->info[p->tb_info[b]].id; n++; }
	for (int b = 0; b < p->n1; b++) { if (n < cap) ids[n] = p->info[p->z1_info[b]].id; n++; }
	return n;
}

/* header {n_dim, p_dim} of block `id` as the reference writes it; 0 if found */
int temu_header(void *h, int id, uint64_t *hdr)
{
	temu_t *t = (temu_t *)h;
	for (int b = 0; b < t->plan.nblocks; b++)
		if (t->plan.info[b].id == id) {
			hdr[0] = t->plan.info[b].Nn;
			hdr[1] = t->plan.info[b].Np;
			return 0;
		}
	return -1;
}

void temu_stats(void *h, int64_t *v)
{
	temu_t *t = (temu_t *)h;
	const jn_tplan_t *p = &t->plan;
	v[0] = p->nelem; v[1] = p->nms; v[2] = p->jt.nconfig; v[3] = p->n2; v[4] = p->n1; v[5] = p->jt.n;
}

void temu_close(void *h)
{
	temu_t *t = (temu_t *)h;
	if (!t) return;
	jn_tplan_free(&t->plan);
	free(t->out);
	free(t);
}
