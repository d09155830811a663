/*
 * transform3_emulator.c — test helper: a CPU model of jn_jjj_to_m_kernel.
 *
 * It builds the product's three-body transform plan (jn_transform3.c) and
 * evaluates every three-body matrix element with the kernel's arithmetic:
 * separately rounded multiplies and adds (compile with -ffp-contract=off),
 * J_abc ascending, bra coupled states outer, ket coupled states inner, sign
 * applied last.  The tests compare it with the reference's own transform
 * (oracle/_ref/ref_mercury3) without a GPU, and the GPU tests compare the
 * kernel with it bit for bit.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../jupiterncsm_gb300/csrc/jn_transform3.h"

static char g_err[1024];
const char *t3emu_error(void) { return g_err; }

typedef struct {
	jn_t3plan_t plan;
	double *out;
} t3emu_t;

static double element(const jn_t3plan_t *p, int blk, int64_t i)
{
	const jn_t3block_t *b = &p->tb[blk];
	int32_t ket, bra;
	int neg;
	if (b->kind == 0) {
		ket = p->conn_ket[b->conn + i];
		bra = p->conn_bra[b->conn + i];
		neg = p->conn_sign[b->conn + i] < 0;
	} else {
		int64_t kp = i / b->nn, kn = i - kp * b->nn;
		const jn_p3conn_t *c = &p->pc[b->conn + kp];
		const jn_nconn_t *n = &p->nc[b->nconn + kn];
		int32_t k = p->lut[c->ket_lut + (int64_t)c->p_ann * c->ket_nn + n->n_ann];
		int32_t r = p->lut[c->bra_lut + (int64_t)c->p_cre * c->bra_nn + n->n_cre];
		neg = 0;
		if (k < 0) { k = -k - 1; neg ^= 1; }
		if (r < 0) { r = -r - 1; neg ^= 1; }
		ket = k; bra = r;
	}
	const jn_m3state_t *K = &p->ms[ket], *B = &p->ms[bra];
	const int jlo = K->jlo > B->jlo ? K->jlo : B->jlo, jhi = K->jhi < B->jhi ? K->jhi : B->jhi;
	const int64_t *vo = p->voff + (int64_t)b->eb * p->nslots;
	const int32_t *vl = p->vld + (int64_t)b->eb * p->nslots;
	int ik = K->ent, ib = B->ent;
	const int ek = K->ent + K->nent, eb = B->ent + B->nent;
	double acc = 0.0;
	while (ik < ek && ib < eb) {
		const int sk = p->term[ik].slot, sb = p->term[ib].slot;
		if (sk < sb) { ik++; continue; }
		if (sb < sk) { ib++; continue; }
		int gk = ik, gb = ib;
		while (gk < ek && p->term[gk].slot == sk) gk++;
		while (gb < eb && p->term[gb].slot == sk) gb++;
		if (sk >= jlo && sk <= jhi && vo[sk] >= 0) {
			const double *Vs = p->V + vo[sk];
			double d = 0.0;
			for (int q = ib; q < gb; q++) {
				const double *row = Vs + (int64_t)p->term[q].v * vl[sk];
				double inner = 0.0;
				for (int r = ik; r < gk; r++) {
					double x = p->term[r].s * row[p->term[r].v];
					inner = inner + x;
				}
				double y = inner * p->term[q].s;
				d = d + y;
			}
			acc = acc + d;
		}
		ik = gk;
		ib = gb;
	}
	return neg ? -acc : acc;
}

void *t3emu_open(const char *comb, const char *lists, int Z, int N, int emax, const char *jdir)
{
	t3emu_t *t = (t3emu_t *)calloc(1, sizeof *t);
	if (jn_t3plan_build(&t->plan, comb, lists, Z, N, emax, jdir, g_err, sizeof g_err)) {
		free(t);
		return NULL;
	}
	const jn_t3plan_t *p = &t->plan;
	t->out = (double *)malloc((p->nelem ? p->nelem : 1) * sizeof(double));
	for (int b = 0; b < p->n3; b++)
		for (int64_t i = 0; i < p->tb[b].count; i++) t->out[p->tb[b].out + i] = element(p, b, i);
	return t;
}

/* elements of three-body block `id` (count only when out is NULL); -1 if absent */
int64_t t3emu_block(void *h, int id, double *out)
{
	t3emu_t *t = (t3emu_t *)h;
	const jn_t3plan_t *p = &t->plan;
	for (int b = 0; b < p->n3; b++)
		if (p->info[p->tb_info[b]].id == id) {
			if (out) memcpy(out, t->out + p->tb[b].out, p->tb[b].count * sizeof(double));
			return p->tb[b].count;
		}
	return -1;
}

/* ids of the three-body blocks; returns their number */
int t3emu_ids(void *h, int *ids, int cap)
{
	t3emu_t *t = (t3emu_t *)h;
	const jn_t3plan_t *p = &t->plan;
	int n = 0;
	for (int b = 0; b < p->n3; b++) { if (n < cap) ids[n] = p->info[p->tb_info[b]].id; n++; }
	return n;
}

/* The two launches' arithmetic on the plan's shared-inner-sum layout
 * (jn_t3plan_shared): T = V(eb, slot) s_ket for every segment, then each
 * element from T, as jn_jjj_inner_kernel and jn_jjj_to_m_kernel compute
 * them.  Returns the number of elements that differ, bit for bit, from the
 * element-by-element model (-1 on a plan error); out[0..2] = pairs,
 * segments, inner sums. */
int64_t t3emu_check_shared(void *h, int64_t *out)
{
	t3emu_t *t = (t3emu_t *)h;
	jn_t3plan_t *p = &t->plan;
	if (jn_t3plan_shared(p, g_err, sizeof g_err)) return -1;
	out[0] = p->npairs; out[1] = p->nseg; out[2] = p->nT;
	double *T = (double *)malloc((p->nT ? p->nT : 1) * sizeof(double));
	if (!T) return -1;
	for (int64_t g = 0; g < p->nseg; g++) {
		const jn_t3seg_t *sg = &p->seg[g];
		if (sg->toff < 0) continue;
		const int64_t vi = (int64_t)sg->eb * p->nslots + sg->slot;
		const double *Vs = p->V + p->voff[vi];
		for (int v = 0; v < sg->rows; v++) {
			double inner = 0.0;
			for (int r = sg->term0; r < sg->term0 + sg->nterm; r++) {
				double x = p->term[r].s * Vs[(int64_t)v * p->vld[vi] + p->term[r].v];
				inner = inner + x;
			}
			T[sg->toff + v] = inner;
		}
	}
	int64_t bad = 0;
	for (int blk = 0; blk < p->n3; blk++) {
		const jn_t3block_t *b = &p->tb[blk];
		for (int64_t i = 0; i < b->count; i++) {
			int32_t ket, bra;
			int neg;
			if (b->kind == 0) {
				ket = p->conn_ket[b->conn + i];
				bra = p->conn_bra[b->conn + i];
				neg = p->conn_sign[b->conn + i] < 0;
			} else {
				int64_t kp = i / b->nn, kn = i - kp * b->nn;
				const jn_p3conn_t *c = &p->pc[b->conn + kp];
				const jn_nconn_t *n = &p->nc[b->nconn + kn];
				int32_t k = p->lut[c->ket_lut + (int64_t)c->p_ann * c->ket_nn + n->n_ann];
				int32_t r = p->lut[c->bra_lut + (int64_t)c->p_cre * c->bra_nn + n->n_cre];
				neg = 0;
				if (k < 0) { k = -k - 1; neg ^= 1; }
				if (r < 0) { r = -r - 1; neg ^= 1; }
				ket = k; bra = r;
			}
			const jn_m3state_t *K = &p->ms[ket], *B = &p->ms[bra];
			const int jlo = K->jlo > B->jlo ? K->jlo : B->jlo, jhi = K->jhi < B->jhi ? K->jhi : B->jhi;
			const int32_t pr = p->elem_pair[b->out + i];
			int64_t j = p->pair_seg[pr];
			const int64_t j1 = p->pair_seg[pr + 1];
			int ib = B->ent;
			const int eb = B->ent + B->nent;
			double acc = 0.0;
			while (j < j1 && ib < eb) {
				const jn_t3seg_t *sg = &p->seg[j];
				const int sb = p->term[ib].slot;
				if (sg->slot < sb) { j++; continue; }
				int gb = ib;
				while (gb < eb && p->term[gb].slot == sb) gb++;
				if (sb < sg->slot) { ib = gb; continue; }
				if (sb >= jlo && sb <= jhi && sg->toff >= 0) {
					double d = 0.0;
					for (int q = ib; q < gb; q++) {
						double y = T[sg->toff + p->term[q].v] * p->term[q].s;
						d = d + y;
					}
					acc = acc + d;
				}
				j++;
				ib = gb;
			}
			const double v = neg ? -acc : acc, w = t->out[b->out + i];
			if (memcmp(&v, &w, sizeof v)) bad++;
		}
	}
	free(T);
	return bad;
}

/* elements, M-scheme states, terms, coupled states, file states, file elements, V entries, energy blocks */
void t3emu_stats(void *h, int64_t *v)
{
	t3emu_t *t = (t3emu_t *)h;
	const jn_t3plan_t *p = &t->plan;
	v[0] = p->nelem; v[1] = p->nms; v[2] = p->nterm; v[3] = p->coupled_states; v[4] = p->file_states;
	v[5] = p->file_elements; v[6] = p->nv; v[7] = p->neb;
}

void t3emu_close(void *h)
{
	t3emu_t *t = (t3emu_t *)h;
	if (!t) return;
	jn_t3plan_free(&t->plan);
	free(t->out);
	free(t);
}
