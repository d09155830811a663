/*
 * jn_transform.h — host plan of the J-scheme -> M-scheme two-body transform
 * (Mercury's mercury_J_scheme_to_internal, two-body part).
 *
 * The reference decouples, per (bra energies, ket energies, Tz) and per
 * total M, a dense matrix D_M = sum_{J,T} S_bra^T V_JT S_ket
 * (src/Neptune/block_transform/block_transform.c:358-415,
 * src/Neptune/matrix_transform/matrix_transform.c:431-486) and then reads
 * one element of D_M per connection of a matrix-element block
 * (src/Mercury/transform_2nf_block_manager/transform_2nf_block_manager.c:157-268).
 *
 * For a fixed (J, T) every M-scheme pair state |a b> overlaps exactly one
 * coupled state, the one built from the shells of a and b, so each column
 * of S_JT has one nonzero.  D_M[bra][ket] is therefore the short sum
 *     sum_{J,T} S_bra(J,T) * V_JT[alpha_bra(J,T)][alpha_ket(J,T)] * S_ket(J,T)
 * over at most 2 (2 j_max + 1) terms, and the plan keeps, for every
 * M-scheme pair state, its coefficient S and coupled state alpha per (J, T).
 * The device computes each matrix element directly from that, in the
 * reference's order of operations, without forming D_M.
 */
#ifndef JN_TRANSFORM_H
#define JN_TRANSFORM_H

#include <stddef.h>
#include <stdint.h>

#include "jn_jt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* one M-scheme pair state as the device sees it (16 bytes) */
typedef struct {
	int32_t coef;           /* first (J, T) slot in the coefficient arrays */
	int16_t jlo, nj;        /* J range [jlo, jlo + nj) of the slots, two T each */
	int32_t mindex;         /* position inside its total-M block */
	int16_t M;              /* total 2M */
	int16_t phase;          /* +1 / -1: sign of ordering the pair as the basis does */
} jn_mstate_t;

/* one matrix-element block (40 bytes) */
typedef struct {
	int64_t out;            /* first element in the output array */
	int64_t count;          /* elements */
	int32_t kind;           /* 0: single species (list of connections), 1: proton x neutron */
	int32_t nn;             /* neutron connections (kind 1) */
	int32_t conn;           /* kind 0: first entry of conn_ket/conn_bra; kind 1: first proton connection */
	int32_t nconn;          /* kind 1: first neutron connection */
	int32_t tz;             /* column of the interaction: 0 (Tz=-2), 1 (Tz=0), 2 (Tz=+2) */
	int32_t pad;
} jn_tblock_t;

/* kind 1 connections are pairs of single-particle positions in the basis
 * files; the pair state of a ket is lut[ket_lut + p_pos * ket_nn + n_pos] */
typedef struct {
	int32_t p_ann, p_cre;   /* proton positions (annihilated in the ket file, created in the bra file) */
	int32_t ket_lut, bra_lut;
	int32_t ket_nn, bra_nn;
} jn_pconn_t;

typedef struct {
	int32_t n_ann, n_cre;
} jn_nconn_t;

typedef struct {
	int id;
	int np, nn;             /* particles of each species (1 or 2 in total) */
	int dEp, dMp, dp, dEn, dMn, dn;
	uint64_t Np, Nn;        /* proton / neutron combinations (comb.txt) */
} jn_meblock_info_t;

typedef struct {
	/* inputs */
	int Z, N, emax1, emax2, jmax;
	jn_jt_basis_t jt;
	double *V;              /* 3 x nconfig: Tz = -2, 0, +2 columns, kinetic term included */
	/* blocks */
	int nblocks;            /* all one- and two-body blocks of the table */
	jn_meblock_info_t *info;
	int n2;                 /* two-body blocks, in table order */
	jn_tblock_t *tb;
	int *tb_info;           /* tb[i] -> info index */
	int64_t nelem;
	/* pair states and their (J, T) expansions */
	int64_t nms;
	jn_mstate_t *ms;
	int64_t ncoef;
	double *coef_s;
	int32_t *coef_a;        /* global coupled-state index or -1 */
	/* connections */
	int64_t nconn1;
	int32_t *conn_ket, *conn_bra;   /* kind 0: pair-state ids */
	int32_t *conn_sign;             /* kind 0: +1 / -1 */
	int64_t npc, nnc, nlut;
	jn_pconn_t *pc;
	jn_nconn_t *nc;
	int32_t *lut;           /* kind 1: pair-state id, negated-minus-one when the pair flips sign */
	/* one-body blocks: zero blocks of the connection count (mercury_J_scheme_to_internal.c:108-139) */
	int n1;
	int *z1_info;
	int64_t *z1_count;
	/* statistics */
	double dense_flops;     /* flops of the reference's dense formulation, for comparison */
} jn_tplan_t;

/* The matrix-element rows of a combination table ("Matrix-elements V"
 * sections), in table order; *rows is malloc'ed.  Returns 0 or sets *err. */
int jn_read_me_blocks(const char *comb, jn_meblock_info_t **rows, int *n, char *err, size_t errlen);

/* Build the plan; returns 0 or sets *err (static text) and returns -1. */
int jn_tplan_build(jn_tplan_t *p, const char *comb, const char *lists_dir, int Z, int N, int emax1, int emax2,
		   const char *antoine, int include_kinetic, char *err, size_t errlen);
void jn_tplan_free(jn_tplan_t *p);

#ifdef __cplusplus
}
#endif
#endif
