/*
 * jn_transform3.h — host plan of the J-scheme -> M-scheme three-body
 * transform (Mercury's mercury_J_scheme_to_internal, three-body part, with
 * the J-scheme elements in the reference's ASCII format).
 *
 * The reference decouples, per (Tz, ket energies, bra energies) and per
 * total M, a dense matrix D_M = sum_{J_abc} S_bra^T V_J S_ket over the
 * jjj-coupled states of the two M-scheme bases
 * (src/Neptune/block_transform/block_transform.c:147-356,
 * src/Neptune/jjj_transformation/jjj_transformation.c:13-159) and reads one
 * element of D_M per connection of a matrix-element block
 * (src/Mercury/transformed_block/transformed_block.c:113-147).
 *
 * A column of S (one M-scheme state |abc>) is nonzero only on coupled states
 * built from a permutation of the shells of a, b and c, a handful per J_abc,
 * so the plan keeps for every M-scheme state its short list of
 * (J_abc, coupled state, S) terms, ordered as the reference sums them, and
 * the device evaluates each needed element of D_M directly:
 *     D[bra][ket] = sum_J sum_{a in bra(J)} (sum_{a' in ket(J)} S_ket V[a][a']) S_bra
 * with every multiply and add rounded on its own, in the reference's order.
 * V is stored densely per (energy block, J_abc) over the coupled states that
 * the bra and ket bases reach.
 */
#ifndef JN_TRANSFORM3_H
#define JN_TRANSFORM3_H

#include <stddef.h>
#include <stdint.h>

#include "jn_transform.h"

#ifdef __cplusplus
extern "C" {
#endif

/* one M-scheme three-particle state as the device sees it (8 bytes) */
typedef struct {
	int32_t ent;            /* first expansion term */
	int16_t nent;           /* terms, ordered by (J_abc, position in the coupled block) */
	int8_t jlo, jhi;        /* J_abc slots (J_abc = 2 slot + 1, doubled) its M block loops over */
} jn_m3state_t;

/* one expansion term (16 bytes) */
typedef struct {
	double s;               /* <coupled state | M-scheme state> */
	int32_t v;              /* row (bra side) or column (ket side) of the state in V */
	int32_t slot;           /* J_abc slot */
} jn_m3term_t;

/* one three-body matrix-element block (48 bytes) */
typedef struct {
	int64_t out;            /* first element in the output array */
	int64_t count;
	int32_t kind;           /* 0: one species (list of connections), 1: protons x neutrons */
	int32_t nn;             /* neutron connections (kind 1) */
	int32_t conn;           /* kind 0: first connection; kind 1: first proton connection */
	int32_t nconn;          /* kind 1: first neutron connection */
	int32_t eb;             /* energy block: V tables and the parity check */
	int32_t pad;
} jn_t3block_t;

/* one slot of a (energy block, ket) pair (24 bytes): T[toff + v] =
 * sum_r S_r V(eb, slot)[v][v_r] over the ket's terms r of the slot, v < rows */
typedef struct {
	int64_t toff;           /* first T entry; -1 when V(eb, slot) is absent */
	int32_t term0;          /* the ket's first term of the slot */
	int16_t nterm, slot;
	int32_t rows;
	int32_t eb;
} jn_t3seg_t;

/* kind 1: a ket (bra) state is lut[ket_lut + p_pos * ket_nn + n_pos] */
typedef struct {
	int32_t p_ann, p_cre;
	int32_t ket_lut, bra_lut;
	int32_t ket_nn, bra_nn;
} jn_p3conn_t;

typedef struct {
	int32_t Z, N, emax;             /* single-particle energy of the manager's shells */
	int nslots;                     /* J_abc slots: J_abc = 2 s + 1, s < nslots */
	/* blocks of the combination table */
	int nblocks;
	jn_meblock_info_t *info;
	int n3;                         /* three-body blocks, in table order */
	jn_t3block_t *tb;
	int *tb_info;
	int64_t nelem;
	/* M-scheme states and their expansions */
	int64_t nms;
	jn_m3state_t *ms;
	int64_t nterm;
	jn_m3term_t *term;
	/* V per (energy block, slot): offset and row length, zero rows when the parities differ */
	int neb;
	int64_t *voff;                  /* neb x nslots */
	int32_t *vld;                   /* neb x nslots */
	int32_t *vrows;                 /* neb x nslots: rows (the bra basis' coupled states) */
	int64_t nv;
	double *V;
	/* shared inner sums (jn_t3plan_shared): T = V(eb, slot) s_ket over every row, for each
	   (energy block, ket state) pair that elements use and each slot of the ket */
	int64_t npairs;
	int32_t *elem_pair;             /* per element: its (energy block, ket) pair */
	int64_t *pair_seg;              /* per pair: its first segment (npairs + 1 entries) */
	int64_t nseg;
	jn_t3seg_t *seg;
	int64_t nT;                     /* T entries */
	/* connections */
	int64_t nconn0;
	int32_t *conn_ket, *conn_bra, *conn_sign;
	int64_t npc, nnc, nlut;
	jn_p3conn_t *pc;
	jn_nconn_t *nc;
	int32_t *lut;                   /* state id, or -id-1 when sorting the connection's orbitals flips the sign */
	/* input statistics */
	int64_t file_states, file_elements, coupled_states;
	int64_t mblocks;
	double dense_flops;             /* flops of the reference's dense formulation */
} jn_t3plan_t;

/* Build the plan from a combination table, Anicre basis files and a
 * J-scheme directory (one .cnf and one .mat file); returns 0 or sets *err. */
int jn_t3plan_build(jn_t3plan_t *p, const char *comb, const char *lists_dir, int Z, int N, int emax,
		    const char *jscheme_dir, char *err, size_t errlen);
void jn_t3plan_free(jn_t3plan_t *p);
/* The shared-inner-sum layout of a built plan (elem_pair, pair_seg, seg, nT);
 * returns 0 or sets *err. */
int jn_t3plan_shared(jn_t3plan_t *p, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
