/*
 * jn_jt.h — the coupled (J, T) two-particle basis of Antoine-format
 * interaction files and the Clebsch-Gordan coefficients that connect it to
 * the M-scheme.
 *
 * Everything here is integer bookkeeping plus one floating-point function
 * (the Clebsch-Gordan coefficient); all of it runs on the host when a
 * transform is planned.  Angular momenta, their projections and isospin
 * projections are stored doubled (j = 3 means j = 3/2), except J and T of a
 * coupled pair, which are stored as plain integers, as in the reference.
 */
#ifndef JN_JT_H
#define JN_JT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One harmonic-oscillator shell (n, l, j) of energy e = 2n + l; j doubled. */
typedef struct {
	int e, n, l, j;
} jn_shell_t;

/* Antoine shell order (src/Neptune/bases/shells.c:72-130): e ascending,
 * then l ascending from e & 1, then j ascending from |2l - 1| to 2l + 1.
 * Returns the number of shells with e <= emax, (emax+1)(emax+2)/2, and
 * fills out[] when it is not NULL. */
int jn_antoine_shells(int emax, jn_shell_t *out);

/* One coupled state |a b; J T> with shell indices a <= b. */
typedef struct {
	int a, b, J, T, parity;
} jn_jt_state_t;

/*
 * The Antoine JT basis (src/Neptune/bases/jt_basis.c:70-101, 250-287):
 * blocks in the order of the bit field {parity:1, T:1, J}, i.e.
 * index = 4 J + 2 T + parity, for J = 0 .. emax2 + 1; inside a block the
 * pairs a <= b in shell order with e_a + e_b <= emax2 that satisfy the
 * triangle rule, the block's parity and the Pauli rule (a != b or J + T odd).
 *
 * The interaction file stores one row per configuration: a pair of states
 * (left <= right) of the same J, T and parity, enumerated left by left
 * (src/Neptune/bases/jt_basis.c:130-166).  cfg_first[i] is the row of
 * (i, i); rows of (i, k), k in [i, cfg_end[i]), follow consecutively.
 */
typedef struct {
	int emax1, emax2;
	int nshells;
	jn_shell_t *shells;
	int n;                          /* number of states */
	jn_jt_state_t *st;
	int nJ;                         /* J = 0 .. nJ-1 */
	int *blk_first, *blk_count;     /* per (J, T): index 2J + T; both parities */
	int64_t nconfig;
	int64_t *cfg_first;
	int *cfg_end;
} jn_jt_basis_t;

int jn_jt_basis_build(int emax1, int emax2, jn_jt_basis_t *basis);
void jn_jt_basis_free(jn_jt_basis_t *basis);

/* configuration row of states (i, k) or -1 if they share no (J, T, parity)
 * block (src/Neptune/input/read_2nf_antoine_format.c:225-242: the pair is
 * ordered first) */
int64_t jn_jt_config(const jn_jt_basis_t *basis, int i, int k);

/*
 * <j1 m1 j2 m2 | j3 m3>, all arguments doubled, through the Wigner 3j symbol
 * as src/Neptune/clebsch_gordan/clebsch_gordan.c:31-42 defines it:
 *     CG = 3j(j1 j2 j3; m1 m2 -m3) sqrt(j3 + 1) (-1)^((j1 - j2 + m3)/2).
 * The 3j symbol is the Racah sum, evaluated exactly: the alternating sum of
 * multinomial coefficients is an integer (128-bit), and the square-root
 * prefactor is a ratio of factorials kept as prime exponents.  The result
 * is within a few units in the last place of the exact value.
 */
double jn_cg(int j1, int j2, int j3, int m1, int m2, int m3);
double jn_three_j(int j1, int j2, int j3, int m1, int m2, int m3);

#ifdef __cplusplus
}
#endif
#endif
