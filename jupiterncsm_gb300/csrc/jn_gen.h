/*
 * jn_gen.h — synthetic NCSM problem generator (Anicre-format stand-in).
 *
 * Writes a complete JupiterNCSM input directory (comb.txt, index lists,
 * matrix-element blocks, evaluation order, Anicre basis files, bacchus.conf)
 * for an harmonic-oscillator M-scheme basis with a seeded random M-scheme
 * interaction.  All entry points return 0 on success or a JN_GEN_E* code;
 * jn_gen_last_error() describes the last failure.
 */
#ifndef JN_GEN_H
#define JN_GEN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { JN_GEN_OK = 0, JN_GEN_EINVAL = 1, JN_GEN_EIO = 2, JN_GEN_ENOMEM = 3 };

typedef struct {
	int Z, N;               /* protons, neutrons */
	int Nmax;               /* excitation truncation in HO quanta */
	int M2;                 /* total 2*M */
	int parity;             /* 0 positive, 1 negative */
	int nbody;              /* 2: two-body, 3: two- plus three-body */
	uint64_t seed;
	double hbar_omega;      /* MeV; 0 disables the oscillator term */
	double sigma2, sigma3;  /* widths of the two- and three-body deviates (MeV) */
	int me_only;            /* write only matrix-element blocks into me_subdir */
	const char *me_subdir;  /* default "matrix_elements" */
	int write_basis_files;  /* Anicre basis_energy_<E> files under anicr/ */
	int lanczos_iterations; /* written into bacchus.conf */
	int antoine;            /* two-body interaction as a J-scheme Antoine file (antoine_2nf.bin)
				   instead of M-scheme blocks: the two-body matrix-element blocks are
				   then left to the J->M transform */
	int anicre_lists;       /* also write the index lists as Anicre names them, under
				   anicr_lists/<type>_inds_index_lists/: 1 raw triples, 2 rows "in out +-k"
				   (the input of aurora.x) */
} jn_gen_config;

typedef struct {
	size_t dimension;
	int num_basis_blocks;
	size_t num_lists, list_entries;
	size_t num_me_blocks, me_elements;
	size_t num_calc_blocks;
	unsigned long long multiplications;
	int num_orbitals, num_proton_sds, num_neutron_sds;
	int emax_single, emax_pair;     /* largest orbital and pair energies (the transform's
					   --single-particle-energy and --two-particle-energy) */
} jn_gen_summary;

void jn_gen_default_config(jn_gen_config *cfg);
int jn_generate(const jn_gen_config *cfg, const char *outdir, jn_gen_summary *summary);
const char *jn_gen_last_error(void);
/*
 * Write a seeded two-body interaction in the Antoine J-scheme format that
 * Mercury reads (src/Neptune/input/read_2nf_antoine_format.c:13-257): three
 * Fortran unformatted records, a title, the header {int ncol; float hw;
 * int nrow} and float[nrow][ncol], one row per configuration of the JT basis
 * built with (emax1, emax2).  Columns 3, 4 and 5 (Tz = -2, +2, 0) are
 * sigma * N(0,1) deviates keyed by the configuration; column 0 is the
 * coefficient k with 2 hw k / A = hw (e_a + e_b) / (A - 1) on diagonal
 * configurations and 0 elsewhere, so that the transformed interaction
 * carries the oscillator term hw * (number of quanta).  Columns 1 and 2 are 0.
 */
int jn_gen_antoine(const char *path, int emax1, int emax2, int num_particles, double hbar_omega, uint64_t seed,
		   double sigma);

/* the seeded N(0,1) deviate attached to the unordered pair {ka, kb} */
double jn_gen_pair_normal(uint64_t seed, uint64_t tag, uint64_t ka, uint64_t kb);

/* A seeded jjj-coupled three-body interaction in the reference's ASCII
 * format: <dir>/jjj.cnf and <dir>/jjj.mat, every coupled state the
 * three-body transform can reach with shells up to emax and three-particle
 * energy up to e3max, elements ~ N(0, sigma^2) symmetric in bra <-> ket.
 * Returns 0 or an error code (jn_gen_last_error). */
int jn_gen_jjj_ascii(const char *dir, int emax, int e3max, uint64_t seed, double sigma, int64_t *num_states,
		     int64_t *num_elements);

#ifdef __cplusplus
}
#endif
#endif
