/*
 * jn_jt.c — Antoine shells, the coupled JT basis and Clebsch-Gordan
 * coefficients (see jn_jt.h).
 */
#include "jn_jt.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

int jn_antoine_shells(int emax, jn_shell_t *out)
{
	int k = 0;
	for (int e = 0; e <= emax; e++)
		for (int l = e & 1; l <= e; l += 2)
			for (int j = abs(2 * l - 1); j <= 2 * l + 1; j += 2) {
				if (out) {
					out[k].e = e;
					out[k].n = (e - l) / 2;
					out[k].l = l;
					out[k].j = j;
				}
				k++;
			}
	return k;
}

void jn_jt_basis_free(jn_jt_basis_t *b)
{
	if (!b) return;
	free(b->shells); free(b->st); free(b->blk_first); free(b->blk_count); free(b->cfg_first); free(b->cfg_end);
	memset(b, 0, sizeof *b);
}

int jn_jt_basis_build(int emax1, int emax2, jn_jt_basis_t *b)
{
	memset(b, 0, sizeof *b);
	if (emax1 < 0 || emax2 < 0 || emax1 > 60 || emax2 > 120) return -1;
	b->emax1 = emax1;
	b->emax2 = emax2;
	b->nshells = jn_antoine_shells(emax1, NULL);
	b->shells = (jn_shell_t *)calloc(b->nshells, sizeof(jn_shell_t));
	jn_antoine_shells(emax1, b->shells);
	b->nJ = emax2 + 2;
	const int nblocks = 4 * b->nJ;
	/* first pass counts, second fills */
	int cap = 0;
	for (int pass = 0; pass < 2; pass++) {
		int n = 0;
		for (int idx = 0; idx < nblocks; idx++) {
			const int parity = idx & 1, T = (idx >> 1) & 1, J = idx >> 2;
			for (int a = 0; a < b->nshells; a++) {
				const jn_shell_t *sa = &b->shells[a];
				if (2 * sa->e > emax2) break;
				for (int c = a; c < b->nshells; c++) {
					const jn_shell_t *sc = &b->shells[c];
					if (sa->e + sc->e > emax2) break;
					if (!(sa->j + sc->j >= 2 * J && abs(sa->j - sc->j) <= 2 * J)) continue;
					if (((sa->l + sc->l) & 1) != parity) continue;
					if (a == c && ((J + T) & 1) == 0) continue;
					if (pass) {
						jn_jt_state_t *s = &b->st[n];
						s->a = a; s->b = c; s->J = J; s->T = T; s->parity = parity;
					}
					n++;
				}
			}
		}
		if (!pass) {
			cap = n;
			b->st = (jn_jt_state_t *)calloc(cap ? cap : 1, sizeof(jn_jt_state_t));
		}
		b->n = n;
	}
	b->blk_first = (int *)calloc((size_t)(2 * b->nJ), sizeof(int));
	b->blk_count = (int *)calloc((size_t)(2 * b->nJ), sizeof(int));
	for (int i = 0; i < 2 * b->nJ; i++) b->blk_first[i] = -1;
	for (int i = 0; i < b->n; i++) {
		int k = 2 * b->st[i].J + b->st[i].T;
		if (b->blk_first[k] < 0) b->blk_first[k] = i;
		b->blk_count[k]++;
	}
	const size_t nst = b->n > 0 ? (size_t)b->n : 1;
	b->cfg_first = (int64_t *)calloc(nst, sizeof(int64_t));
	b->cfg_end = (int *)calloc(nst, sizeof(int));
	int64_t cfg = 0;
	for (int i = 0; i < b->n; i++) {
		int k = i;
		while (k < b->n && b->st[k].J == b->st[i].J && b->st[k].T == b->st[i].T &&
		       b->st[k].parity == b->st[i].parity)
			k++;
		b->cfg_first[i] = cfg;
		b->cfg_end[i] = k;
		cfg += k - i;
	}
	b->nconfig = cfg;
	return 0;
}

int64_t jn_jt_config(const jn_jt_basis_t *b, int i, int k)
{
	if (i > k) { int t = i; i = k; k = t; }
	if (i < 0 || k >= b->n || k >= b->cfg_end[i]) return -1;
	return b->cfg_first[i] + (k - i);
}

/* ------------------------------------------------------------------ */
/* Wigner 3j by the Racah sum, exactly                                 */
/* ------------------------------------------------------------------ */
static const int g_primes[] = { 2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47 };
#define NPRIMES ((int)(sizeof g_primes / sizeof g_primes[0]))
#define MAX_SUM 45      /* j1 + j2 + j3 (plain) up to 45: multinomials below 2^117 */

/* ex[p] += sign * (exponent of prime p in n!), n <= MAX_SUM + 1 */
static void add_factorial(int *ex, int n, int sign)
{
	for (int i = 0; i < NPRIMES; i++) {
		int e = 0;
		for (int q = g_primes[i]; q <= n; q *= g_primes[i]) e += n / q;
		ex[i] += sign * e;
	}
}

/* s! / (x[0]! ... x[5]!) with sum x = s, exactly */
static unsigned __int128 multinomial(int s, const int *x)
{
	unsigned __int128 r = 1;
	int left = s;
	for (int i = 0; i < 6; i++) {
		/* r *= C(left, x[i]) */
		unsigned __int128 c = 1;
		for (int k = 1; k <= x[i]; k++) c = c * (unsigned)(left - x[i] + k) / (unsigned)k;
		r *= c;
		left -= x[i];
	}
	return r;
}

double jn_three_j(int j1, int j2, int j3, int m1, int m2, int m3)
{
	if (m1 + m2 + m3 != 0) return 0.0;
	if (j1 < 0 || j2 < 0 || j3 < 0) return 0.0;
	if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
	if (((j1 + m1) & 1) || ((j2 + m2) & 1) || ((j3 + m3) & 1) || ((j1 + j2 + j3) & 1)) return 0.0;
	const int a = j1 + j2 - j3, b = j1 - j2 + j3, c = -j1 + j2 + j3;
	if (a < 0 || b < 0 || c < 0) return 0.0;
	const int s = (j1 + j2 + j3) / 2;
	if (s > MAX_SUM) return NAN;
	const int t2 = (j3 - j2 + m1) / 2, t3 = (j3 - j1 - m2) / 2, t4 = a / 2, t5 = (j1 - m1) / 2, t6 = (j2 + m2) / 2;
	int kmin = 0, kmax = t4;
	if (-t2 > kmin) kmin = -t2;
	if (-t3 > kmin) kmin = -t3;
	if (t5 < kmax) kmax = t5;
	if (t6 < kmax) kmax = t6;
	if (kmin > kmax) return 0.0;
	__int128 N = 0;
	for (int k = kmin; k <= kmax; k++) {
		const int x[6] = { k, t2 + k, t3 + k, t4 - k, t5 - k, t6 - k };
		__int128 t = (__int128)multinomial(s, x);
		N += (k & 1) ? -t : t;
	}
	if (N == 0) return 0.0;
	/* R = a! b! c! / (s+1)! * prod (j +- m)! / (s!)^2, as prime exponents */
	int ex[NPRIMES];
	memset(ex, 0, sizeof ex);
	add_factorial(ex, a / 2, 1);
	add_factorial(ex, b / 2, 1);
	add_factorial(ex, c / 2, 1);
	add_factorial(ex, s + 1, -1);
	add_factorial(ex, (j1 + m1) / 2, 1);
	add_factorial(ex, (j1 - m1) / 2, 1);
	add_factorial(ex, (j2 + m2) / 2, 1);
	add_factorial(ex, (j2 - m2) / 2, 1);
	add_factorial(ex, (j3 + m3) / 2, 1);
	add_factorial(ex, (j3 - m3) / 2, 1);
	add_factorial(ex, s, -2);
	/* sqrt(R) = (hn / hd) * sqrt(rn / rd) with the square parts taken out */
	double hn = 1.0, hd = 1.0, rn = 1.0, rd = 1.0;
	for (int i = 0; i < NPRIMES; i++) {
		int e = ex[i];
		if (e > 0) {
			for (int q = 0; q < e / 2; q++) hn *= g_primes[i];
			if (e & 1) rn *= g_primes[i];
		} else if (e < 0) {
			for (int q = 0; q < (-e) / 2; q++) hd *= g_primes[i];
			if ((-e) & 1) rd *= g_primes[i];
		}
	}
	double v = (double)N * hn / hd * sqrt(rn / rd);
	const int ph = (j1 - j2 - m3) / 2;
	return (ph & 1) ? -v : v;
}

double jn_cg(int j1, int j2, int j3, int m1, int m2, int m3)
{
	double r = jn_three_j(j1, j2, j3, m1, m2, -m3);
	const int ph = (j1 - j2 + m3) / 2;
	r *= sqrt((double)(j3 + 1));
	return (ph & 1) ? -r : r;
}
