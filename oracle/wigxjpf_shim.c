/*
 * oracle/wigxjpf_shim.c — test infrastructure only.
 *
 * The Wigner 3j symbol behind the wigxjpf interface that the reference's
 * clebsch_gordan.c calls (src/Neptune/clebsch_gordan/clebsch_gordan.c:8-42).
 * wigxjpf 1.10 is a dependency of the reference that its tree does not
 * include; its published algorithm is the Racah single-sum formula, which
 * is restated here in long double arithmetic with a factorial table:
 *
 *   (j1 j2 j3; m1 m2 m3) = (-1)^(j1-j2-m3) sqrt(Delta) sqrt(prod (j_i +- m_i)!)
 *       * sum_k (-1)^k / [k! (j3-j2+k+m1)! (j3-j1+k-m2)! (j1+j2-j3-k)!
 *                         (j1-k-m1)! (j2-k+m2)!],
 *   Delta = (j1+j2-j3)! (j1-j2+j3)! (-j1+j2+j3)! / (j1+j2+j3+1)!,
 *
 * with all angular momenta passed doubled.  Accuracy is checked against
 * exact values in tests/test_transform.py.
 */
#include <math.h>
#include <stdlib.h>

#include "wigxjpf_shim/wigxjpf.h"

struct wigxjpf_temp { int unused; };

static long double g_fact[128];

void wigxjpf_fill_factors(int max_factorial)
{
	(void)max_factorial;
	g_fact[0] = 1.0L;
	for (int i = 1; i < 128; i++) g_fact[i] = g_fact[i - 1] * (long double)i;
}

struct wigxjpf_temp *wigxjpf_temp_alloc(int max_two_j)
{
	(void)max_two_j;
	return (struct wigxjpf_temp *)calloc(1, sizeof(struct wigxjpf_temp));
}

void wigxjpf_temp_free(struct wigxjpf_temp *temp) { free(temp); }

static long double F(int twice) { return g_fact[twice / 2]; }

void calc_3j_double(double *result, int j1, int j2, int j3, int m1, int m2, int m3, struct wigxjpf_temp *temp)
{
	(void)temp;
	*result = 0.0;
	if (g_fact[0] == 0.0L) wigxjpf_fill_factors(0);
	if (m1 + m2 + m3 != 0 || j1 < 0 || j2 < 0 || j3 < 0) return;
	if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return;
	if (((j1 + m1) | (j2 + m2) | (j3 + m3) | (j1 + j2 + j3)) & 1) return;
	if (j1 + j2 - j3 < 0 || j1 - j2 + j3 < 0 || -j1 + j2 + j3 < 0) return;
	if ((j1 + j2 + j3) / 2 + 1 >= 128) return;
	long double delta = F(j1 + j2 - j3) * F(j1 - j2 + j3) * F(-j1 + j2 + j3) / F(j1 + j2 + j3 + 2);
	long double pre = sqrtl(delta * F(j1 + m1) * F(j1 - m1) * F(j2 + m2) * F(j2 - m2) * F(j3 + m3) * F(j3 - m3));
	long double sum = 0.0L;
	for (int k = 0;; k++) {
		const int x3 = j1 + j2 - j3 - 2 * k, x4 = j1 - 2 * k - m1, x5 = j2 - 2 * k + m2;
		if (x3 < 0 || x4 < 0 || x5 < 0) break;
		const int x1 = j3 - j2 + 2 * k + m1, x2 = j3 - j1 + 2 * k - m2;
		if (x1 < 0 || x2 < 0) continue;
		long double d = F(2 * k) * F(x1) * F(x2) * F(x3) * F(x4) * F(x5);
		sum += (k & 1) ? -1.0L / d : 1.0L / d;
	}
	int ph = (j1 - j2 - m3) / 2;
	long double v = pre * sum;
	*result = (double)((ph & 1) ? -v : v);
}
