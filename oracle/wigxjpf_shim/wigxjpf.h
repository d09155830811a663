/*
 * Stand-in for the header of wigxjpf 1.10 (the Wigner-symbol library the
 * reference links for its Clebsch-Gordan coefficients; not vendored in the
 * reference tree).  Test infrastructure: it lets the oracle compile the
 * reference's own transform sources.  Only the four calls the reference
 * makes (src/Neptune/clebsch_gordan/clebsch_gordan.c:8-42) are declared.
 */
#ifndef ORACLE_WIGXJPF_SHIM_H
#define ORACLE_WIGXJPF_SHIM_H
struct wigxjpf_temp;
void wigxjpf_fill_factors(int max_factorial);
struct wigxjpf_temp *wigxjpf_temp_alloc(int max_two_j);
void wigxjpf_temp_free(struct wigxjpf_temp *temp);
void calc_3j_double(double *result, int two_j1, int two_j2, int two_j3, int two_m1, int two_m2, int two_m3,
		    struct wigxjpf_temp *temp);
#endif
