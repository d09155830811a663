/*
 * jn_vulcan — drop-in for vulcan.x (src/Vulcan/programs/vulcan.c:47-112,
 * src/Vulcan/arguments/arguments.c:22-75):
 *   jn_vulcan <output_path> <comb.txt> <num protons> <num neutrons> [operator_path [-c/--coefficient <value>]]...
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/jncsm.h"

int main(int argc, char **argv)
{
	if (argc < 5) {
		printf("Usage: %s <output_path> <comb.txt> <num protons> <num neutrons> "
		       "[operator_path [-c/--coefficient <value>]]...\n", argv[0]);
		return EXIT_FAILURE;
	}
	const char **ops = calloc((size_t)argc, sizeof(char *));
	double *coef = calloc((size_t)argc, sizeof(double));
	int n = 0;
	for (int i = 5; i < argc; i++) {
		if (!strcmp(argv[i], "-c") || !strcmp(argv[i], "--coefficient")) {
			char *end;
			if (i + 1 >= argc || n == 0) {
				fprintf(stderr, "a coefficient must follow an operator path\n");
				return EXIT_FAILURE;
			}
			coef[n - 1] = strtod(argv[++i], &end);
			if (*end) {
				fprintf(stderr, "Argument @ %d, %s is not a double\n", i, argv[i]);
				return EXIT_FAILURE;
			}
		} else {
			ops[n] = argv[i];
			coef[n++] = 1.0;
		}
	}
	jn_status s = jn_vulcan(argv[2], atoi(argv[3]), atoi(argv[4]), n, ops, coef, argv[1]);
	free(ops);
	free(coef);
	if (s != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	return EXIT_SUCCESS;
}
