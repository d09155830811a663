/*
 * jn_mars — drop-in for mars.x (src/Mars/programs/mars.c:64-90,
 * src/Mars/settings/settings.c):
 *   jn_mars <combination table file> <output file> [--num-protons <int>] [--num-neutrons <int>]
 *           [--only-two-nucleon-forces]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/jncsm.h"

int main(int argc, char **argv)
{
	if (argc < 3) {
		printf("Usage: %s <combination table file> <output file> [--num-protons <integer>] "
		       "[--num-neutrons <integer>] [--only-two-nucleon-forces]\n", argv[0]);
		return EXIT_FAILURE;
	}
	int Z = 0, N = 0, two = 0;
	for (int i = 3; i < argc; i++) {
		if (!strcmp(argv[i], "--num-protons") && i + 1 < argc) Z = atoi(argv[++i]);
		else if (!strcmp(argv[i], "--num-neutrons") && i + 1 < argc) N = atoi(argv[++i]);
		else if (!strcmp(argv[i], "--only-two-nucleon-forces")) two = 1;
	}
	if (jn_mars(argv[1], Z, N, argv[2], two, NULL) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	return EXIT_SUCCESS;
}
