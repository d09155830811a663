/*
 * jn_aurora — drop-in for aurora.x (src/Aurora/programs/aurora.c:21-62):
 *   jn_aurora <comb.txt> <index_list_path> <output_path> <Z> <N> [--human-readable] [--no-3NF]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/jncsm.h"

int main(int argc, char **argv)
{
	if (argc < 6) {
		printf("Usage %s <comb.txt> <index_list_path> <output_path> <Z> <N> [--human-readable] [--no-3NF]\n", argv[0]);
		return EXIT_FAILURE;
	}
	int human = 0, no3 = 0;
	for (int i = 6; i < argc; i++) {
		if (!strcmp(argv[i], "--human-readable")) human = 1;
		if (!strcmp(argv[i], "--no-3NF")) no3 = 1;
	}
	int n = 0;
	if (jn_aurora(argv[1], argv[2], argv[3], atoi(argv[4]), atoi(argv[5]), human, no3, &n) != JN_OK) {
		fprintf(stderr, "%s\n", jn_last_error());
		return EXIT_FAILURE;
	}
	return EXIT_SUCCESS;
}
