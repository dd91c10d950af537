/* c5_balls_check.c -- prints the large-domain workload's balls (the
 * seeded draws of alis_gb300/bench/c5_balls.h) for the host tests:
 *
 *   c5_balls_check <seed> <count> <ni> <nj> <nk> <dx>
 *
 * one line per ball: x y z r (nm), then the domain bounds. */
#include <stdio.h>
#include <stdlib.h>
#include "../../alis_gb300/bench/c5_balls.h"

int main(int argc, char **argv)
{
	if (argc < 7) return 2;
	const unsigned long long seed = strtoull(argv[1], 0, 10);
	const int count = atoi(argv[2]);
	const int n[3] = { atoi(argv[3]) - 34, atoi(argv[4]) - 34, atoi(argv[5]) - 34 };
	const c5Real dx = (c5Real)atof(argv[6]);
	c5Real lo[3], hi[3];
	c5Domain(n, dx, lo, hi);
	c5Ball *B = calloc(count > 0 ? count : 1, sizeof *B);
	c5Balls(seed, count, lo, hi, dx, B);
	for (int q = 0; q < count; q++) printf("%.9g %.9g %.9g %.9g\n", B[q].x, B[q].y, B[q].z, B[q].r);
	printf("domain %.9g %.9g %.9g %.9g %.9g %.9g\n", lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]);
	free(B);
	return 0;
}
