/*
 * c2_spectrum.c -- the dispersive-scatterer benchmark world
 * (alis_gb300/bench/c2.c) run for a number of steps; prints its phaser
 * spectrum as one JSON object: per frequency f, the normalisation A and
 * the outgoing flux (phaserPoyntingOut).  Linked against the engine, the
 * oracle and the oracle's FP64 build, to state the spectral error of
 * each against FP64 at the benchmark's own size.
 *
 *   c2_spectrum <half-size nm> <steps>
 */
#include "../../alis_gb300/bench/c2.c"

int main(int argc, char **argv)
{
	int half = argc > 1 ? atoi(argv[1]) : 230;
	int steps = argc > 2 ? atoi(argv[2]) : 4000;
	long cells = c2_build(half, 64);
	c2_steps(steps);
	printf("{\"cells\": %ld, \"steps\": %d, \"bytes_per_real\": %d, \"f\": [", cells, steps, (int)sizeof(float));
	for (int n = 0; P[n].f; n++) printf("%s%.17g", n ? ", " : "", (double)P[n].f);
	printf("], \"A\": [");
	for (int n = 0; P[n].f; n++) printf("%s%.17g", n ? ", " : "", (double)P[n].A);
	printf("], \"flux\": [");
	for (int n = 0; P[n].f; n++) printf("%s%.17g", n ? ", " : "", (double)phaserPoyntingOut(P + n));
	printf("]}\n");
	deleteWorld(W);
	return 0;
}
