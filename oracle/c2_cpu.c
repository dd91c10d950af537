/*
 * c2_cpu.c -- ORACLE (test infrastructure only): CPU baseline of the
 * dispersive-scatterer benchmark.  The benchmark world of
 * alis_gb300/bench/c2.c is built through the public API and stepped by the
 * oracle restatement of the reference loops (cpu_step.c) on all host
 * cores with OpenMP, as the reference build runs.  Prints one JSON object
 * with the timing (also updateE + updateH and updatePhaser apart) and the
 * outgoing flux of every phaser frequency after the last step.  With `c1` in place of the half size the vacuum
 * plane-wave world of c1_build (128^3 cells) is built instead.
 *
 *   c2_cpu <half-size nm | c1> <timed steps> <warm-up steps>
 */
#include <omp.h>
#include <sys/time.h>
#include "../alis_gb300/bench/c2.c"

static double now(void)
{
	struct timeval t;
	gettimeofday(&t, 0);
	return t.tv_sec + 1e-6 * t.tv_usec;
}

int main(int argc, char **argv)
{
	const char *what = argc > 1 ? argv[1] : "230";
	int steps = argc > 2 ? atoi(argv[2]) : 5;
	int warm = argc > 3 ? atoi(argv[3]) : 1;
	double t0 = now();
	long cells = strcmp(what, "c1") ? c2_build(atoi(what), 64) : c1_build(128);
	double t1 = now();
	c2_steps(warm);
	double t2 = now();
	/* the steps of c2_steps, with updateE + updateH and updatePhaser timed apart */
	double tUpdate = 0, tPhaser = 0;
	for (int q = 0; q < steps; q++) {
		const double a = omp_get_wtime();
		updateE(W);
		updateH(W);
		const double b = omp_get_wtime();
		updatePhaser(W, P);
		tUpdate += b - a, tPhaser += omp_get_wtime() - b;
	}
	double t3 = now();
	printf("{\"cells\": %ld, \"steps\": %d, \"seconds\": %.6f, \"update_seconds\": %.6f, \"phaser_seconds\": %.6f, "
	       "\"setup_seconds\": %.3f, \"warmup_seconds\": %.3f, \"threads\": %d, \"flux\": [",
	       cells, steps, t3 - t2, tUpdate, tPhaser, t1 - t0, t2 - t1, omp_get_max_threads());
	for (int f = 0; f < c2_nfreq(); f++) printf("%s%.9g", f ? ", " : "", c2_flux(f));
	printf("]}\n");
	return 0;
}
