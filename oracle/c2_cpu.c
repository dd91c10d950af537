/*
 * c2_cpu.c -- ORACLE (test infrastructure only): CPU baseline of the
 * dispersive-scatterer benchmark.  The benchmark world of
 * alis_gb300/bench/c2.c is built through the public API and stepped by the
 * oracle restatement of the reference loops (cpu_step.c) on all host
 * cores with OpenMP, as the reference build runs.  Prints one JSON object.
 *
 *   c2_cpu <half-size nm> <timed steps> <warm-up steps>
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
	int half = argc > 1 ? atoi(argv[1]) : 230;
	int steps = argc > 2 ? atoi(argv[2]) : 5;
	int warm = argc > 3 ? atoi(argv[3]) : 1;
	double t0 = now();
	long cells = c2_build(half, 64);
	double t1 = now();
	c2_steps(warm);
	double t2 = now();
	c2_steps(steps);
	double t3 = now();
	printf("{\"cells\": %ld, \"steps\": %d, \"seconds\": %.6f, \"setup_seconds\": %.3f, \"warmup_seconds\": %.3f, \"threads\": %d}\n",
	       cells, steps, t3 - t2, t1 - t0, t2 - t1, omp_get_max_threads());
	return 0;
}
