/*
 * serve.c -- a request loop over the ALiS API: many simulations resident
 * on one GPU at once, admitted by device footprint as requests arrive and
 * stepped in turn, each world on streams of its own so that their steps
 * overlap on the device.
 *
 *   serve <mode> <requests> <rate/s> <seed> <small|large|sweep> [slots] [budget GB]
 *
 * mode served:     Poisson arrivals at <rate>; a request is admitted when
 *                  a slot is free and its footprint fits the budget; the
 *                  admitted worlds advance CHUNK steps per round, stepped
 *                  by SERVE_THREADS host threads (default 8) at once.
 * mode sequential: the same requests one after another, each run to its
 *                  end alone on the default streams (the plain path).
 * mode alone <id>: request <id> by itself (its result, for comparison).
 * mode batched:    the requests in waves -- as many as fit the budget and
 *                  the slots, in arrival order -- whose worlds step
 *                  together: every step's updateE, updateH and
 *                  updatePhaser calls of the wave's worlds are recorded
 *                  between alisBatchBegin and alisBatchEnd and run as a
 *                  few launches over all of them; SERVE_THREADS host
 *                  threads record a share of the wave each.
 *
 * The mix follows the served-stream workload in miniature: half vacuum
 * with a dielectric ball, three tenths a Drude bowtie antenna with a gap
 * of 5-30 nm, a fifth photonic-crystal slab k-point runs (Bloch-periodic,
 * complex fields, several k-points per request); 1-3 dipoles with Band or
 * Pulse waveforms; grid and step counts drawn per request.  Each request
 * reports the outgoing flux of its phaser box summed over frequencies
 * (and k-points) as its result.
 *
 * The sweep mix is the batched metasurface sweep instead: unit cells of
 * 32-96 cells laterally (periodic) and 64-256 along z (10-cell CPML on
 * both z faces), a TiO2-like Lorentz pillar of radius 40-120 nm and
 * height 200-600 nm on a glass substrate, a normal-incidence pulse
 * through a TFSF box, and a transmission phaser plane of 32 wavelengths;
 * 3000 steps each (SERVE_STEPS overrides).  Result: the plane's flux
 * summed over the wavelengths.
 *
 * Output: one line per finished request "R id kind cells steps latency_ms
 * result(hex)", then one JSON line with throughput and latency percentiles.
 */
#include <alis.h>
#include <time.h>
#include <stdint.h>
#include <unistd.h>
#include <omp.h>

#define MAXREQ 4096
#define MAXK 16
#define CHUNK 32

static double now(void)
{
	struct timespec t;
	clock_gettime(CLOCK_MONOTONIC, &t);
	return t.tv_sec + 1e-9 * t.tv_nsec;
}

static unsigned long long rng;
static double uniform(void)
{
	rng = rng * 6364136223846793005ULL + 1442695040888963407ULL;
	return (double)(rng >> 11) / 9007199254740992.0;
}

typedef struct {
	int kind, half, steps, nk, ndip, gap;
	int nx, nz;                              /* unit cell: lateral and z cells */
	float rad, hgt;                          /* unit cell: pillar radius and height (nm) */
	float dip[3][3];
	int wave[3];
	double arrival;
	/* while running */
	world W[MAXK];
	phaser P[MAXK];
	int done;
	long cells;
	double start, finish;
	double result;
} request;

static request R[MAXREQ];
static int small = 1, sweep = 0;
/* host wall time spent setting requests up, stepping them, finishing them */
static double tSetup, tStep, tFinish;

/* draw request q (the draw order is fixed, so every mode sees the same stream) */
static void drawRequest(int q, double *t, double rate)
{
	request *r = &R[q];
	if (sweep) {
		r->kind = 3, r->nk = 1;
		r->nx = 32 + (int)(65 * uniform());
		r->nz = 64 + (int)(193 * uniform());
		r->rad = (float)(40 + 80 * uniform());
		r->hgt = (float)(200 + 400 * uniform());
		const char *e = getenv("SERVE_STEPS");
		r->steps = e ? atoi(e) : 3000;
		*t += -log(1 - uniform()) / rate;
		r->arrival = *t;
		return;
	}
	double u = uniform();
	r->kind = u < 0.5 ? 0 : u < 0.8 ? 1 : 2;
	int lo = small ? 14 : 40, hi = small ? 24 : 96;                /* half size in cells */
	r->half = lo + (int)((hi - lo + 1) * uniform());
	int slo = small ? 120 : 1000, shi = small ? 240 : 2000;
	r->steps = slo + (int)((shi - slo + 1) * uniform());
	r->nk = r->kind == 2 ? (small ? 2 : 8) + (int)((small ? 2 : 9) * uniform()) : 1;
	r->ndip = 1 + (int)(3 * uniform());
	r->gap = 5 + (int)(26 * uniform());
	for (int d = 0; d < 3; d++) {
		for (int a = 0; a < 3; a++) r->dip[d][a] = (float)(20 * (uniform() - 0.5));
		r->wave[d] = uniform() < 0.5;
	}
	*t += -log(1 - uniform()) / rate;
	r->arrival = *t;
}

/* the worlds of request q, set up through the public API */
static void setupRequest(int q, int streams)
{
	double t0 = now();
	request *r = &R[q];
	float L = 10.0f * r->half;
	r->cells = 0;
	if (r->kind == 3) {
		/* a unit cell of the sweep: the pillar sits on the substrate, whose
		 * top lies 50 nm above the lower CPML; the TFSF box starts 50 nm
		 * below the substrate top and ends 120 nm below the upper CPML; the
		 * phaser plane lies 20 nm above the TFSF box */
		float a = 10.0f * r->nx, Lz = 10.0f * r->nz;
		dom D = {{-a / 2, a / 2 - 10}, {-a / 2, a / 2 - 10}, {-Lz / 2, Lz / 2 - 10}};
		res Re = {5, {10}, {1240}};
		sur S = {{PBC}, {PBC}, {PML, PML}, {10}};
		world W = createWorld(D, Re, S, "");
		float zb = -Lz / 2 + 150, ztop = Lz / 2 - 10 - 100 - 120;
		float h = r->hgt < ztop - zb - 40 ? r->hgt : ztop - zb - 40;
		float rr = r->rad < a / 2 - 20 ? r->rad : a / 2 - 20;
		object Pillar = {RodZ, {{-rr, rr}, {-rr, rr}, {zb, zb + h}}};
		object Sub = {Box, {{-INF, INF}, {-INF, INF}, {-INF, zb}}};
		matter TiO2 = {{5.5}, {{4.5, 0.05, 1.0}}};
		putObjects(W, TiO2, Pillar, n(1.45), Sub, Air);
		dom T = {{D.x.Min, D.x.Max}, {D.y.Min, D.y.Max}, {zb - 50, ztop}};
		planewave(W, T, Ppol, 0, 0, Pulse, 600, 150);
		phaser P = createPhasers(W, 400, 800, 400.0f / 31, -INF, INF, -INF, INF, ztop + 20, ztop + 20);
		if (streams) alisWorldStreams(W);
		r->W[0] = W, r->P[0] = P;
		r->cells = (long)W->iNUM * W->jNUM * W->kNUM;
		r->done = 0;
		tSetup += now() - t0;
		return;
	}
	for (int k = 0; k < r->nk; k++) {
		world W;
		if (r->kind == 0) {
			dom D = {{-L, L - 10}, {-L, L - 10}, {-L, L - 10}};
			res Re = {5, {10}, {1240}};
			sur S = {{PML}, {PML}, {PML}, {8}};
			W = createWorld(D, Re, S, "");
			object Ball1 = {Ball, {{-0.4f * L, 0.3f * L}, {-0.3f * L, 0.3f * L}, {-0.2f * L, 0.4f * L}}};
			putObjects(W, n(1.5), Ball1, Air);
		} else if (r->kind == 1) {
			float g = r->gap, a = 0.25f * L, s3 = sqrtf(3);
			dom D = {{-L, L - 10}, {-L, L - 10}, {-L, L - 10}};
			res Re = {5, {10}, {1240}};
			sur S = {{PML}, {PML}, {PML}, {8}};
			W = createWorld(D, Re, S, "");
			object Bowtie = {Combination, {{2}}, objects {
				{Intersection, {{2}}, objects {
					{Box, {{g / 2, g / 2 + 2 * a}, {-2 * a / s3, 2 * a / s3}, {-15, 15}}},
					{DRodZ, {{g / 2 - 2 * a, g / 2 + 2 * a}, {-2 * a / s3, 2 * a / s3}, {-15, 15}}}}},
				{Intersection, {{2}}, objects {
					{Box, {{-g / 2 - 2 * a, -g / 2}, {-2 * a / s3, 2 * a / s3}, {-15, 15}}},
					{DRodZ, {{-g / 2 - 2 * a, -g / 2 + 2 * a}, {-2 * a / s3, 2 * a / s3}, {-15, 15}}}}}}};
			matter Ag = {{4.0}, {{9.0, 0.02}}};
			putObjects(W, Ag, Bowtie, Air);
		} else {
			/* k-point k of a path through the Brillouin zone */
			float kk = 0.1f + 2.8f * k / r->nk, kx, ky;
			if (kk < 1) kx = 0, ky = kk;
			else if (kk < 2) kx = kk - 1, ky = 1;
			else kx = 3 - kk, ky = 3 - kk;
			float a = 2 * L;
			dom D = {{-L, L - 10}, {-L, L - 10}, {-L, L - 10}};
			res Re = {5, {10}, {1240}};
			sur S = {{BBC, a * 3 / kx}, {BBC, a * 3 / ky}, {PML}, {8}};
			W = createWorld(D, Re, S, "");
			object Slab = {Difference, {{2}}, objects {
				{Box, {{-INF, INF}, {-INF, INF}, {-0.2f * L, 0.2f * L}}},
				{RodZ, {{-0.4f * L, 0.4f * L}, {-0.4f * L, 0.4f * L}, {-INF, INF}}}}};
			putObjects(W, n(3.5), Slab, Air);
		}
		for (int d = 0; d < r->ndip; d++)
			pointDipole(W, d == 0 ? Ez : d == 1 ? Hx : Ey, r->dip[d][0], r->dip[d][1], r->dip[d][2],
			            r->wave[d] ? Band : Pulse, 500, r->wave[d] ? 800 : 100);
		/* the phaser box 10 nm inside the CPML */
		float b = L - 90;
		phaser P = createPhasers(W, 500, 800, 100, -b, b, -b, b, -b, b);
		if (streams) alisWorldStreams(W);
		r->W[k] = W, r->P[k] = P;
		r->cells += (long)W->iNUM * W->jNUM * W->kNUM;
	}
	r->done = 0;
	tSetup += now() - t0;
}

/* device bytes of request q: fields (complex: twice), eps^-1, CPML psi
 * slabs, phaser accumulators and ring -- an estimate from the grid */
static double footprint(int q)
{
	request *r = &R[q];
	if (r->kind == 3) {
		/* fields, eps^-1, two CPML slabs, a phaser plane of 32 wavelengths, the TFSF column */
		double cells = (r->nx + 2.0) * (r->nx + 2.0) * (r->nz + 2.0), face = (r->nx + 2.0) * (r->nx + 2.0);
		return cells * (24 + 12) + 2 * 10 * face * 32 + face * (4 * 8 * 32 * 2 + 16 * 64);
	}
	double n = 2 * r->half + 2;
	double cells = n * n * n, face = n * n;
	double per = (r->kind == 2 ? 2 : 1) * 6 * 4.0 + 12 + 0.5 * 16;
	return r->nk * (cells * per + 6 * face * 4 * 8 * 4 * 2 + 6 * face * 16 * 64);
}

/* (host threads step different requests at once; timing at the callers) */
static void stepRequest(int q, int n)
{
	request *r = &R[q];
	for (int s = 0; s < n && r->done < r->steps; s++, r->done++)
		for (int k = 0; k < r->nk; k++) {
			updateE(r->W[k]);
			updateH(r->W[k]);
			updatePhaser(r->W[k], r->P[k]);
		}
}

static void finishRequest(int q)
{
	double t0 = now();
	request *r = &R[q];
	double sum = 0;
	for (int k = 0; k < r->nk; k++) {
		for (int f = 0; r->P[k][f].f; f++) sum += phaserPoyntingOut(r->P[k] + f);
		deletePhaser(r->P[k]);
		deleteWorld(r->W[k]);
	}
	r->result = sum;
	r->finish = now();
	tFinish += r->finish - t0;
}

static int cmpd(const void *a, const void *b)
{
	double x = *(const double *)a, y = *(const double *)b;
	return x < y ? -1 : x > y;
}

int main(int argc, char **argv)
{
	if (argc < 6) {
		fprintf(stderr, "usage: %s served|sequential|alone|batched requests rate seed small|large|sweep [slots|id] [budget GB]\n", argv[0]);
		return 2;
	}
	const char *mode = argv[1];
	int nreq = atoi(argv[2]);
	double rate = atof(argv[3]);
	rng = strtoull(argv[4], 0, 10);
	small = strcmp(argv[5], "large") != 0 && strcmp(argv[5], "sweep") != 0;
	sweep = strcmp(argv[5], "sweep") == 0;
	int slots = argc > 6 ? atoi(argv[6]) : 16;
	const char *te = getenv("SERVE_THREADS");
	int threads = te ? atoi(te) : 8;
	if (threads < 1) threads = 1;
	double budget = (argc > 7 ? atof(argv[7]) : 64) * 1e9;
	if (nreq < 1 || nreq > MAXREQ) return 2;
	double t = 0;
	for (int q = 0; q < nreq; q++) drawRequest(q, &t, rate);
	/* silence the library's progress lines */
	fflush(stdout);
	int saved = dup(1);
	freopen("/dev/null", "w", stdout);

	double t0 = now(), cellSteps = 0;
	int finished = 0;
	if (!strcmp(mode, "alone")) {
		int q = slots;
		setupRequest(q, 0);
		R[q].start = now();
		double ts = now();
		stepRequest(q, R[q].steps);
		tStep += now() - ts;
		finishRequest(q);
		cellSteps = (double)R[q].cells * R[q].steps;
		R[q].arrival = 0, R[q].finish -= t0;
		finished = 1;
		nreq = q + 1;
		for (int p = 0; p < q; p++) R[p].finish = -1;
	} else if (!strcmp(mode, "sequential")) {
		for (int q = 0; q < nreq; q++) {
			setupRequest(q, 0);
			double ts = now();
			stepRequest(q, R[q].steps);
			tStep += now() - ts;
			finishRequest(q);
			R[q].finish -= t0;
			R[q].arrival = 0;
			cellSteps += (double)R[q].cells * R[q].steps;
			finished++;
		}
	} else if (!strcmp(mode, "batched")) {
		int next = 0, wave[MAXREQ];
		while (next < nreq) {
			int n = 0, longest = 0;
			double used = 0;
			while (next < nreq && n < slots && (n == 0 || used + footprint(next) <= budget)) {
				setupRequest(next, 0);
				R[next].start = now();
				used += footprint(next);
				if (R[next].steps > longest) longest = R[next].steps;
				wave[n++] = next++;
			}
			/* each host thread records the steps of its share of the wave */
			double ts = now();
			const int nth = threads < n ? threads : n;
			#pragma omp parallel num_threads(nth)
			{
				const int me = omp_get_thread_num();
				const int a0 = n * me / nth, a1 = n * (me + 1) / nth;
				for (int s = 0; s < longest; s++) {
					alisBatchBegin();
					for (int a = a0; a < a1; a++) if (R[wave[a]].done < R[wave[a]].steps)
						for (int k = 0; k < R[wave[a]].nk; k++) updateE(R[wave[a]].W[k]);
					for (int a = a0; a < a1; a++) if (R[wave[a]].done < R[wave[a]].steps)
						for (int k = 0; k < R[wave[a]].nk; k++) updateH(R[wave[a]].W[k]);
					for (int a = a0; a < a1; a++) if (R[wave[a]].done < R[wave[a]].steps)
						for (int k = 0; k < R[wave[a]].nk; k++) updatePhaser(R[wave[a]].W[k], R[wave[a]].P[k]);
					alisBatchEnd();
					for (int a = a0; a < a1; a++) if (R[wave[a]].done < R[wave[a]].steps) R[wave[a]].done++;
				}
			}
			tStep += now() - ts;
			for (int a = 0; a < n; a++) {
				const int q = wave[a];
				finishRequest(q);
				R[q].finish -= t0;
				R[q].arrival = 0;
				cellSteps += (double)R[q].cells * R[q].steps;
				finished++;
			}
		}
	} else {
		int active[MAXREQ], nact = 0, next = 0;
		double used = 0;
		while (finished < nreq) {
			double tn = now() - t0;
			/* admit the arrived requests that fit, in arrival order */
			while (next < nreq && R[next].arrival <= tn && nact < slots && (nact == 0 || used + footprint(next) <= budget)) {
				setupRequest(next, 1);
				used += footprint(next);
				active[nact++] = next++;
			}
			if (!nact) {
				/* idle until the next arrival */
				while (now() - t0 < R[next].arrival) ;
				continue;
			}
			/* the admitted requests advance in parallel host threads: each
			 * world is stepped by one thread, in order, on its own streams */
			double ts = now();
			#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
			for (int a = 0; a < nact; a++) stepRequest(active[a], CHUNK);
			tStep += now() - ts;
			for (int a = 0; a < nact; a++) {
				int q = active[a];
				if (R[q].done < R[q].steps) continue;
				finishRequest(q);
				R[q].finish -= t0;
				used -= footprint(q);
				cellSteps += (double)R[q].cells * R[q].steps;
				finished++;
				active[a--] = active[--nact];
			}
		}
	}
	double wall = now() - t0;

	fflush(stdout);
	dup2(saved, 1);
	double lat[MAXREQ];
	int nl = 0;
	for (int q = 0; q < nreq; q++) {
		if (R[q].finish < 0) continue;
		double l = R[q].finish - R[q].arrival;
		lat[nl++] = l;
		union { double d; uint64_t u; } v = { R[q].result };
		printf("R %d %d %ld %d %.3f %016llx\n", q, R[q].kind, R[q].cells, R[q].steps, 1e3 * l, (unsigned long long)v.u);
	}
	qsort(lat, nl, sizeof *lat, cmpd);
	double p50 = lat[(nl - 1) / 2], p99 = lat[(int)(0.99 * (nl - 1))];
	printf("{\"mode\": \"%s\", \"requests\": %d, \"offered_per_s\": %g, \"seed\": %s, \"mix\": \"%s\", \"slots\": %d, "
	       "\"budget_gb\": %g, \"wall_s\": %.4f, \"cell_updates\": %.6g, \"gcell_per_s\": %.4f, "
	       "\"latency_ms\": {\"p50\": %.3f, \"p99\": %.3f, \"max\": %.3f}, \"achieved_per_s\": %.3f, "
	       "\"host_s\": {\"setup\": %.4f, \"step\": %.4f, \"finish\": %.4f}, \"threads\": %d}\n",
	       mode, finished, rate, argv[4], argv[5], slots, budget / 1e9, wall, cellSteps,
	       cellSteps / wall / 1e9, 1e3 * p50, 1e3 * p99, 1e3 * lat[nl - 1], finished / wall, tSetup, tStep, tFinish,
	       strcmp(mode, "served") && strcmp(mode, "batched") ? 1 : threads);
	return 0;
}
