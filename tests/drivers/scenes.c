/*
 * scenes.c -- parity scenarios written against the public ALiS API.
 *
 * One source, three builds: the reference library (golden fixtures), the
 * oracle restatement (CPU checker) and the GPU engine.  Each scenario
 * builds a world, runs `steps` time steps with phaser accumulation, and
 * dumps material maps, fields, ADE currents, phaser faces, fluxes and a
 * few far-field values (dump.h format).
 *
 *   scenes <scene> <out.bin> [scale] [steps]
 *
 * Scenes (scaled-down versions of the benchmark configurations):
 *   c1      vacuum plane wave, periodic x/y, CPML z, planar phasers
 *   nug     non-uniform (graded) grid, dispersive block, dipole, CPML
 *   beam    focused beam over the whole domain; beamtf through a TFSF box
 *           with a 3-D auxiliary world
 *   shg     second-order coupling: second harmonic of a pump world and
 *           three-wave mixing of a signal world with itself and the pump
 *   spheres 20 seeded Drude-Lorentz balls in a dielectric host
 *   unitcell periodic metasurface unit cell (TiO2-like pillar, substrate)
 *   bowtie  Drude bowtie antenna: symmetry planes, graded grid, edge-rule
 *           sub-pixel filling, compound shapes
 *   c2      gold block (Drude + 2 critical-point poles) in a TFSF box,
 *           CPML on all faces, box phasers, far field
 *   dipole  soft dipole, dielectric ball (12^3 supersampling) and a
 *           Drude box, CPML box
 *   bloch   oblique plane wave, Bloch x (complex fields), Lorentz pillar
 *           on a substrate
 *   sym     dipole on two symmetry planes, Drude-Lorentz sphere
 *   hbc     hexagonal-Bloch lattice slab with an iHz dipole
 *   multi   overlapping Drude-Lorentz spheres in a dielectric host
 *   shapes  every shape of the object API, nested compounds, plain and
 *           dispersive matter; 4^3 supersampling (shapespt: point
 *           samples, shapesedge: the edge rule)
 *   contour a height-map object, filled by the host loops
 *   pec     a PEC mirror under silver and a lossy (nk) film, symmetry
 *           planes and periodic walls, a single-wavelength phaser
 *   aniso   an anisotropic Drude-Lorentz ball, box phasers, far-field
 *           intensities and ring fluxes
 *   lattice a dipole array (symmetry planes and periodic walls) with a
 *           phaser box over three periods: replicated phasers and the
 *           far field's lattice factor
 *   farmaps the dipole world's far-field maps: farFieldProfile images of
 *           all seven polarisations over two projections (one of them
 *           logarithmic) and the farFieldTheta / farFieldPhi cuts
 *   c5      a (64 scale)^3 window of the large-domain precision world:
 *           its seeded Drude-Lorentz balls clipped to the window in a
 *           dielectric host, 16-cell CPML, two pulsed dipoles, box phasers
 */
#include <alis.h>
#include "dump.h"
#include "../../alis_gb300/bench/c5_balls.h"

static int scale = 1;

/* seeded Drude + critical-point gold: CP amplitude A in [0.3,1.5], phase
 * in [-pi,pi), mapped to ALiS (f, g) by g = -2A sin(phi),
 * f = 2A cos(phi) + g Gamma/Omega */
static matter seededGold(unsigned long long seed)
{
	lcgSeed(seed);
	matter M = {{2.1452}, {{8.557, 0.0658}, {2.6203, 0.2147}, {3.1543, 1.1662}}};
	for (int p = 1; p <= 2; p++) {
		float A = 0.3f + 1.2f * lcgUniform();
		float ph = -PI + 2 * PI * lcgUniform();
		float g = -2 * A * sinf(ph);
		M.P[p].g = g;
		M.P[p].f = 2 * A * cosf(ph) + g * M.P[p].r / M.P[p].w;
	}
	return M;
}

static void farSamples(phaser P, const char *tag)
{
	float th[5] = { 0, 30, 60, 150, 180 }, ph[5] = { 0, 45, 0, 90, 0 };
	char nm[64];
	for (int a = 0; a < 5; a++) {
		snprintf(nm, 64, "%s.ffP.%d", tag, a); dumpCScalar(nm, farField(P, Ppol, th[a], ph[a]));
		snprintf(nm, 64, "%s.ffS.%d", tag, a); dumpCScalar(nm, farField(P, Spol, th[a], ph[a]));
	}
}

/* called after every step of run() when set: per-step observers */
static void (*perStep)(world W, int n, int steps);

static void run(world W, phaser P, int steps)
{
	for (int n = 1; n <= steps; n++) {
		updateE(W);
		updateH(W);
		if (P) updatePhaser(W, P);
		if (perStep) perStep(W, n, steps);
	}
}

/* a slice writer that dumps frames 1 and 4 (phase 0 and 90 degrees) of
 * each sliceFreqDom output and the scale it was given */
static void dumpFrames(world W, slice S, float Max, char *F, char *filename, unsigned long int *cmap)
{
	(void)W, (void)F, (void)cmap;
	size_t n = strlen(filename);
	if (n < 2 || (strcmp(filename + n - 2, "01") && strcmp(filename + n - 2, "04"))) return;
	static int count;
	char nm[160];
	snprintf(nm, sizeof nm, "FD.%s.%d", filename, count);
	dumpField(nm, S->F, S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
	snprintf(nm, sizeof nm, "FD.%s.%d.max", filename, count++);
	dumpScalar(nm, Max);
}

/* frequency-domain slices: E/H samples the device accumulates, and
 * currents and incident/scattered fields the host loop does */
static slice fdA, fdB;

static void fdSym(world W, int n, int steps)
{
	(void)n;
	sliceFreqDom(W, Ex, fdA, steps / 2, 600, dumpFrames, "a%%");
	sliceFreqDom(W, Hz, fdA, steps / 2, 550, dumpFrames, "a%%");
	sliceFreqDom(W, rawEy, fdB, steps / 2, 600, dumpFrames, "b%%");
	sliceFreqDom(W, Jx, fdA, steps / 2, 600, dumpFrames, "a%%");
}

static void fdBloch(world W, int n, int steps)
{
	(void)n;
	sliceFreqDom(W, Ex, fdA, steps / 2, 550, dumpFrames, "a%%");
	sliceFreqDom(W, iEx, fdA, steps / 2, 550, dumpFrames, "a%%");
	sliceFreqDom(W, iHy, fdB, steps / 2, 550, dumpFrames, "b%%");
	sliceFreqDom(W, rawHz, fdB, steps / 2, 500, dumpFrames, "b%%");
}

static void fdC2(world W, int n, int steps)
{
	(void)n;
	sliceFreqDom(W, Ez, fdA, steps / 2, 600, dumpFrames, "a%%");
	sliceFreqDom(W, Hy, fdB, steps / 2, 600, dumpFrames, "b%%");
	sliceFreqDom(W, ScEx, fdA, steps / 2, 600, dumpFrames, "a%%");
	sliceFreqDom(W, Jx, fdB, steps / 2, 600, dumpFrames, "b%%");
}

static void sceneC1(int steps)
{
	int half = 16 * scale;                       /* cells per lateral half */
	dom D = {{-10*half, 10*(half-1)}, {-10*half, 10*(half-1)}, {-10*20*scale, 10*20*scale}};
	res R = {5, {10}, {1240}};
	sur S = {{PBC}, {PBC}, {PML, PML}, {16}};
	world W = createWorld(D, R, S, "");
	dom T = {{D.x.Min, D.x.Max}, {D.y.Min, D.y.Max}, {W->ktoz(W, W->kMIN+20), W->zMax-30}};
	planewave(W, T, Ppol, 180, 0, Pulse, 600, 90);
	phaser P = createPhasers(W, 400, 800, 400.0/15, -INF, INF, -INF, INF, 100, 100);
	run(W, P, steps);
	dumpWorld(W, "W");
	dumpWorld(W->S->W, "A");
	dumpPhasers(P, "P");
}

static void sceneC2(int steps)
{
	float L = 60 * scale;
	dom D = {{-L, L-2}, {-L, L-2}, {-L, L-2}};
	dom T = {{-L+10, L-12}, {-L+10, L-12}, {-L+10, L-12}};
	res R = {1, {2}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {12}};
	world W = createWorld(D, R, S, "");
	object Block = {Box, {{-40, 40}, {-20, 20}, {-15, 15}}};
	putObjects(W, seededGold(1234), Block, Air);
	planewave(W, T, Ppol, 0, 0, Pulse, 600, 200);
	phaser P = createPhasers(W, 400, 800, 400.0/7, -L+6, L-8, -L+6, L-8, -L+6, L-8);
	fdA = createSlice(W, -INF, INF, 0, 0, -INF, INF);
	fdB = createSlice(W, -30, 30, -20, 20, L-12, L-12);
	perStep = fdC2;
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Block));
	dumpWorld(W, "W");
	dumpWorld(W->S->W, "A");
	dumpPhasers(P, "P");
	farSamples(P + 3, "F");
}

static void sceneDipole(int steps)
{
	float L = 100 * scale;
	dom D = {{L}, {L}, {L}};
	res R = {5, {10}, {1240}};
	sur S = {{PML}};
	world W = createWorld(D, R, S, "");
	object Ball1 = {Ball, {{-60, 20}, {-40, 40}, {-30, 50}}};
	object Bar = {Box, {{20, 70}, {-20, 20}, {-80, -40}}};
	matter Ag1 = {{4.0323}, {{9.1864, 0.021}}};
	putObjects(W, n(1.5), Ball1, Ag1, Bar, Air);
	pointDipole(W, Ez, 5, 0, 0, Band, 400, 800);
	pointDipole(W, Hx, -20, 10, 30, Pulse, 500, 100, 0.5, 30);
	phaser P = createPhasers(W, 400, 800, 100, -L+20, L-20, -L+20, L-20, -L+20, L-20);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Bar));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
	farSamples(P + 1, "F");
}

static void sceneBloch(int steps)
{
	int half = 8 * scale;
	dom D = {{-10*half, 10*(half-1)}, {-10*half, 10*(half-1)}, {-300, 300}};
	res R = {5, {10}, {1240}};
	sur S = {{BBC}, {PBC}, {PML}, {10}};
	world W = createWorld(D, R, S, "");
	object Pillar = {RodZ, {{-50, 40}, {-40, 50}, {-100, 100}}};
	object Sub = {Box, {{-INF, INF}, {-INF, INF}, {-INF, -100}}};
	matter TiO2 = {{5.5}, {{4.5, 0.05, 1.0}}};
	putObjects(W, TiO2, Pillar, n(1.45), Sub, Air);
	dom T = {{D.x.Min, D.x.Max}, {D.y.Min, D.y.Max}, {-200, 250}};
	planewave(W, T, Ppol, 150, 0, Pulse, 550, 120);
	phaser P = createPhasers(W, 450, 700, 125, -INF, INF, -INF, INF, -250, -250);
	fdA = createSlice(W, -INF, INF, 0, 0, -INF, INF);
	fdB = createSlice(W, -INF, INF, -INF, INF, 150, 150);
	perStep = fdBloch;
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Pillar));
	dumpWorld(W, "W");
	dumpWorld(W->S->W, "A");
	dumpPhasers(P, "P");
}

static void sceneSym(int steps)
{
	float L = 80 * scale;
	dom D = {{L}, {L}, {L}};
	res R = {5, {10}, {1240}};
	sur S = {{SYM, PML}, {SYM, PML}, {PML}};
	world W = createWorld(D, R, S, "");
	object Sphere = {Ball, {{-40, 40}, {-40, 40}, {20, 60}}};
	matter DL = {{2.0}, {{7.0, 0.1}, {3.0, 0.3, 1.5}}};
	putObjects(W, DL, Sphere, Air);
	pointDipole(W, Ex, 0, 0, -20, Band, 400, 800);
	phaser P = createPhasers(W, 400, 800, 100, -L+20, L-20, -L+20, L-20, -L+20, L-20);
	/* slices reaching across the symmetry planes (mirrored samples) */
	fdA = createSlice(W, -60, 60, -60, 60, 40, 40);
	fdB = createSlice(W, -70, 70, 10, 10, -20, -20);
	perStep = fdSym;
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Sphere));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
	farSamples(P + 1, "F");
}

static void sceneHBC(int steps)
{
	float kx = 0.2f, ky = 1;
	dom D = {{100}, {0, 100*sqrtf(3)}, {200}};
	res R = {5, {10, 5*sqrtf(3), 10}, {1240}};
	sur S = {{BBC, 200*3/kx}, {HBC, 200*sqrtf(3)/ky}, {SYM, PML}};
	world W = createWorld(D, R, S, "");
	object Slab = {Difference, {2}, objects {
		{Box, {{-INF, INF}, {-INF, INF}, {-40, 40}}},
		{DLattice, {{200}, {200*sqrtf(3)}}, objects {{RodZ, {{-60, 60}, {-60, 60}, {-INF, INF}}}}},
	}};
	putObjects(W, n(3.5), Slab, Air);
	pointDipole(W, iHz, 40, 20*sqrtf(3), 0, Band, 750, 2000);
	run(W, 0, steps);
	dumpWorld(W, "W");
	(void)scale;
}

static void sceneMulti(int steps)
{
	float L = 80 * scale;
	dom D = {{-L, L-5}, {-L, L-5}, {-L, L-5}};
	res R = {2.5, {5}, {1240}};
	sur S = {{PBC}, {PBC}, {PML}, {8}};
	world W = createWorld(D, R, S, "");
	lcgSeed(99);
	object O[7];
	matter M[7];
	for (int q = 0; q < 6; q++) {
		float r = 10 + 20 * lcgUniform(), x = -50 + 100 * lcgUniform(), y = -50 + 100 * lcgUniform(), z = -40 + 80 * lcgUniform();
		O[q] = (object){Ball, {{x-r, x+r}, {y-r, y+r}, {z-r, z+r}}};
		M[q] = (matter){{1.5f + lcgUniform()}, {{6 + 3*lcgUniform(), 0.05f + 0.1f*lcgUniform()}, {2.5f + lcgUniform(), 0.2f, 0.5f + lcgUniform()}}};
	}
	O[6] = (object){0};
	M[6] = n(1.5);
	putObjectArray(W, M, O);
	dom T = {{D.x.Min, D.x.Max}, {D.y.Min, D.y.Max}, {-L+15, L-20}};
	planewave(W, T, Spol, 180, 0, Pulse, 600, 150);
	phaser P = createPhasers(W, 450, 750, 150, -INF, INF, -INF, INF, L-15, L-15);
	run(W, P, steps);
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* non-uniform grid (graded cells near the centre on every axis), a
 * Drude-Lorentz block off-centre, a dipole, CPML, box phasers */
static void sceneNug(int steps)
{
	float L = 200 * scale;
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {5, {20}, {1240}, {{3, 60}, {2, 80}, {4, 50}}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world W = createWorld(D, R, S, "");
	object Blk = {Box, {{30, 90}, {-40, 20}, {-30, 50}}};
	matter DL = {{2.5}, {{6.0, 0.2}, {3.5, 0.4, 1.2}}};
	putObjects(W, DL, Blk, Air);
	pointDipole(W, Ez, -20, 10, 0, Band, 400, 800);
	phaser P = createPhasers(W, 400, 800, 100, -L+40, L-40, -L+40, L-40, -L+40, L-40);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Blk));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
	farSamples(P + 1, "F");
}

/* focused beams: injected directly over the whole domain (tf = 0) or
 * through a TFSF box whose auxiliary world is a 3-D world (tf = 1) */
static void sceneBeam(int steps, int tf)
{
	float L = 300 * scale;
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {10, {20}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world W = createWorld(D, R, S, "");
	object Ball1 = {Ball, {{-60, 60}, {-60, 60}, {40, 160}}};
	putObjects(W, n(1.8), Ball1, Air);
	if (tf) {
		dom T = {{-L+60, L-60}, {-L+60, L-60}, {-L+60, L-60}};
		focusedBeam(W, T, Ex, 0, INF, 0, 0, Sine, 500, 3, 150);
	} else {
		focusedBeam(W, D, Ey, 0, INF, 0, 0, Sine, 500, 3, 150);
	}
	phaser P = createPhasers(W, 450, 550, 50, -L+40, L-40, -L+40, L-40, -L+40, L-40);
	run(W, P, steps);
	dumpWorld(W, "W");
	if (W->S) dumpWorld(W->S->W, "A");
	dumpPhasers(P, "P");
}

/* second-order coupling: a pump world driven by a dipole, a signal world
 * with a chi2 dispersive block, second-harmonic generation from the pump
 * and three-wave mixing of the signal with the pump */
static void sceneSHG(int steps)
{
	float L = 120 * scale;
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {5, {10}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world WP = createWorld(D, R, S, "");
	world WS = createWorld(D, R, S, "");
	object Blk = {Box, {{-50, 50}, {-40, 30}, {-30, 40}}};
	matter Chi = {{4.5}, {{6.0, 0.1, 0.5}}, {{0.1, 0.2, 0, 0, 0.3, 0}, {0, 0, 0.15, 0.4, 0, 0.2}, {0.3, 0.1, 0.5, 0, 0, 0.25}}};
	putObjects(WS, Chi, Blk, Air);
	putObjects(WP, n(2.0), Blk, Air);
	pointDipole(WP, Ez, -30, 10, 0, Pulse, 500, 100, 50);
	for (int n = 1; n <= steps; n++) {
		updateE(WP);
		updateH(WP);
		nonLinearSHG(WS, WP, 1);
		nonLinearTWM(WS, WS, WP, -0.5);
		updateE(WS);
		updateH(WS);
	}
	dumpWorld(WS, "W");
	dumpWorld(WP, "A");
}

/* the large-domain study in miniature: 20 seeded Drude-Lorentz balls in
 * a dielectric host (more than 8 dispersive objects: the kernels' per-tile
 * object lists), overlaps resolved by list order, a dipole, box phasers */
static void sceneSpheres(int steps)
{
	float L = 160 * scale;
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {5, {10}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world W = createWorld(D, R, S, "");
	enum { NB = 20 };
	object O[NB + 1];
	matter M[NB + 1];
	lcgSeed(99);
	for (int q = 0; q < NB; q++) {
		/* one draw per statement: the order is fixed */
		float r = 20 + 40 * lcgUniform();
		float x = -L + 50 + (2 * L - 100) * lcgUniform();
		float y = -L + 50 + (2 * L - 100) * lcgUniform();
		float z = -L + 50 + (2 * L - 100) * lcgUniform();
		float e = 1.5 + lcgUniform(), wp = 5 + 4 * lcgUniform(), g = 0.05 + 0.2 * lcgUniform();
		float w0 = 3 + lcgUniform(), f0 = 0.5 + lcgUniform();
		O[q] = (object){Ball, {{x - r, x + r}, {y - r, y + r}, {z - r, z + r}}};
		M[q] = (matter){{e}, {{wp, g}, {w0, 0.2, f0}}};
	}
	O[NB] = (object){0};
	M[NB] = n(1.5);
	putObjectArray(W, M, O);
	pointDipole(W, Ex, 5, -10, 15, Band, 400, 800);
	phaser P = createPhasers(W, 400, 800, 200, -L+30, L-30, -L+30, L-30, -L+30, L-30);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, O[3]));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* the large-domain precision workload's sub-runs (configuration 5): a
 * (64 scale)^3-cell window at the centre of the 1024 x 1024 x 512 world,
 * with a 16-cell CPML of its own: the full world's 200 balls from seed 99
 * (c5_balls.h, as the bench world draws them), clipped to the window --
 * those reaching at least 2 cells into it -- in the n = 1.5 host; two
 * pulsed dipoles and a 16-frequency phaser box 4 cells inside the CPML.
 * Scale 4 is the 256^3 sub-run of the precision study. */
static void sceneC5(int steps)
{
	const float dx = 5;
	const int full[3] = { 1024 - 34, 1024 - 34, 512 - 34 }, in = 64 * scale - 34;
	const int sub[3] = { in, in, in };
	c5Real flo[3], fhi[3], lo[3], hi[3];
	c5Domain(full, dx, flo, fhi);
	c5Domain(sub, dx, lo, hi);
	dom D = {{lo[0], hi[0]}, {lo[1], hi[1]}, {lo[2], hi[2]}};
	res R = {2.5, {dx}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {16}};
	world W = createWorld(D, R, S, "");
	enum { NB = 200 };
	static c5Ball B[NB];
	c5Balls(99, NB, flo, fhi, dx, B);
	object O[NB + 1];
	matter M[NB + 1];
	int nb = 0;
	for (int q = 0; q < NB; q++) {
		const c5Ball b = B[q];
		const c5Real c[3] = { b.x, b.y, b.z };
		c5Real d2 = 0;
		for (int a = 0; a < 3; a++) {
			const c5Real e = c[a] < lo[a] ? lo[a] - c[a] : c[a] > hi[a] ? c[a] - hi[a] : 0;
			d2 += e * e;
		}
		const c5Real deep = b.r - 2 * dx;
		if (deep <= 0 || d2 >= deep * deep) continue;
		O[nb] = (object){Ball, {{b.x - b.r, b.x + b.r}, {b.y - b.r, b.y + b.r}, {b.z - b.r, b.z + b.r}}};
		M[nb++] = (matter){{b.e}, {{b.wp, b.g}, {b.w0, 0.2, b.f0}}};
	}
	O[nb] = (object){0};
	M[nb] = n(1.5);
	putObjectArray(W, M, O);
	pointDipole(W, Ex, 0, 0, D.z.Min / 2, Pulse, 600, 150);
	pointDipole(W, Ez, D.x.Max / 3, D.y.Min / 3, 0, Pulse, 500, 100);
	const float m = 4 * dx;
	phaser P = createPhasers(W, 400, 800, 400.0 / 15, D.x.Min + m, D.x.Max - m, D.y.Min + m, D.y.Max - m, D.z.Min + m, D.z.Max - m);
	run(W, P, steps);
	dumpScalar("S.balls", nb);
	if (nb) dumpScalar("S.abs", objectAbsorption(W, O[0]));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* a metasurface unit cell of the batched sweep: periodic x/y, CPML z, a
 * TiO2-like Lorentz pillar on a glass substrate, a normal-incidence pulse,
 * a transmission phaser plane */
static void sceneUnitCell(int steps)
{
	float a = 240 * scale;
	dom D = {{-a/2, a/2 - 10}, {-a/2, a/2 - 10}, {-400, 400}};
	res R = {5, {10}, {1240}};
	sur S = {{PBC}, {PBC}, {PML, PML}, {10}};
	world W = createWorld(D, R, S, "");
	object Pillar = {RodZ, {{-70, 70}, {-70, 70}, {-200, 150}}};
	object Sub = {Box, {{-INF, INF}, {-INF, INF}, {-INF, -200}}};
	matter TiO2 = {{5.5}, {{4.5, 0.05, 1.0}}};
	putObjects(W, TiO2, Pillar, n(1.45), Sub, Air);
	dom T = {{D.x.Min, D.x.Max}, {D.y.Min, D.y.Max}, {-300, 300}};
	planewave(W, T, Ppol, 0, 0, Pulse, 600, 150);
	phaser P = createPhasers(W, 450, 750, 100, -INF, INF, -INF, INF, 320, 320);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Pillar));
	dumpWorld(W, "W");
	dumpWorld(W->S->W, "A");
	dumpPhasers(P, "P");
}

/* a Drude-metal bowtie antenna of the served mix: symmetry planes, a
 * graded grid, the edge rule of sub-pixel filling (subN < 0), compound
 * shapes, a substrate, a dipole in the gap */
static void sceneBowtie(int steps)
{
	float g = 20, r = 20, d = 60 * scale;
	dom D = {{160 * scale}, {120 * scale}, {-100, 100}};
	res R = {2.5, {5}, {1240, -1}, {{3, g/2 + d}, {3, r + (d - 2*r) / sqrtf(3)}, {3, 15}}};
	sur S = {{SYM, PML}, {SYM, PML}, {PML, PML}, {8}};
	world W = createWorld(D, R, S, "");
	float s3 = sqrtf(3);
	object Bowtie = {Combination, {3}, objects {
		{RodZ, {{g/2, g/2 + r*2}, {-r, r}, {-15, 15}}},
		{RodZ, {{g/2 - r*2 + d, g/2 + d}, {-r + (d - 2*r)/s3, r + (d - 2*r)/s3}, {-15, 15}}},
		{Intersection, {2}, objects {
			{Box, {{g/2 + r/2, g/2 + d}, {-(d - r/2)/s3, (d - r/2)/s3}, {-15, 15}}},
			{DRodZ, {{g/2 - r, g/2 - r*2 + d*2}, {-(d - r/2)/s3, (d - r/2)/s3}, {-15, 15}}},
		}}
	}};
	object Substrate = {Box, {{-INF, INF}, {-INF, INF}, {-INF, -15}}};
	matter Ag2 = {{4.0}, {{9.0, 0.02}}};
	putObjects(W, Ag2, Bowtie, n(1.5), Substrate, Air);
	pointDipole(W, Ex, 0, 0, 0, Band, 400, 1000);
	phaser P = createPhasers(W, 400, 1000, 200, -INF, INF, -INF, INF, -80, 80);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Bowtie));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* every shape of the object API in one list: basic shapes, translated,
 * rotated, set operations, finite, doubled, infinite and rotational
 * lattices, nested up to three deep; plain and dispersive matter,
 * overlaps resolved by list order, sub-pixel filling by subN
 * (supersampling, point samples or the edge rule for subN < 0) */
static void sceneShapes(int steps, int subN)
{
	float L = 200 * scale;
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {5, {10}, {1240, subN}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world W = createWorld(D, R, S, "");
	matter Drude = {{2.0}, {{8.0, 0.05}}};
	matter Lorentz = {{2.5}, {{4.0, 0.1, 0.8}}};
	float zb[2] = { -130, -70 };
#define AT(x, y) {{(x) - 28, (x) + 28}, {(y) - 28, (y) + 28}, {zb[0], zb[1]}}
	object O[] = {
		/* basic shapes, z in [-130, -70] */
		{Ball, AT(-120, -120)}, {Diamond, AT(-40, -120)}, {BiconeX, AT(40, -120)}, {BiconeY, AT(120, -120)},
		{BiconeZ, AT(-120, -40)}, {RodX, AT(-40, -40)}, {RodY, AT(40, -40)}, {RodZ, AT(120, -40)},
		{DRodX, AT(-120, 40)}, {DRodY, AT(-40, 40)}, {DRodZ, AT(40, 40)}, {HRodXY, AT(120, 40)},
		{HRodYZ, AT(-120, 120)}, {HRodZX, AT(-40, 120)}, {HRodXZ, AT(40, 120)}, {HRodYX, AT(120, 120)},
		/* compound shapes, z around 0 */
		{HRodZY, {{-150, -90}, {-150, -90}, {-30, 30}}},
		{Translation, {{-40, -120, 0}}, objects {{Ball, {{-25, 25}, {-20, 20}, {-30, 30}}}}},
		{Rotation, {{30, 20, 45}, {40, -120, 0}}, objects {{Box, {{-25, 25}, {-15, 15}, {-20, 20}}}}},
		{Difference, {{2}}, objects {
			{Box, {{95, 150}, {-150, -95}, {-25, 25}}},
			{Ball, {{110, 140}, {-140, -110}, {-40, 40}}}}},
		{Combination, {{3}}, objects {
			{Box, {{-150, -110}, {-60, -20}, {-20, 20}}},
			{RodX, {{-110, -60}, {-50, -30}, {-15, 15}}},
			{Intersection, {{2}}, objects {
				{Ball, {{-75, -25}, {-65, -15}, {-25, 25}}},
				{Box, {{-60, -20}, {-80, 0}, {-10, 30}}}}}}},
		{Translation, {{80, -40, 0}}, objects {{Lattice, {{25, 3}, {25, 2}, {0}}, objects {
			{Ball, {{-8, 8}, {-9, 9}, {-20, 20}}}}}}},
		{Translation, {{-80, 40, 0}}, objects {{DLattice, {{22, 3}, {22, 3}, {0}}, objects {
			{Box, {{-6, 6}, {-6, 6}, {-25, 25}}}}}}},
		{CLatticeZ, {{5}, {80, 40}}, objects {{RodZ, {{95, 112}, {32, 48}, {-30, 30}}}}},
		{CLatticeX, {{6}, {120, 0}}, objects {{Ball, {{-150, -95}, {128, 146}, {-9, 9}}}}},
		{CLatticeY, {{4}, {-40, 0}}, objects {{RodY, {{-28, -12}, {100, 150}, {12, 28}}}}},
		{Intersection, {{2}}, objects {
			{Box, {{20, 150}, {100, 150}, {-30, 30}}},
			{Lattice, {{25, 0}, {0}, {0}}, objects {{RodY, {{-6, 6}, {-INF, INF}, {-20, 20}}}}}}},
		/* a dispersive slab on top, partly under earlier objects, and a
		 * rotated compound */
		{Box, {{-150, 150}, {-150, 0}, {60, 110}}},
		{Rotation, {{-20, 35, 10}, {60, 80, 90}}, objects {{Combination, {{2}}, objects {
			{RodZ, {{-12, 12}, {-12, 12}, {-25, 25}}},
			{Translation, {{10, 0, 0}}, objects {{Box, {{-5, 25}, {-5, 5}, {-20, 20}}}}}}}}},
		{0},
	};
#undef AT
	int N = sizeof O / sizeof *O - 1;
	matter M[sizeof O / sizeof *O];
	for (int o = 0; o < N; o++) M[o] = n(1.3 + 0.07 * o);
	M[7] = Drude, M[19] = Lorentz, M[24] = Drude, M[27] = Lorentz;
	M[N] = Air;
	putObjectArray(W, M, O);
	pointDipole(W, Ez, 5, -10, 0, Band, 400, 800);
	phaser P = createPhasers(W, 400, 800, 200, -L+50, L-50, -L+50, L-50, -L+50, L-50);
	run(W, P, steps);
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* a height-map object (ImportContour) in the list: filled by the host
 * loops, as are lists holding any shape outside the object API's own */
static float contourMap[16][16], *contourRows[16];

static void sceneContour(int steps)
{
	float L = 160 * scale;
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {5, {10}, {1240, 3}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world W = createWorld(D, R, S, "");
	for (int i = 0; i < 16; i++) {
		contourRows[i] = contourMap[i];
		for (int j = 0; j < 16; j++) contourMap[i][j] = (i - 7.5f) * (i - 7.5f) + 0.5f * (j - 7.5f) * (j - 7.5f);
	}
	object Hill = {Intersection, {{2}}, objects {
		{Box, {{-INF, INF}, {-INF, INF}, {-40, 40}}},
		{ImportContour, {{-100, 100, 16}, {-100, 100, 16}, {0, 30}}, contourRows}}};
	object Cap = {Ball, {{-50, 50}, {-50, 50}, {20, 80}}};
	matter Drude = {{2.0}, {{8.0, 0.05}}};
	putObjects(W, Drude, Cap, n(2), Hill, Air);
	pointDipole(W, Ex, 5, -10, 100, Band, 400, 800);
	phaser P = createPhasers(W, 400, 800, 200, -L+50, L-50, -L+50, L-50, -L+50, L-50);
	run(W, P, steps);
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* a PEC mirror: z-min PEC under a silver layer and a lossy film (nk: a
 * static conductivity and no poles), periodic x and y with symmetry
 * planes at their lower ends, a dipole on both symmetry planes, a
 * single-wavelength phaser plane */
static void scenePEC(int steps)
{
	float a = 60 * scale;
	dom D = {{a}, {a}, {-60, 240}};
	res R = {5, {10}, {1240}};
	sur S = {{SYM, PBC}, {SYM, PBC}, {PEC, PML}, {8}};
	world W = createWorld(D, R, S, "");
	matter Lossy = nk(2.2, 0.12, 1240/550);
	object Film = {Box, {{-INF, INF}, {-INF, INF}, {20, 60}}};
	object Mirror = {Box, {{-INF, INF}, {-INF, INF}, {-INF, 0}}};
	putObjects(W, Lossy, Film, Ag, Mirror, Air);
	pointDipole(W, Ex, 0, 0, 100, Pulse, 550, 60);
	phaser P = createPhaser(W, 550, -INF, INF, -INF, INF, 200, 200);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Film));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
}

/* an anisotropic dispersive ball (per-axis eps, one Drude and one Lorentz
 * pole per axis) lit by a dipole in a CPML box; box phasers and the
 * far-field aggregates: intensities per polarisation and ring fluxes */
static void sceneAniso(int steps)
{
	float L = 100 * scale;
	dom D = {{L}, {L}, {L}};
	res R = {5, {10}, {1240}};
	sur S = {{PML}};
	world W = createWorld(D, R, S, "");
	matter Aniso = {{2.0, 2.5, 3.0}, {{8.0, 0.1}, {7.5, 0.12}, {7.0, 0.15}, {3.0, 0.3, 1.5}, {3.2, 0.3, 1.2}, {3.4, 0.3, 1.0}}};
	object Egg = {Ball, {{-40, 30}, {-30, 30}, {-20, 40}}};
	putObjects(W, Aniso, Egg, Air);
	pointDipole(W, Ey, 10, -50, 0, Pulse, 500, 120);
	phaser P = createPhasers(W, 450, 750, 150, -L+20, L-20, -L+20, L-20, -L+20, L-20);
	run(W, P, steps);
	dumpScalar("S.abs", objectAbsorption(W, Egg));
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
	char nm[64];
	float th[4] = { 0, 35, 90, 140 }, ph[4] = { 0, 60, 20, 250 };
	tfield (*pol[3])(phaser, float, float) = { Ppol, Spol, Unpol };
	for (int a = 0; a < 4; a++) for (int q = 0; q < 3; q++) {
		snprintf(nm, 64, "FA.I.%d.%d", a, q); dumpScalar(nm, farFieldI(P + 1, pol[q], th[a], ph[a]));
	}
	dumpScalar("FA.flux.0", farFieldFlux(P + 1, Unpol, 0, 0, 30));
	dumpScalar("FA.flux.1", farFieldFlux(P + 1, Ppol, 180, 0, 10, 40, 5));
}

/* a dipole array: one cell with symmetry planes at its lower ends and
 * periodic upper walls, a dielectric post; the phaser box spans three
 * periods each way, so the phasers replicate over the lattice and the far
 * field carries the lattice factor */
static void sceneLattice(int steps)
{
	float a = 40 * scale;
	dom D = {{a}, {a}, {150}};
	res R = {5, {10}, {1240}};
	sur S = {{SYM, PBC}, {SYM, PBC}, {PML}};
	world W = createWorld(D, R, S, "");
	object Post = {Box, {{-20, 20}, {-20, 20}, {-60, -20}}};
	putObjects(W, n(2.0), Post, Air);
	pointDipole(W, Ex, 0, 0, 20, Pulse, 550, 100);
	phaser P = createPhasers(W, 450, 700, 125, -3*a, 3*a, -3*a, 3*a, -100, 100);
	run(W, P, steps);
	dumpWorld(W, "W");
	dumpPhasers(P, "P");
	char nm[64];
	for (int q = 0; P[q].f; q++) {
		snprintf(nm, 64, "FL.%d.num", q); dumpScalar(nm, P[q].xNUM * 1000 + P[q].yNUM);
	}
	farSamples(P + 1, "FL");
}

/* an image writer for farFieldProfile: dumps the image and the scale it
 * was given under the name of the file it would have written */
static void dumpImage(world W, slice S, float Max, char *F, char *filename, unsigned long int *cmap)
{
	(void)W, (void)F, (void)cmap;
	char nm[160];
	snprintf(nm, sizeof nm, "FP.%s", filename);
	dumpField(nm, S->F, S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
	snprintf(nm, sizeof nm, "FP.%s.max", filename);
	dumpScalar(nm, Max);
}

/* the rows farFieldTheta / farFieldPhi wrote to <name>.txt, as an
 * n x 4 array (angle, unpolarised, P, S) */
static void dumpRows(const char *name, const char *path)
{
	fflush(NULL);
	FILE *f = fopen(path, "r");
	if (!f) { perror(path); exit(2); }
	float v[360][4];
	int n = 0;
	while (n < 360 && fscanf(f, "%f %f %f %f", &v[n][0], &v[n][1], &v[n][2], &v[n][3]) == 4) n++;
	fclose(f);
	dumpHeader(name, DUMP_REAL, n, 4, 1);
	for (int r = 0; r < n; r++) for (int c = 0; c < 4; c++) fwrite(&v[r][c], sizeof(float), 1, dumpFile);
}

/* the far-field maps: a dispersive ball and a silver bar lit by two
 * dipoles in a CPML box; polarisation images over a cylindrical and an
 * azimuthal (logarithmic) projection, and the theta and phi cuts */
static void sceneFarMaps(int steps)
{
	float L = 100 * scale;
	dom D = {{L}, {L}, {L}};
	res R = {5, {10}, {1240}};
	sur S = {{PML}};
	world W = createWorld(D, R, S, "");
	object Ball1 = {Ball, {{-60, 20}, {-40, 40}, {-30, 50}}};
	object Bar = {Box, {{20, 70}, {-20, 20}, {-80, -40}}};
	matter Ag1 = {{4.0323}, {{9.1864, 0.021}}};
	putObjects(W, n(1.5), Ball1, Ag1, Bar, Air);
	pointDipole(W, Ez, 5, 0, 0, Band, 400, 800);
	pointDipole(W, Hx, -20, 10, 30, Pulse, 500, 100, 0.5, 30);
	phaser P = createPhasers(W, 400, 800, 100, -L+20, L-20, -L+20, L-20, -L+20, L-20);
	run(W, P, steps);
	dumpPhasers(P, "P");
	farFieldProfile(W, P + 1, CylindericalMap, 16, 9, dumpImage, "cyl");
	farFieldProfile(W, P + 2, AzimuthalMap, 12, 7, dumpImage, "azLog");
	farFieldTheta(W, P + 1, 30, "theta");
	farFieldPhi(W, P + 2, 60, "phi");
	char path[1100];
	snprintf(path, sizeof path, "%stheta.txt", W->ID);
	dumpRows("FT.theta", path);
	snprintf(path, sizeof path, "%sphi.txt", W->ID);
	dumpRows("FT.phi", path);
}

int main(int argc, char **argv)
{
	if (argc < 3) {
		fprintf(stderr, "usage: %s scene out.bin [scale] [steps]\n", argv[0]);
		return 2;
	}
	if (argc > 3) scale = atoi(argv[3]);
	int steps = argc > 4 ? atoi(argv[4]) : 100;
	dumpOpen(argv[2]);
	const char *s = argv[1];
	if (!strcmp(s, "c1")) sceneC1(steps);
	else if (!strcmp(s, "c2")) sceneC2(steps);
	else if (!strcmp(s, "dipole")) sceneDipole(steps);
	else if (!strcmp(s, "bloch")) sceneBloch(steps);
	else if (!strcmp(s, "sym")) sceneSym(steps);
	else if (!strcmp(s, "hbc")) sceneHBC(steps);
	else if (!strcmp(s, "multi")) sceneMulti(steps);
	else if (!strcmp(s, "nug")) sceneNug(steps);
	else if (!strcmp(s, "beam")) sceneBeam(steps, 0);
	else if (!strcmp(s, "beamtf")) sceneBeam(steps, 1);
	else if (!strcmp(s, "shg")) sceneSHG(steps);
	else if (!strcmp(s, "spheres")) sceneSpheres(steps);
	else if (!strcmp(s, "unitcell")) sceneUnitCell(steps);
	else if (!strcmp(s, "bowtie")) sceneBowtie(steps);
	else if (!strcmp(s, "shapes")) sceneShapes(steps, 4);
	else if (!strcmp(s, "shapespt")) sceneShapes(steps, 1);
	else if (!strcmp(s, "shapesedge")) sceneShapes(steps, -1);
	else if (!strcmp(s, "contour")) sceneContour(steps);
	else if (!strcmp(s, "pec")) scenePEC(steps);
	else if (!strcmp(s, "aniso")) sceneAniso(steps);
	else if (!strcmp(s, "lattice")) sceneLattice(steps);
	else if (!strcmp(s, "farmaps")) sceneFarMaps(steps);
	else if (!strcmp(s, "c5")) sceneC5(steps);
	else { fprintf(stderr, "unknown scene %s\n", s); return 2; }
	dumpClose();
	return 0;
}
