/*
 * c2.c -- the dispersive-scatterer benchmark world, written against the
 * public ALiS API (the same calls a user program makes).
 *
 * 256^3 cells including CPML: dx = 2 nm, dt = 1 nm/c (Courant 0.5),
 * domain [-230, 228] nm per axis, 12-cell CPML on all faces; a gold block
 * 80 x 40 x 30 nm with one Drude pole (wp = 8.557 eV = 1.3e16 rad/s,
 * gamma = 0.0658 eV = 1e14 rad/s) and two critical-point poles (Omega,
 * Gamma of the Au fit; amplitude in [0.3, 1.5] and phase in [-pi, pi)
 * drawn from seed 1234); a Ppol pulse plane wave (600 nm, supplement 200)
 * from a TFSF box [-160, 158]^3 nm; 64-frequency box phasers (400-800 nm,
 * uniform in frequency) just outside the TFSF box.
 *
 * Exported for bench.py (engine build) and compiled into the CPU
 * baseline program (oracle build).  `half` scales the domain (230 = the
 * full configuration).
 *
 * c1_build makes the vacuum plane-wave workload in its place and c5_build
 * the large-domain precision workload (the stepping, result and byte
 * functions below serve whichever was built).  c5_build:
 * ni x nj x nk cells with a 16-cell CPML on all faces, dx = 5 nm, a
 * dielectric host (n = 1.5) holding `balls` Drude-Lorentz balls of radius
 * 20-80 cells drawn from seed 99 (c5_balls.h), two pulsed dipoles and an
 * `nfreq`-frequency phaser box 4 cells inside the CPML (1024 x 1024 x
 * 512, 200 balls, 128 frequencies: the full configuration).  E and H are
 * stored as float, or as half values with ALIS_FIELD_STORAGE=half.
 */
#include <alis.h>
#include "c5_balls.h"

static world W;
static phaser P;
static int nfreqs;

/* 64-bit LCG, top 24 bits -> [0, 1) */
static unsigned long long rngState;
static float uniform01(void)
{
	rngState = rngState * 6364136223846793005ULL + 1442695040888963407ULL;
	return (float)(rngState >> 40) / 16777216.0f;
}

static matter seededGold(unsigned long long seed)
{
	rngState = seed * 6364136223846793005ULL + 1442695040888963407ULL;
	matter M = {{2.1452}, {{8.557, 0.0658}, {2.6203, 0.2147}, {3.1543, 1.1662}}};
	for (int p = 1; p <= 2; p++) {
		float A = 0.3f + 1.2f * uniform01();
		float ph = -PI + 2 * PI * uniform01();
		float g = -2 * A * sinf(ph);
		M.P[p].g = g;
		M.P[p].f = 2 * A * cosf(ph) + g * M.P[p].r / M.P[p].w;
	}
	return M;
}

/* Build the world; returns the total cell count (iNUM jNUM kNUM). */
long c2_build(int half, int nfreq)
{
	float L = half;
	float T = half * 160.0f / 230.0f, Pb = T + 4;
	dom D = {{-L, L-2}, {-L, L-2}, {-L, L-2}};
	dom DT = {{-T, T-2}, {-T, T-2}, {-T, T-2}};
	res R = {1, {2}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {12}};
	W = createWorld(D, R, S, "");
	object Block = {Box, {{-40, 40}, {-20, 20}, {-15, 15}}};
	putObjects(W, seededGold(1234), Block, Air);
	planewave(W, DT, Ppol, 0, 0, Pulse, 600, 200);
	int want = nfreq > 1 ? nfreq : 64;
	P = createPhasers(W, 400, 800, 400.0f/(want-1), -Pb, Pb-2, -Pb, Pb-2, -Pb, Pb-2);
	for (nfreqs = 0; P[nfreqs].f; nfreqs++);
	return (long)W->iNUM * W->jNUM * W->kNUM;
}

/* the vacuum plane-wave workload in its place: n x n x n cells with the
 * CPML, dx = 10 nm, dt = 5 nm/c (Courant 0.5), periodic x and y, a 16-cell
 * CPML on both z faces, an x-polarized pulse plane wave (600 nm,
 * supplement 90) from the plane 20 cells above the low z CPML, and a
 * 16-wavelength (400-800 nm) phaser plane at z = 100 nm */
long c1_build(int n)
{
	const int h = n / 2, nz = n - 34;                /* interior z cells */
	dom D = {{-10*h, 10*(h-1)}, {-10*h, 10*(h-1)}, {-10*(nz/2), 10*(nz - nz/2 - 1)}};
	res R = {5, {10}, {1240}};
	sur S = {{PBC}, {PBC}, {PML, PML}, {16}};
	W = createWorld(D, R, S, "");
	dom T = {{D.x.Min, D.x.Max}, {D.y.Min, D.y.Max}, {W->ktoz(W, W->kMIN+20), W->zMax-30}};
	planewave(W, T, Ppol, 180, 0, Pulse, 600, 90);
	P = createPhasers(W, 400, 800, 400.0/15, -INF, INF, -INF, INF, 100, 100);
	for (nfreqs = 0; P[nfreqs].f; nfreqs++);
	return (long)W->iNUM * W->jNUM * W->kNUM;
}

long c5_build(int ni, int nj, int nk, int balls, int nfreq)
{
	const float dx = 5;
	const int n[3] = { ni - 34, nj - 34, nk - 34 };     /* interior cells */
	c5Real lo[3], hi[3];
	c5Domain(n, dx, lo, hi);
	dom D = {{lo[0], hi[0]}, {lo[1], hi[1]}, {lo[2], hi[2]}};
	res R = {2.5, {dx}, {1240}};
	sur S = {{PML}, {PML}, {PML}, {16}};
	W = createWorld(D, R, S, "");
	c5Ball *B = calloc(balls, sizeof *B);
	object *O = calloc(balls + 1, sizeof *O);
	matter *M = calloc(balls + 1, sizeof *M);
	c5Balls(99, balls, lo, hi, dx, B);
	for (int q = 0; q < balls; q++) {
		const c5Ball b = B[q];
		O[q] = (object){Ball, {{b.x - b.r, b.x + b.r}, {b.y - b.r, b.y + b.r}, {b.z - b.r, b.z + b.r}}};
		M[q] = (matter){{b.e}, {{b.wp, b.g}, {b.w0, 0.2, b.f0}}};
	}
	M[balls] = n(1.5);
	putObjectArray(W, M, O);
	free(B), free(O), free(M);
	pointDipole(W, Ex, 0, 0, D.z.Min / 2, Pulse, 600, 150);
	pointDipole(W, Ez, D.x.Max / 3, D.y.Min / 3, 0, Pulse, 500, 100);
	int want = nfreq > 1 ? nfreq : 128;
	const float m = 4 * dx;
	P = createPhasers(W, 400, 800, 400.0f/(want-1), D.x.Min + m, D.x.Max - m, D.y.Min + m, D.y.Max - m, D.z.Min + m, D.z.Max - m);
	for (nfreqs = 0; P[nfreqs].f; nfreqs++);
	return (long)W->iNUM * W->jNUM * W->kNUM;
}

/* n time steps: E half step, H half step, phaser accumulation */
void c2_steps(int n)
{
	for (int q = 0; q < n; q++) {
		updateE(W);
		updateH(W);
		updatePhaser(W, P);
	}
}

/* the same steps recorded into batched launches (alisBatchBegin/End), the
 * form that steps many worlds together, here with this world alone */
void c2_steps_batched(int n)
{
	for (int q = 0; q < n; q++) {
		alisBatchBegin();
		updateE(W);
		updateH(W);
		updatePhaser(W, P);
		alisBatchEnd();
	}
}

/* result of the run so far: total outgoing flux over all frequencies
 * (brings the phaser accumulators to the host) */
double c2_result(void)
{
	double s = 0;
	for (int f = 0; P[f].f; f++) s += phaserPoyntingOut(P + f);
	return s;
}

/* bytes moved per step by the reference formulation (one E+H update of
 * every cell; see the roofline accounting of the half-step kernel):
 * interior 84 B (72 without eps^-1 maps), +32 B per CPML slab a cell lies
 * in, +12 B fill + 24 B per Drude pole + 48 B per pair pole in dispersive
 * boxes. */
double c2_step_bytes(void)
{
	double cells = (double)W->iNUM * W->jNUM * W->kNUM;
	double bytes = cells * (W->CE->x ? 84 : 72);
	int lo[3] = { W->iMin - W->iMIN - 1, W->jMin - W->jMIN - 1, W->kMin - W->kMIN - 1 };
	int hi[3] = { W->iMAX - W->iMax - 1, W->jMAX - W->jMax - 1, W->kMAX - W->kMax - 1 };
	int num[3] = { W->iNUM, W->jNUM, W->kNUM };
	for (int a = 0; a < 3; a++) {
		double slab = (double)(MAX(lo[a], 0) + MAX(hi[a], 0));
		bytes += 32.0 * slab * (cells / num[a]);
	}
	coeffs *C = W->CE;
	for (int n = 0; n < C->N; n++) {
		double box = (double)(1 + C->iMax[n] - C->iMin[n]) * (1 + C->jMax[n] - C->jMin[n]) * (1 + C->kMax[n] - C->kMin[n]);
		bytes += box * (12 + 24.0 * C->NJ[n] + 48.0 * (C->NK[n] - C->NJ[n]));
	}
	return bytes;
}

/* the same with E and H stored as half values (ALIS_FIELD_STORAGE=half):
 * 36 of the 72 field bytes per cell */
double c2_step_bytes_half(void)
{
	return c2_step_bytes() - 36.0 * W->iNUM * W->jNUM * W->kNUM;
}

/* host bytes moved per step by the public-API path: source increments
 * and phase factors up, nothing down until c2_result */
double c2_step_h2d_bytes(void)
{
	long values = 0;
	for (tfsf S = W->S; S; S = S->S) {
		for (source s = S->W->SE; s; s = s->S) values += (1+s->iMax-s->iMin)*(1+s->jMax-s->jMin)*(1+s->kMax-s->kMin);
		for (source s = S->W->SH; s; s = s->S) values += (1+s->iMax-s->iMin)*(1+s->jMax-s->jMin)*(1+s->kMax-s->kMin);
	}
	return 4.0 * values + 16.0 * nfreqs;
}

/* bytes read back by c2_result: the flux of each of the 6 faces at every
 * frequency (the accumulators are reduced where they live) */
double c2_result_d2h_bytes(void)
{
	return 6.0 * sizeof(float) * nfreqs;
}

/* face cells of the phaser box: the faces the phaser keeps (reference
 * src/phaser.c:57-62), one cell thick */
double c2_phaser_face_cells(void)
{
	const double ni = 1 + P->iMax - P->iMin, nj = 1 + P->jMax - P->jMin, nk = 1 + P->kMax - P->kMin;
	const int on[6] = { P->xMin.Ey != 0, P->xMax.Ey != 0, P->yMin.Ez != 0, P->yMax.Ez != 0, P->zMin.Ex != 0, P->zMax.Ex != 0 };
	const double face[3] = { nj * nk, ni * nk, ni * nj };
	double cells = 0;
	for (int s = 0; s < 6; s++) if (on[s]) cells += face[s / 2];
	return cells;
}

/* outgoing flux of phaser frequency f (its accumulators to the host) */
double c2_flux(int f) { return phaserPoyntingOut(P + f); }

long c2_cells(void) { return (long)W->iNUM * W->jNUM * W->kNUM; }
int c2_nfreq(void) { return nfreqs; }
