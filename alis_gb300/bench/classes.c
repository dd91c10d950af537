/*
 * classes.c -- the half step's cost per class of cells: one E + H pair of
 * 256^3-cell worlds (dx = 2 nm, dt = 1 nm/c) that isolate one class each,
 * timed by the engine's per-kernel events (alisgpu_profile) over a number
 * of steps after 16 warm-up steps.
 *
 *   classes <world> [steps]
 *
 *   0  every cell plain: periodic on all axes, a dielectric box (n = 1.5)
 *      over the middle eighth, one pulsed dipole
 *   1  as 0 with a 12-cell CPML on both z faces (k, the fastest axis)
 *   2  as 0 with the CPML on both x faces (i)
 *   3  as 0 with the CPML on both y faces (j)
 *   4  as 0 with a TFSF plane-wave box [-160, 158]^3 nm instead of the
 *      dipole
 *   5  the dispersive-scatterer benchmark world (c2.c)
 *   6  the large-domain world of c5_build at 512 x 512 x 256 cells with 25
 *      balls (about the same ball density), a 16-frequency phaser box
 *   7  as 6 without the balls (the n = 1.5 host only)
 *
 * Prints the cells, the mean E and H launch times, their sum and the
 * algorithmic bytes per step (c2_step_bytes) over it.
 */
#include "c2.c"
#include <alisgpu.h>

int main(int argc, char **argv)
{
	const int kind = argc > 1 ? atoi(argv[1]) : 0;
	const int steps = argc > 2 ? atoi(argv[2]) : 64;
	if (kind == 5) {
		c2_build(230, 64);
	} else if (kind == 6 || kind == 7) {
		c5_build(512, 512, 256, kind == 6 ? 25 : 0, 16);
	} else {
		const float L = 256;
		dom D = {{-L, L-2}, {-L, L-2}, {-L, L-2}};
		res R = {1, {2}, {1240}};
		sur S0 = {{PBC}, {PBC}, {PBC}};
		sur Sk = {{PBC}, {PBC}, {PML, PML}, {12}};
		sur Si = {{PML, PML}, {PBC}, {PBC}, {12}};
		sur Sj = {{PBC}, {PML, PML}, {PBC}, {12}};
		W = createWorld(D, R, kind == 1 ? Sk : kind == 2 ? Si : kind == 3 ? Sj : S0, "");
		object B = {Box, {{-L/2, L/2}, {-L/2, L/2}, {-L/2, L/2}}};
		putObjects(W, n(1.5), B, Air);
		if (kind == 4) {
			const float T = 160;
			dom DT = {{-T, T-2}, {-T, T-2}, {-T, T-2}};
			planewave(W, DT, Ppol, 0, 0, Pulse, 600, 200);
		} else {
			pointDipole(W, Ez, 0, 0, 0, Pulse, 600, 200);
		}
	}
	for (int q = 0; q < 16; q++) updateE(W), updateH(W);
	alisgpu_synchronize();
	alisgpu_profile(1);
	for (int q = 0; q < steps; q++) updateE(W), updateH(W);
	double tE, tH;
	unsigned long long nE, nH;
	alisgpu_profile_read(0, &tE, &nE);
	alisgpu_profile_read(1, &tH, &nH);
	alisgpu_profile(0);
	const double cells = (double)W->iNUM * W->jNUM * W->kNUM, pair = tE / nE + tH / nH;
	printf("world %d cells %.0f (%d x %d x %d) E %.4f ms H %.4f ms pair %.4f ms bytes/step %.4g -> %.0f GB/s\n",
	       kind, cells, W->iNUM, W->jNUM, W->kNUM, tE / nE, tH / nH, pair, c2_step_bytes(), c2_step_bytes() / pair / 1e6);
	return 0;
}
