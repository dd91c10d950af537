/*
 * c5_balls.h -- the balls of the large-domain precision workload: `count`
 * seeded Drude-Lorentz balls of radius 20-80 cells (dx nm per cell) with
 * centres uniform in the box [lo, hi] (nm, per axis), so that each lies
 * wholly inside it.  The draws come from a 64-bit LCG seeded with `seed`,
 * one draw per statement in a fixed order.  A ball that would meet an
 * earlier one is drawn again (at most 10000 times): ALiS stops on an
 * object that earlier objects of the list cover wholly.  The bench world
 * (c5_build) and the parity scene's sub-runs (tests/drivers/scenes.c)
 * both take their balls from here.
 */
#ifndef ALIS_C5_BALLS_H
#define ALIS_C5_BALLS_H

/* single precision in every build: the FP64 build of the test drivers
 * reads `float` as `double` but keeps alis_f32, so both draw the same balls */
#ifdef ALIS_FP64
typedef alis_f32 c5Real;
#else
typedef float c5Real;
#endif

typedef struct { c5Real x, y, z, r, e, wp, g, w0, f0; } c5Ball;

static unsigned long long c5State;
static c5Real c5Uniform(void)
{
	c5State = c5State * 6364136223846793005ULL + 1442695040888963407ULL;
	return (c5Real)(c5State >> 40) / (c5Real)16777216;
}

static void c5Balls(unsigned long long seed, int count, const c5Real lo[3], const c5Real hi[3], c5Real dx, c5Ball *out)
{
	c5State = seed * 6364136223846793005ULL + 1442695040888963407ULL;
	for (int q = 0; q < count; q++) {
		c5Ball b;
		for (int tries = 0;; tries++) {
			b.r = dx * (20 + 60 * c5Uniform());
			b.x = lo[0] + b.r + (hi[0] - lo[0] - 2 * b.r) * c5Uniform();
			b.y = lo[1] + b.r + (hi[1] - lo[1] - 2 * b.r) * c5Uniform();
			b.z = lo[2] + b.r + (hi[2] - lo[2] - 2 * b.r) * c5Uniform();
			int meets = 0;
			for (int p = 0; p < q && !meets; p++) {
				c5Real u = b.x - out[p].x, v = b.y - out[p].y, w = b.z - out[p].z, s = b.r + out[p].r;
				meets = u * u + v * v + w * w < s * s;
			}
			if (!meets || tries == 10000) break;
		}
		b.e = 1.5 + c5Uniform(), b.wp = 5 + 4 * c5Uniform(), b.g = 0.05 + 0.2 * c5Uniform();
		b.w0 = 3 + c5Uniform(), b.f0 = 0.5 + c5Uniform();
		out[q] = b;
	}
}

/* the domain [lo, hi] (nm, per axis) of a world whose interior is n[a]
 * cells of dx nm, centred as createWorld lays cells out */
static void c5Domain(const int n[3], c5Real dx, c5Real lo[3], c5Real hi[3])
{
	for (int a = 0; a < 3; a++) lo[a] = -(n[a] / 2) * dx, hi[a] = (n[a] - n[a] / 2 - 1) * dx;
}

#endif
