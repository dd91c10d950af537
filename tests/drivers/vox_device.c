/*
 * vox_device.c -- one object list put into a world, linked against the
 * engine (the device voxelizer) or against the oracle (the host loops of
 * the same host layer), for the device voxelizer against those loops.
 * Prints the engine's kernel launches during putObjectArray (0 in the
 * oracle build), its wall time and an FNV-1a hash of the eps^-1 maps and
 * of the dispersive objects' fill maps.
 *
 *   vox_device <half size in nm> <subN> [contour]
 *
 * With "contour" the list also holds a height-map object, which the
 * device does not evaluate: the whole list stays with the host loops.
 */
#include <alis.h>
#include <stdint.h>
#include <time.h>

/* the engine's launch counter; absent from the oracle build */
unsigned long long alisgpu_launch_count(void) __attribute__((weak));
static unsigned long long launches(void) { return alisgpu_launch_count ? alisgpu_launch_count() : 0; }

static unsigned long long rng;
static float uniform(void)
{
	rng = rng * 6364136223846793005ULL + 1442695040888963407ULL;
	return (float)(rng >> 40) / 16777216.0f;
}

static uint64_t fnv(uint64_t h, const void *p, size_t n)
{
	const unsigned char *c = p;
	for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ULL;
	return h;
}

static uint64_t hashBox(uint64_t h, float ***F, int i0, int i1, int j0, int j1, int k0, int k1)
{
	for (int i = i0; i <= i1; i++) for (int j = j0; j <= j1; j++) h = fnv(h, &F[i][j][k0], (size_t)(1 + k1 - k0) * sizeof(float));
	return h;
}

static float map[32][32], *rows[32];

int main(int argc, char **argv)
{
	float L = argc > 1 ? atof(argv[1]) : 400;
	int subN = argc > 2 ? atoi(argv[2]) : 8;
	int contour = argc > 3 && !strcmp(argv[3], "contour");
	dom D = {{-L, L}, {-L, L}, {-L, L}};
	res R = {5, {10}, {1240, subN}};
	sur S = {{PML}, {PML}, {PML}, {8}};
	world W = createWorld(D, R, S, "");

	enum { NB = 40, NO = NB + 6 };
	object O[NO + 1];
	matter M[NO + 1];
	rng = 12345;
	for (int q = 0; q < NB; q++) {
		float r = 0.05f * L + 0.1f * L * uniform();
		float x = -0.7f * L + 1.4f * L * uniform(), y = -0.7f * L + 1.4f * L * uniform(), z = -0.7f * L + 1.4f * L * uniform();
		O[q] = (object){q % 3 ? Ball : RodZ, {{x - r, x + r}, {y - r, y + r}, {z - r, z + r}}};
		M[q] = q % 7 ? n(1.2f + 0.05f * q) : (matter){{2.0}, {{8.0, 0.05}}};
	}
	float s = 0.1f * L;
	O[NB + 0] = (object){Rotation, {{30, 20, 45}, {0, 0, 0}}, objects {{Box, {{-2*s, 2*s}, {-s, s}, {-s, s}}}}};
	O[NB + 1] = (object){Lattice, {{s, 5}, {s, 5}, {0}}, objects {{Ball, {{-0.3f*s, 0.3f*s}, {-0.3f*s, 0.3f*s}, {-0.8f*L, -0.6f*L}}}}};
	O[NB + 2] = (object){CLatticeZ, {{7}, {0, 0}}, objects {{RodZ, {{2*s, 3*s}, {-0.4f*s, 0.4f*s}, {0.5f*L, 0.8f*L}}}}};
	O[NB + 3] = (object){Difference, {{2}}, objects {
		{Box, {{-0.8f*L, -0.4f*L}, {0.4f*L, 0.8f*L}, {-0.2f*L, 0.2f*L}}},
		{Ball, {{-0.7f*L, -0.5f*L}, {0.5f*L, 0.7f*L}, {-0.3f*L, 0.3f*L}}}}};
	for (int i = 0; i < 32; i++) {
		rows[i] = map[i];
		for (int j = 0; j < 32; j++) map[i][j] = (i - 15.5f) * (i - 15.5f) + (j - 15.5f) * (j - 15.5f);
	}
	O[NB + 4] = contour ? (object){Intersection, {{2}}, objects {
		{Box, {{-INF, INF}, {-INF, INF}, {-0.9f*L, -0.85f*L}}},
		{ImportContour, {{-0.5f*L, 0.5f*L, 32}, {-0.5f*L, 0.5f*L, 32}, {0, 200}}, rows}}}
		: (object){Box, {{-0.5f*L, 0.5f*L}, {-0.5f*L, 0.5f*L}, {-0.9f*L, -0.85f*L}}};
	O[NB + 5] = (object){Box, {{-INF, INF}, {-INF, INF}, {-INF, -0.9f*L}}};
	for (int o = NB; o < NO; o++) M[o] = n(1.5f + 0.1f * (o - NB));
	M[NB + 1] = (matter){{2.5}, {{4.0, 0.1, 0.8}}};
	O[NO] = (object){0};
	M[NO] = Air;

	unsigned long long l0 = launches();
	struct timespec t0, t1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	putObjectArray(W, M, O);
	clock_gettime(CLOCK_MONOTONIC, &t1);
	unsigned long long l1 = launches();

	coeffs *C = W->CE;
	uint64_t h = 1469598103934665603ULL;
	h = hashBox(h, C->x, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX, W->kMIN, W->kMAX);
	h = hashBox(h, C->y, W->iMIN, W->iMAX, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX);
	h = hashBox(h, C->z, W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMIN, W->kMAX+1);
	for (int n = 0; n < C->N; n++) {
		h = hashBox(h, C->Jx[n], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
		h = hashBox(h, C->Jy[n], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
		h = hashBox(h, C->Jz[n], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
	}
	long cells = (long)(1 + W->iMAX - W->iMIN) * (1 + W->jMAX - W->jMIN) * (1 + W->kMAX - W->kMIN);
	printf("cells %ld\n", cells);
	printf("dispersive %d\n", C->N);
	printf("launches %llu\n", l1 - l0);
	printf("seconds %.6f\n", (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
	printf("hash %016llx\n", (unsigned long long)h);
	deleteWorld(W);
	return 0;
}
