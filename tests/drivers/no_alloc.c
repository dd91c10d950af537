/*
 * no_alloc.c -- alisgpu_farfield_sums_static against alisgpu_farfield_sums
 * through the device C ABI.
 *
 * A 24^3 world with seeded fields, a 6-face phaser box [4, 19]^3 with 3
 * frequencies and a ring of 4 steps, 6 recorded steps with seeded phase
 * factors; then two calls in a row of each entry point on the same batch
 * of 5 directions (seeded test fields and line tables).  Prints the
 * largest difference relative to the largest sum, checks that a batch too
 * large for the static array is refused with ALISGPU_ERANGE, and exits 0
 * when the results agree within 1e-12.
 *
 * With the argument "errors" it checks the error paths of both entry
 * points instead, each without a launch: an injected allocation failure
 * (ALISGPU_ENOMEM), a frequency outside the phaser's and test fields
 * shorter than the phaser box (ALISGPU_EINVAL); and that a call after
 * them still gives the same sums.  Then the storage form's refusals:
 * after a write, a bad kind, complex fields, an upload to a half world.
 */
#include <alisgpu.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static unsigned long long rng = 0x9e3779b97f4a7c15ULL;
static double uni(void)                     /* [-1, 1) */
{
	rng = rng * 6364136223846793005ULL + 1442695040888963407ULL;
	return (double)(rng >> 11) / 4503599627370496.0 - 1.0;
}

#define CHECK(call) do { int rc_ = (call); if (rc_) { fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, alisgpu_last_error()); return 2; } } while (0)

int main(int argc, char **argv)
{
	const int errors = argc > 1 && !strcmp(argv[1], "errors");
	CHECK(alisgpu_init());
	const int N = 24, L = 4, U = 19, NF = 3, NA = 5;
	alisgpu_geometry geo = { 0, N-1, 0, N-1, 0, N-1, 0, N-1, 0, N-1, 0, N-1, 0, {0, 0, 0, 0, 0, 0} };
	alisgpu_world *w;
	CHECK(alisgpu_world_create(&geo, &w));
	const size_t n3 = (size_t)(N+2) * (N+2) * (N+2);
	float *host = malloc(n3 * sizeof(float));
	alisgpu_face faces[6] = {
		{0, L, L, L, U, L, U}, {0, U, U, L, U, L, U},
		{1, L, U, L, L, L, U}, {1, L, U, U, U, L, U},
		{2, L, U, L, U, L, L}, {2, L, U, L, U, U, U},
	};
	alisgpu_phaser *p;
	CHECK(alisgpu_phaser_create(w, NF, 6, faces, 4, 0, &p));
	float phE[2*NF], phH[2*NF];
	for (int step = 0; step < 6; step++) {
		for (int fld = 0; fld < 2; fld++) for (int c = 0; c < 3; c++) {
			for (size_t q = 0; q < n3; q++) host[q] = (float)uni();
			CHECK(alisgpu_field_upload(w, fld, 0, c, host));
		}
		for (int f = 0; f < NF; f++) {
			double a = 3.0 * uni(), b = 3.0 * uni();
			phE[2*f] = (float)cos(a), phE[2*f+1] = (float)sin(a);
			phH[2*f] = (float)cos(b), phH[2*f+1] = (float)sin(b);
		}
		CHECK(alisgpu_phaser_record(p, phE, phH));
	}
	CHECK(alisgpu_phaser_flush(p));

	/* line tables and test fields in the layout the host layer builds */
	alisgpu_farfield_geom g = { 0 };
	g.iMin = L, g.iMax = U, g.jMin = L, g.jMax = U, g.kMin = L, g.kMax = U, g.kMIN = 0;
	for (int q = 0; q < 6; q++) g.faceOn[q] = 1;
	g.cosk[0] = g.cosk[1] = g.cosk[2] = 1;
	g.xLen = 1 + U - L, g.yLen = 1 + U - L, g.zLen = 2 + U - 0;
	double *tab = malloc(sizeof(double) * (4*g.xLen + 4*g.yLen + 2*g.zLen));
	double *t = tab;
	g.xE = t, t += g.xLen; g.xH = t, t += g.xLen; g.dxE = t, t += g.xLen; g.dxH = t, t += g.xLen;
	g.yE = t, t += g.yLen; g.yH = t, t += g.yLen; g.dyE = t, t += g.yLen; g.dyH = t, t += g.yLen;
	g.dzE = t, t += g.zLen; g.dzH = t, t += g.zLen;
	for (int q = 0; q < g.xLen; q++) {
		((double *)g.xE)[q] = 2.0 * (L + q), ((double *)g.xH)[q] = 2.0 * (L + q) - 1.0;
		((double *)g.dxE)[q] = 2.0 + 0.01 * uni(), ((double *)g.dxH)[q] = 2.0 + 0.01 * uni();
	}
	for (int q = 0; q < g.yLen; q++) {
		((double *)g.yE)[q] = 2.0 * (L + q), ((double *)g.yH)[q] = 2.0 * (L + q) - 1.0;
		((double *)g.dyE)[q] = 2.0 + 0.01 * uni(), ((double *)g.dyH)[q] = 2.0 + 0.01 * uni();
	}
	for (int q = 0; q < g.zLen; q++) ((double *)g.dzE)[q] = 2.0 + 0.01 * uni(), ((double *)g.dzH)[q] = 2.0 + 0.01 * uni();
	const int nk = g.zLen;
	double *T = malloc(sizeof(double) * NA * 6 * nk * 2);
	unsigned char pr[NA * 6];
	double kx[NA], ky[NA];
	for (int q = 0; q < NA * 6 * nk * 2; q++) T[q] = uni();
	for (int q = 0; q < NA * 6; q++) pr[q] = 1;
	for (int a = 0; a < NA; a++) kx[a] = 0.02 * uni(), ky[a] = 0.02 * uni();

	if (errors) {
		double a[NA * 12], b[NA * 12];
		CHECK(alisgpu_farfield_sums(p, 1, &g, NA, T, nk, pr, kx, ky, a));
		unsigned long long before = alisgpu_launch_count();
		alisgpu_inject_alloc_failures(3);
		int oom = alisgpu_farfield_sums(p, 1, &g, NA, T, nk, pr, kx, ky, b);
		alisgpu_inject_alloc_failures(0);
		int badF = alisgpu_farfield_sums(p, NF, &g, NA, T, nk, pr, kx, ky, b);
		int badFs = alisgpu_farfield_sums_static(p, -1, &g, NA, T, nk, pr, kx, ky, b);
		int shortT = alisgpu_farfield_sums(p, 1, &g, NA, T, nk - 3, pr, kx, ky, b);
		int shortTs = alisgpu_farfield_sums_static(p, 1, &g, NA, T, nk - 3, pr, kx, ky, b);
		int launched = alisgpu_launch_count() != before;
		CHECK(alisgpu_farfield_sums(p, 1, &g, NA, T, nk, pr, kx, ky, b));
		int same = !memcmp(a, b, sizeof a);
		printf("enomem %d einval_f %d %d einval_nk %d %d launched %d same_after %d\n",
		       oom == ALISGPU_ENOMEM, badF == ALISGPU_EINVAL, badFs == ALISGPU_EINVAL,
		       shortT == ALISGPU_EINVAL, shortTs == ALISGPU_EINVAL, launched, same);
		/* the storage form: only before a world's first step or write,
		 * real fields only; a half world refuses uploads, and switching
		 * back and forth before a step is allowed */
		int written = alisgpu_world_set_storage(w, ALISGPU_STORAGE_HALF);
		int badKind = alisgpu_world_set_storage(w, 7);
		alisgpu_geometry cg = geo;
		cg.complexField = 1;
		alisgpu_world *wc, *wh;
		CHECK(alisgpu_world_create(&cg, &wc));
		int cplx = alisgpu_world_set_storage(wc, ALISGPU_STORAGE_HALF);
		CHECK(alisgpu_world_create(&geo, &wh));
		size_t b0 = alisgpu_world_bytes(wh);
		int toHalf = alisgpu_world_set_storage(wh, ALISGPU_STORAGE_HALF);
		size_t b1 = alisgpu_world_bytes(wh);
		int upload = alisgpu_field_upload(wh, 0, 0, 1, host);
		int down = alisgpu_field_download(wh, 1, 0, 2, host);
		int zero = 1;
		for (size_t q = 0; q < n3; q++) zero &= host[q] == 0.0f;
		int back = alisgpu_world_set_storage(wh, ALISGPU_STORAGE_FLOAT);
		size_t b2 = alisgpu_world_bytes(wh);
		int again = alisgpu_world_set_storage(wh, ALISGPU_STORAGE_HALF);
		int storageOk = written == ALISGPU_EINVAL && badKind == ALISGPU_EINVAL && cplx == ALISGPU_ENOTSUP && toHalf == 0 &&
		                b1 < b0 && upload == ALISGPU_ENOTSUP && down == 0 && zero && back == 0 && b2 == b0 && again == 0;
		printf("storage %d (written %d kind %d complex %d half %d bytes %zu -> %zu -> %zu upload %d download %d zero %d back %d again %d)\n",
		       storageOk, written, badKind, cplx, toHalf, b0, b1, b2, upload, down, zero, back, again);
		alisgpu_world_destroy(wc);
		alisgpu_world_destroy(wh);
		alisgpu_phaser_destroy(p);
		alisgpu_world_destroy(w);
		return oom == ALISGPU_ENOMEM && badF == ALISGPU_EINVAL && badFs == ALISGPU_EINVAL && shortT == ALISGPU_EINVAL &&
		       shortTs == ALISGPU_EINVAL && !launched && same && storageOk ? 0 : 1;
	}

	double ref[2][NA * 12], got[2][NA * 12];
	for (int rep = 0; rep < 2; rep++) {
		for (int f = 0; f < NF; f++) {
			CHECK(alisgpu_farfield_sums(p, f, &g, NA, T, nk, pr, kx, ky, ref[rep]));
			CHECK(alisgpu_farfield_sums_static(p, f, &g, NA, T, nk, pr, kx, ky, got[rep]));
		}
	}
	double top = 0, diff = 0;
	for (int rep = 0; rep < 2; rep++) for (int q = 0; q < NA * 12; q++) {
		top = fmax(top, fabs(ref[rep][q]));
		diff = fmax(diff, fabs(ref[rep][q] - got[rep][q]));
	}
	/* a batch larger than the static array is refused, nothing launched */
	int big = (int)(ALISGPU_FF_STATIC_BYTES / (6.0 * nk * 16)) + 16;
	double *Tbig = calloc((size_t)big * 6 * nk * 2, sizeof(double));
	unsigned char *prBig = calloc((size_t)big * 6, 1);
	double *kBig = calloc(big, sizeof(double)), *outBig = calloc((size_t)big * 12, sizeof(double));
	unsigned long long before = alisgpu_launch_count();
	int rc = alisgpu_farfield_sums_static(p, NF - 1, &g, big, Tbig, nk, prBig, kBig, kBig, outBig);
	int refused = rc == ALISGPU_ERANGE && alisgpu_launch_count() == before;
	printf("max_abs_diff %.3e max_abs %.3e rel %.3e refused_oversize %d (%s)\n", diff, top, top > 0 ? diff / top : 0.0,
	       refused, alisgpu_last_error());
	alisgpu_phaser_destroy(p);
	alisgpu_world_destroy(w);
	return (top > 0 && diff <= 1e-12 * top && refused) ? 0 : 1;
}
