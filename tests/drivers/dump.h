/*
 * dump.h -- binary dump of ALiS state for the parity tests.
 *
 * Record format (little endian): char name[64]; int32 kind (0 float32,
 * 1 complex64, 2 float64, 3 complex128); int32 n0, n1, n2; then n0*n1*n2
 * elements.  The same driver source is compiled against the reference
 * library, the oracle, the oracle's FP64 build (float read as double:
 * kinds 2 and 3) and the GPU engine; tests/alis_dump.py reads the files.
 */
#ifndef DUMP_H
#define DUMP_H
#include <stdio.h>
#include <string.h>
#include <stdint.h>

/* The GPU engine exports alisSyncHost; the other builds do not need it. */
extern void alisSyncHost(world W) __attribute__((weak));

static FILE *dumpFile;

#define DUMP_REAL (sizeof(float) == 8 ? 2 : 0)
#define DUMP_COMPLEX (sizeof(float) == 8 ? 3 : 1)

static void dumpOpen(const char *path)
{
	dumpFile = fopen(path, "wb");
	if (!dumpFile) { perror(path); exit(2); }
}

static void dumpHeader(const char *name, int kind, int n0, int n1, int n2)
{
	char nm[64] = {0};
	strncpy(nm, name, 63);
	int32_t h[4] = { kind, n0, n1, n2 };
	fwrite(nm, 1, 64, dumpFile);
	fwrite(h, 4, 4, dumpFile);
}

/* a float*** block with index ranges [i0,i1]x[j0,j1]x[k0,k1] */
static void dumpField(const char *name, float ***f, int i0, int i1, int j0, int j1, int k0, int k1)
{
	if (!f) return;
	dumpHeader(name, DUMP_REAL, 1+i1-i0, 1+j1-j0, 1+k1-k0);
	for (int i = i0; i <= i1; i++) for (int j = j0; j <= j1; j++)
		fwrite(&f[i][j][k0], sizeof(float), 1+k1-k0, dumpFile);
}

static void dumpCField(const char *name, float complex ***f, int i0, int i1, int j0, int j1, int k0, int k1)
{
	if (!f) return;
	dumpHeader(name, DUMP_COMPLEX, 1+i1-i0, 1+j1-j0, 1+k1-k0);
	for (int i = i0; i <= i1; i++) for (int j = j0; j <= j1; j++)
		fwrite(&f[i][j][k0], sizeof(float complex), 1+k1-k0, dumpFile);
}

static void dumpScalar(const char *name, float v)
{
	dumpHeader(name, DUMP_REAL, 1, 1, 1);
	fwrite(&v, sizeof v, 1, dumpFile);
}

static void dumpCScalar(const char *name, float complex v)
{
	dumpHeader(name, DUMP_COMPLEX, 1, 1, 1);
	fwrite(&v, sizeof v, 1, dumpFile);
}

/* material maps, fields, ADE currents of a world */
/* instantaneous Poynting fluxes through planes of W: whole planes, a
 * sub-rectangle and a zero-width strip per axis, and a closed box */
static void dumpPoynting(world W, const char *tag)
{
	char nm[64];
	float lo[3] = { W->xMin, W->yMin, W->zMin }, hi[3] = { W->xMax, W->yMax, W->zMax };
	int sym[3] = { W->xMinSur == SYM, W->yMinSur == SYM, W->zMinSur == SYM };
	float at[3][2], a0[3], a1[3];
	/* a symmetry plane at 0: ranges on the stored half only (the
	 * reference mirrors plane positions, not range ends) */
	for (int a = 0; a < 3; a++) if (sym[a] && lo[a] < 0) lo[a] = 0;
	for (int a = 0; a < 3; a++) {
		at[a][0] = lo[a] + 0.5f * (hi[a] - lo[a]);
		at[a][1] = lo[a] + 0.2f * (hi[a] - lo[a]);
		a0[a] = lo[a] + 0.15f * (hi[a] - lo[a]), a1[a] = hi[a] - 0.3f * (hi[a] - lo[a]);
	}
	for (int p = 0; p < 2; p++) {
		snprintf(nm, 64, "%s.x%d", tag, p); dumpScalar(nm, poyntingX(W, at[0][p]));
		snprintf(nm, 64, "%s.y%d", tag, p); dumpScalar(nm, poyntingY(W, at[1][p]));
		snprintf(nm, 64, "%s.z%d", tag, p); dumpScalar(nm, poyntingZ(W, at[2][p]));
		snprintf(nm, 64, "%s.xs%d", tag, p); dumpScalar(nm, poyntingX(W, at[0][p], a0[1], a1[1], a0[2], a1[2]));
		snprintf(nm, 64, "%s.ys%d", tag, p); dumpScalar(nm, poyntingY(W, at[1][p], a0[0], a1[0], a0[2], a1[2]));
		snprintf(nm, 64, "%s.zs%d", tag, p); dumpScalar(nm, poyntingZ(W, at[2][p], a0[0], a1[0], a0[1], a1[1]));
		snprintf(nm, 64, "%s.zl%d", tag, p); dumpScalar(nm, poyntingZ(W, at[2][p], a0[0], a0[0], a0[1], a1[1]));
	}
	snprintf(nm, 64, "%s.out", tag); dumpScalar(nm, poyntingOut(W, a0[0], a1[0], a0[1], a1[1], a0[2], a1[2]));
	/* point probes (get) of several field functions at a few positions,
	 * including the domain's lower corner (a symmetry plane, if any) */
	field *F[8] = { Ex, Ey, Hz, Sz, EE, UE, ScEx, SoEz };
	const char *fn[8] = { "Ex", "Ey", "Hz", "Sz", "EE", "UE", "ScEx", "SoEz" };
	float px[3] = { at[0][0], at[0][1], lo[0] }, py[3] = { at[1][0], at[1][1], lo[1] }, pz[3] = { at[2][1], at[2][0], lo[2] };
	for (int q = 0; q < 3; q++) for (int f = 0; f < 8; f++) {
		if (f >= 6 && !W->S) continue;
		snprintf(nm, 64, "%s.get.%s.%d", tag, fn[f], q); dumpScalar(nm, get(W, F[f], px[q], py[q], pz[q]));
	}
	/* slice reductions: a z plane through the middle and a sub-box */
	slice S1 = createSlice(W, lo[0], hi[0], lo[1], hi[1], at[2][0], at[2][0]);
	slice S2 = createSlice(W, a0[0], a1[0], a0[1], a1[1], a0[2], a1[2]);
	snprintf(nm, 64, "%s.slice.EE", tag); dumpScalar(nm, sliceSum(W, EE, S1));
	snprintf(nm, 64, "%s.slice.Ex", tag); dumpScalar(nm, sliceMax(W, Ex, S1));
	snprintf(nm, 64, "%s.slice.HH", tag); dumpScalar(nm, sliceSum(W, HH, S2));
	snprintf(nm, 64, "%s.slice.Sz", tag); dumpScalar(nm, sliceMax(W, Sz, S2));
	deleteSlice(S1);
	deleteSlice(S2);
}

static void dumpWorld(world W, const char *tag)
{
	char nm[64];
	if (alisSyncHost) alisSyncHost(W);
	coeffs *C = W->CE;
	if (C->x) {
		snprintf(nm, 64, "%s.CEx", tag); dumpField(nm, C->x, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX, W->kMIN, W->kMAX);
		snprintf(nm, 64, "%s.CEy", tag); dumpField(nm, C->y, W->iMIN, W->iMAX, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX);
		snprintf(nm, 64, "%s.CEz", tag); dumpField(nm, C->z, W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMIN, W->kMAX+1);
	}
	for (int n = 0; n < C->N; n++) {
		int r[6] = { C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n] };
		snprintf(nm, 64, "%s.fill%d.x", tag, n); dumpField(nm, C->Jx[n], r[0], r[1], r[2], r[3], r[4], r[5]);
		snprintf(nm, 64, "%s.fill%d.y", tag, n); dumpField(nm, C->Jy[n], r[0], r[1], r[2], r[3], r[4], r[5]);
		snprintf(nm, 64, "%s.fill%d.z", tag, n); dumpField(nm, C->Jz[n], r[0], r[1], r[2], r[3], r[4], r[5]);
		for (int p = 0; p < C->NK[n]; p++) {
			float c[9] = { C->JJx[n][p], C->JJy[n][p], C->JJz[n][p], C->JEx[n][p], C->JEy[n][p], C->JEz[n][p],
			               C->ax[n], C->ay[n], C->az[n] };
			for (int q = 0; q < 9; q++) { snprintf(nm, 64, "%s.coef%d.%d.%d", tag, n, p, q); dumpScalar(nm, c[q]); }
			if (p >= C->NJ[n]) {
				float d[9] = { C->JKx[n][p], C->KJx[n][p], C->KKx[n][p], C->KEx[n][p], C->JKy[n][p], C->KJy[n][p], C->KKy[n][p], C->KEy[n][p], C->KEz[n][p] };
				for (int q = 0; q < 9; q++) { snprintf(nm, 64, "%s.kcoef%d.%d.%d", tag, n, p, q); dumpScalar(nm, d[q]); }
			}
		}
	}
	for (int m = 0; m <= W->complexField; m++) {
		int a = W->iMIN-1, b = W->iMAX+1, c = W->jMIN-1, d = W->jMAX+1, e = W->kMIN-1, f = W->kMAX+1;
		snprintf(nm, 64, "%s.E%d.x", tag, m); dumpField(nm, W->E[m].x, a, b, c, d, e, f);
		snprintf(nm, 64, "%s.E%d.y", tag, m); dumpField(nm, W->E[m].y, a, b, c, d, e, f);
		snprintf(nm, 64, "%s.E%d.z", tag, m); dumpField(nm, W->E[m].z, a, b, c, d, e, f);
		snprintf(nm, 64, "%s.H%d.x", tag, m); dumpField(nm, W->H[m].x, a, b, c, d, e, f);
		snprintf(nm, 64, "%s.H%d.y", tag, m); dumpField(nm, W->H[m].y, a, b, c, d, e, f);
		snprintf(nm, 64, "%s.H%d.z", tag, m); dumpField(nm, W->H[m].z, a, b, c, d, e, f);
		for (int n = 0; n < C->N; n++) {
			int r[6] = { C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n] };
			for (int p = 0; p < C->NK[n]; p++) {
				snprintf(nm, 64, "%s.J%d.%d.%d.x", tag, m, n, p); dumpField(nm, W->E[m].Jx[n][p], r[0], r[1], r[2], r[3], r[4], r[5]);
				snprintf(nm, 64, "%s.J%d.%d.%d.y", tag, m, n, p); dumpField(nm, W->E[m].Jy[n][p], r[0], r[1], r[2], r[3], r[4], r[5]);
				snprintf(nm, 64, "%s.J%d.%d.%d.z", tag, m, n, p); dumpField(nm, W->E[m].Jz[n][p], r[0], r[1], r[2], r[3], r[4], r[5]);
			}
			for (int p = C->NJ[n]; p < C->NK[n]; p++) {
				snprintf(nm, 64, "%s.K%d.%d.%d.x", tag, m, n, p); dumpField(nm, W->E[m].Kx[n][p], r[0], r[1], r[2], r[3], r[4], r[5]);
				snprintf(nm, 64, "%s.K%d.%d.%d.y", tag, m, n, p); dumpField(nm, W->E[m].Ky[n][p], r[0], r[1], r[2], r[3], r[4], r[5]);
				snprintf(nm, 64, "%s.K%d.%d.%d.z", tag, m, n, p); dumpField(nm, W->E[m].Kz[n][p], r[0], r[1], r[2], r[3], r[4], r[5]);
			}
		}
	}
	snprintf(nm, 64, "%s.t", tag); dumpScalar(nm, W->t);
	if (!strcmp(tag, "W")) dumpPoynting(W, "S");
}

/* accumulated DFT faces of every frequency of a phaser set, plus its flux */
static void dumpPhasers(phaser P, const char *tag)
{
	char nm[64];
	if (alisSyncHost) alisSyncHost(P->W);
	for (int n = 0; P[n].f; n++) {
		phaser p = P + n;
		snprintf(nm, 64, "%s.%d.flux", tag, n); dumpScalar(nm, phaserPoyntingOut(p));
		snprintf(nm, 64, "%s.%d.f", tag, n); dumpScalar(nm, p->f);
		snprintf(nm, 64, "%s.%d.A", tag, n); dumpScalar(nm, p->A);
		cfield *c[6] = { &p->xMin, &p->xMax, &p->yMin, &p->yMax, &p->zMin, &p->zMax };
		int r[6][6] = {
			{ p->iMin, p->iMin, p->jMin, p->jMax, p->kMin, p->kMax }, { p->iMax, p->iMax, p->jMin, p->jMax, p->kMin, p->kMax },
			{ p->iMin, p->iMax, p->jMin, p->jMin, p->kMin, p->kMax }, { p->iMin, p->iMax, p->jMax, p->jMax, p->kMin, p->kMax },
			{ p->iMin, p->iMax, p->jMin, p->jMax, p->kMin, p->kMin }, { p->iMin, p->iMax, p->jMin, p->jMax, p->kMax, p->kMax } };
		const char *fn[6] = { "xMin", "xMax", "yMin", "yMax", "zMin", "zMax" };
		for (int s = 0; s < 6; s++) {
			float complex ***a[6] = { c[s]->Ex, c[s]->Ey, c[s]->Ez, c[s]->Hx, c[s]->Hy, c[s]->Hz };
			const char *cn[6] = { "Ex", "Ey", "Ez", "Hx", "Hy", "Hz" };
			for (int q = 0; q < 6; q++) if (a[q]) {
				snprintf(nm, 64, "%s.%d.%s.%s", tag, n, fn[s], cn[q]);
				dumpCField(nm, a[q], r[s][0], r[s][1], r[s][2], r[s][3], r[s][4], r[s][5]);
			}
		}
	}
}

static void dumpClose(void)
{
	fclose(dumpFile);
}

/* deterministic uniform numbers in [0,1) (64-bit LCG, top 24 bits) */
static unsigned long long lcgState;
static void lcgSeed(unsigned long long s) { lcgState = s * 6364136223846793005ULL + 1442695040888963407ULL; }
static float lcgUniform(void)
{
	lcgState = lcgState * 6364136223846793005ULL + 1442695040888963407ULL;
	return (float)(lcgState >> 40) / 16777216.0f;
}
#endif
