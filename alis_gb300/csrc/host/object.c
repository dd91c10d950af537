/*
 * object.c -- voxelization and material coefficients.
 *
 * Builds, from a list of (matter, object) pairs ending with the background
 * matter, the same arrays as the reference src/object.c:
 *   - CE->x/y/z: inverse permittivity on the three staggered E grids,
 *     updated harmonically object by object in reverse list order;
 *   - per dispersive object n: a bounding box, sub-pixel fill maps
 *     CE->Jx/Jy/Jz[n], ADE recursion coefficients and conductivity factors;
 *   - the J/K current containers of W->E.
 * Everything here is float arithmetic whose rounding must equal the
 * reference, so each helper cites the lines it keeps.
 */
#include <string.h>
#include "engine.h"

void alis_make_currents(world W, vfield *F, coeffs *C, int n);
void alis_alloc_current_tables(world W, vfield *F, int N);
void alis_free_currents(world W, vfield *F, coeffs *C);

typedef struct { int iMin, iMax, jMin, jMax, kMin, kMax; } bounds;


/* --- pole algebra (reference src/object.c:23-67) --- */

static float complex poleGamma(matter M, int p) { return M.P[p].r + I * M.P[p].w; }
static float complex poleSigma(matter M, int p) { return I * (M.P[p].f * M.P[p].w - M.P[p].g * poleGamma(M, p)); }

/* Drude-type recursion J' = JJ J + JE fill E (reference src/object.c:33-41) */
static float drudeJJ(world W, matter M, int p)
{
	return (1 - PI * M.P[p].r * W->dt / W->eV) / (1 + PI * M.P[p].r * W->dt / W->eV);
}

static float drudeJE(world W, matter M, int p)
{
	return sq(2 * PI * M.P[p].w * W->dt / W->eV) / (1 + PI * M.P[p].r * W->dt / W->eV);
}

/* Lorentz / critical-point pair recursion written as one complex
 * recursion (reference src/object.c:43-51) */
static float complex pairA(world W, matter M, int p)
{
	return (1 - PI * poleGamma(M, p) * W->dt / W->eV) / (1 + PI * poleGamma(M, p) * W->dt / W->eV);
}

static float complex pairB(world W, matter M, int p)
{
	return - poleGamma(M, p) * poleSigma(M, p) * sq(2 * PI * W->dt / W->eV) / (1 + PI * poleGamma(M, p) * W->dt / W->eV);
}

/* static conductivity of axis q in units of eV (reference src/object.c:53-62) */
static float conductivity(world W, matter M, int q)
{
	int m = M.e.y || M.e.z ? 1 : 0;
	float s = 0;
	for (int p = 0; p < MAXPOLES; p += 1+2*m) {
		int c = p+q*m;
		if (!M.P[c].w && M.P[c].r) s += M.P[c].r;
		if (M.P[c].g) s += M.P[c].g * M.P[c].w;
	}
	return s / W->eV;
}

/* effective static permittivity of axis q (reference src/object.c:64-67) */
static float staticEps(world W, matter M, int q)
{
	return ((q==2 && M.e.z) ? M.e.z : (q==1 && M.e.y) ? M.e.y : M.e.x) + PI * W->dt * conductivity(W, M, q);
}

/* 2: nonlinear tensor set, 1: has poles or conductivity, 0: plain
 * dielectric (reference src/object.c:282-287) */
int alis_needs_currents(matter M)
{
	for (int i = 0; i < 3; i++) for (int j = 0; j < 6; j++) if (M.d[i][j]) return 2;
	if (M.P[0].w || M.P[0].r) return 1;
	return 0;
}


/* --- sub-pixel fill factors (reference src/object.c:70-121) --- */

/* 1 if the point belongs to object o and to none listed before it */
static float owned(world W, object *O, int o, float i, float j, float k)
{
	float x = W->itox(W, i), y = W->jtoy(W, j), z = W->ktoz(W, k);
	if (!O[o].S(O[o], x, y, z)) return 0;
	while (o--) if (O[o].S(O[o], x, y, z)) return 0;
	return 1;
}

/* Fill factor of the E-grid sample (i, j, k) (one coordinate is half
 * integer).  subN 0/1: point sample; subN < 0: point sample, or 1 when
 * both neighbours across an edge are inside; subN >= 2: subN^3
 * supersampling unless all 8 corners agree with the centre. */
static float fillFactor(world W, object *O, int o, float i, float j, float k)
{
	float n = owned(W, O, o, i, j, k);
	if (W->subN < 2) {
		if (n || W->subN >= 0) return n;
		if (floorf(i) < ceilf(i)) {
			if (owned(W, O, o, i-0.5, j-0.5, k) && owned(W, O, o, i+0.5, j-0.5, k)) return 1;
			if (owned(W, O, o, i-0.5, j+0.5, k) && owned(W, O, o, i+0.5, j+0.5, k)) return 1;
			if (owned(W, O, o, i-0.5, j, k-0.5) && owned(W, O, o, i+0.5, j, k-0.5)) return 1;
			if (owned(W, O, o, i-0.5, j, k+0.5) && owned(W, O, o, i+0.5, j, k+0.5)) return 1;
		} else if (floorf(j) < ceilf(j)) {
			if (owned(W, O, o, i-0.5, j-0.5, k) && owned(W, O, o, i-0.5, j+0.5, k)) return 1;
			if (owned(W, O, o, i+0.5, j-0.5, k) && owned(W, O, o, i+0.5, j+0.5, k)) return 1;
			if (owned(W, O, o, i, j-0.5, k-0.5) && owned(W, O, o, i, j+0.5, k-0.5)) return 1;
			if (owned(W, O, o, i, j-0.5, k+0.5) && owned(W, O, o, i, j+0.5, k+0.5)) return 1;
		} else if (floorf(k) < ceilf(k)) {
			if (owned(W, O, o, i-0.5, j, k-0.5) && owned(W, O, o, i-0.5, j, k+0.5)) return 1;
			if (owned(W, O, o, i+0.5, j, k-0.5) && owned(W, O, o, i+0.5, j, k+0.5)) return 1;
			if (owned(W, O, o, i, j-0.5, k-0.5) && owned(W, O, o, i, j-0.5, k+0.5)) return 1;
			if (owned(W, O, o, i, j+0.5, k-0.5) && owned(W, O, o, i, j+0.5, k+0.5)) return 1;
		}
		return 0;
	}
	float h = (W->subN-1.0) / (W->subN*2.0);
	float c[8];
	int q = 0;
	for (int a = -1; a <= 1; a += 2) for (int b = -1; b <= 1; b += 2) for (int d = -1; d <= 1; d += 2)
		c[q++] = owned(W, O, o, i+a*h, j+b*h, k+d*h);
	int uniform = 1;
	for (q = 0; q < 8; q++) if (c[q] != n) uniform = 0;
	if (uniform) return n;
	float part = 0;
	for (int di = 1-W->subN; di < W->subN; di += 2)
		for (int dj = 1-W->subN; dj < W->subN; dj += 2)
			for (int dk = 1-W->subN; dk < W->subN; dk += 2)
				part += owned(W, O, o, i+0.5*di/W->subN, j+0.5*dj/W->subN, k+0.5*dk/W->subN);
	return part / (W->subN * W->subN * W->subN);
}


/* --- bounding boxes (reference src/object.c:229-279) --- */

/* Index box of the cell centres owned by each object, padded by -1/+2
 * and clamped to the grid.  An object that owns no centre stops the
 * program, as in the reference. */
static bounds *objectBounds(world W, object *O, int N, void *vox)
{
	bounds *B;
	MALLOC(B, 0, N);
	for (int o = 0; o < N; o++) B[o] = (bounds){ W->iMAX, W->iMIN, W->jMAX, W->jMIN, W->kMAX, W->kMIN };
	if (!(vox && alis_be_vox_bounds(vox, N, &B[0].iMin)))
	#pragma omp parallel
	{
		bounds *b;
		MALLOC(b, 0, N);
		for (int o = 0; o < N; o++) b[o] = (bounds){ W->iMAX, W->iMIN, W->jMAX, W->jMIN, W->kMAX, W->kMIN };
		#pragma omp for schedule(guided)
		for (int i = W->iMIN; i <= W->iMAX; i++) for (int j = W->jMIN; j <= W->jMAX; j++) for (int k = W->kMIN; k <= W->kMAX; k++) {
			int o = 0;
			float x = W->itox(W, i), y = W->jtoy(W, j), z = W->ktoz(W, k);
			while (O[o].S && !O[o].S(O[o], x, y, z)) o++;
			if (o < N) {
				b[o].iMin = MIN(i, b[o].iMin), b[o].iMax = MAX(i, b[o].iMax);
				b[o].jMin = MIN(j, b[o].jMin), b[o].jMax = MAX(j, b[o].jMax);
				b[o].kMin = MIN(k, b[o].kMin), b[o].kMax = MAX(k, b[o].kMax);
			}
		}
		#pragma omp critical
		for (int o = 0; o < N; o++) {
			B[o].iMin = MIN(b[o].iMin, B[o].iMin), B[o].iMax = MAX(b[o].iMax, B[o].iMax);
			B[o].jMin = MIN(b[o].jMin, B[o].jMin), B[o].jMax = MAX(b[o].jMax, B[o].jMax);
			B[o].kMin = MIN(b[o].kMin, B[o].kMin), B[o].kMax = MAX(b[o].kMax, B[o].kMax);
		}
		free(b);
	}
	for (int o = 0; o < N; o++) {
		if (B[o].iMin <= B[o].iMax && B[o].jMin <= B[o].jMax && B[o].kMin <= B[o].kMax) {
			B[o].iMin = MAX(B[o].iMin-1, W->iMIN), B[o].iMax = MIN(B[o].iMax+2, W->iMAX);
			B[o].jMin = MAX(B[o].jMin-1, W->jMIN), B[o].jMax = MIN(B[o].jMax+2, W->jMAX);
			B[o].kMin = MAX(B[o].kMin-1, W->kMIN), B[o].kMax = MIN(B[o].kMax+2, W->kMAX);
		} else {
			printf("\rVolume of object %d/%d is zero!\n", o+1, N);
			exit(0);
		}
	}
	return B;
}


/* --- coefficient storage (reference src/object.c:124-226) --- */

static void allocCoeffTables(world W, coeffs *C)
{
	int N = C->N;
	MALLOC(C->NJ, 0, N); MALLOC(C->NK, 0, N);
	MALLOC(C->iMin, 0, N); MALLOC(C->iMax, 0, N);
	MALLOC(C->jMin, 0, N); MALLOC(C->jMax, 0, N);
	MALLOC(C->kMin, 0, N); MALLOC(C->kMax, 0, N);
	MALLOC(C->Jx, 0, N); MALLOC(C->Jy, 0, N); MALLOC(C->Jz, 0, N);
	MALLOC(C->ax, 0, N); MALLOC(C->ay, 0, N); MALLOC(C->az, 0, N);
	MALLOC(C->JJx, 0, N); MALLOC(C->JJy, 0, N); MALLOC(C->JJz, 0, N);
	MALLOC(C->JKx, 0, N); MALLOC(C->JKy, 0, N); MALLOC(C->JKz, 0, N);
	MALLOC(C->JEx, 0, N); MALLOC(C->JEy, 0, N); MALLOC(C->JEz, 0, N);
	MALLOC(C->KJx, 0, N); MALLOC(C->KJy, 0, N); MALLOC(C->KJz, 0, N);
	MALLOC(C->KKx, 0, N); MALLOC(C->KKy, 0, N); MALLOC(C->KKz, 0, N);
	MALLOC(C->KEx, 0, N); MALLOC(C->KEy, 0, N); MALLOC(C->KEz, 0, N);
	(void)W;
}

/* eps^-1 maps filled with the background value (reference src/object.c:168-174) */
static void backgroundMaps(world W, coeffs *C, float Cx, float Cy, float Cz)
{
	C->x = makeField(W->iMIN, W->iMAX+1, W->jMIN, W->jMAX, W->kMIN, W->kMAX);
	C->y = makeField(W->iMIN, W->iMAX, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX);
	C->z = makeField(W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMIN, W->kMAX+1);
	float vx = 1/Cx, vy = 1/Cy, vz = 1/Cz;
	#pragma omp parallel for
	for (int i = W->iMIN; i <= W->iMAX+1; i++) for (int j = W->jMIN; j <= W->jMAX+1; j++) for (int k = W->kMIN; k <= W->kMAX+1; k++) {
		if (j <= W->jMAX && k <= W->kMAX) C->x[i][j][k] = vx;
		if (i <= W->iMAX && k <= W->kMAX) C->y[i][j][k] = vy;
		if (i <= W->iMAX && j <= W->jMAX) C->z[i][j][k] = vz;
	}
}

/* box of dispersive object n (the upper bound grows by one where it
 * touches the grid edge) and its coefficient vectors */
static void dispersiveBox(world W, coeffs *C, int n, bounds B)
{
	C->iMin[n] = B.iMin, C->iMax[n] = B.iMax + (B.iMax == W->iMAX ? 1 : 0);
	C->jMin[n] = B.jMin, C->jMax[n] = B.jMax + (B.jMax == W->jMAX ? 1 : 0);
	C->kMin[n] = B.kMin, C->kMax[n] = B.kMax + (B.kMax == W->kMAX ? 1 : 0);
	int NK = C->NK[n], NJ = C->NJ[n];
	MALLOC(C->JJx[n], 0, NK); MALLOC(C->JJy[n], 0, NK); MALLOC(C->JJz[n], 0, NK);
	MALLOC(C->JKx[n], 0, NK); MALLOC(C->JKy[n], 0, NK); MALLOC(C->JKz[n], 0, NK);
	MALLOC(C->JEx[n], 0, NK); MALLOC(C->JEy[n], 0, NK); MALLOC(C->JEz[n], 0, NK);
	MALLOC(C->KJx[n], NJ, NK-NJ); MALLOC(C->KJy[n], NJ, NK-NJ); MALLOC(C->KJz[n], NJ, NK-NJ);
	MALLOC(C->KKx[n], NJ, NK-NJ); MALLOC(C->KKy[n], NJ, NK-NJ); MALLOC(C->KKz[n], NJ, NK-NJ);
	MALLOC(C->KEx[n], NJ, NK-NJ); MALLOC(C->KEy[n], NJ, NK-NJ); MALLOC(C->KEz[n], NJ, NK-NJ);
	C->Jx[n] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
	C->Jy[n] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
	C->Jz[n] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
	alis_make_currents(W, W->E, C, n);
}

/* fill maps, conductivity factors and pole coefficients of dispersive
 * object n = list entry o; m = 1 for anisotropic matter, whose poles come
 * in x/y/z triples (reference src/object.c:290-336) */
static void dispersiveCoeffs(world W, coeffs *C, matter *M, object *O, int n, int o, int m, void *vox)
{
	int box[6] = { C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n] };
	float *at[3] = { &C->Jx[n][box[0]][box[2]][box[4]], &C->Jy[n][box[0]][box[2]][box[4]], &C->Jz[n][box[0]][box[2]][box[4]] };
	if (!(vox && alis_be_vox_fill(vox, o, box, at[0], at[1], at[2])))
	#pragma omp parallel for schedule(guided)
	for (int i = C->iMin[n]; i <= C->iMax[n]; i++) for (int j = C->jMin[n]; j <= C->jMax[n]; j++) for (int k = C->kMin[n]; k <= C->kMax[n]; k++) {
		C->Jx[n][i][j][k] = fillFactor(W, O, o, i-0.5, j, k);
		C->Jy[n][i][j][k] = fillFactor(W, O, o, i, j-0.5, k);
		C->Jz[n][i][j][k] = fillFactor(W, O, o, i, j, k-0.5);
	}
	matter Mo = M[o];
	C->ax[n] = PI * W->dt * conductivity(W, Mo, 0) / (Mo.e.x ? Mo.e.x : Mo.e.x);
	C->ay[n] = PI * W->dt * conductivity(W, Mo, 1) / (Mo.e.y ? Mo.e.y : Mo.e.x);
	C->az[n] = PI * W->dt * conductivity(W, Mo, 2) / (Mo.e.z ? Mo.e.z : Mo.e.x);

	float *JJ[3] = {0}, *JK[3] = {0}, *JE[3] = {0}, *KJ[3] = {0}, *KK[3] = {0}, *KE[3] = {0};
	float **tJJ[3] = { C->JJx, C->JJy, C->JJz }, **tJK[3] = { C->JKx, C->JKy, C->JKz }, **tJE[3] = { C->JEx, C->JEy, C->JEz };
	float **tKJ[3] = { C->KJx, C->KJy, C->KJz }, **tKK[3] = { C->KKx, C->KKy, C->KKz }, **tKE[3] = { C->KEx, C->KEy, C->KEz };
	for (int a = 0; a < 3; a++) JJ[a] = tJJ[a][n], JK[a] = tJK[a][n], JE[a] = tJE[a][n], KJ[a] = tKJ[a][n], KK[a] = tKK[a][n], KE[a] = tKE[a][n];

	for (int p = 0, j = 0, k = C->NJ[n]; p < MAXPOLES; p += 1+2*m) {
		if (!Mo.P[p].w) continue;
		if (!Mo.P[p].f && !Mo.P[p].g) {
			for (int a = 0; a < 3; a++) {
				JJ[a][j] = drudeJJ(W, Mo, p+a*m);
				JE[a][j] = drudeJE(W, Mo, p+a*m) / staticEps(W, Mo, a);
			}
			j++;
		} else {
			for (int a = 0; a < 3; a++) {
				float complex A = pairA(W, Mo, p+a*m);
				float complex Bc = pairB(W, Mo, p+a*m);
				JJ[a][k] = creal(A);
				JK[a][k] =-cimag(A);
				JE[a][k] = creal(Bc) / staticEps(W, Mo, a);
			}
			for (int a = 0; a < 3; a++) {
				KJ[a][k] =-JK[a][k] / JJ[a][k];
				KK[a][k] = JK[a][k] * JK[a][k] / JJ[a][k] + JJ[a][k];
				KE[a][k] = JE[a][k] * JK[a][k] / JJ[a][k] + cimag(pairB(W, Mo, p+a*m)) / staticEps(W, Mo, a);
			}
			k++;
		}
	}
}


/* --- public entry points (reference src/object.c:339-549) --- */

/* harmonic update C = 1/(1/C + d*fill) over a box plus the far plane of
 * the staggered grid where the box touches the grid edge */
#define HARMONIC(map, i, j, k, d, fill) ((map)[i][j][k] = 1 / (1 / (map)[i][j][k] + (d) * (fill)))

/* the non-dispersive branch of putObjectArray with fill factors from the
 * backend's voxelizer; 0 when the host loops are to do it */
static int harmonicOnDevice(world W, coeffs *C, object *O, void *vox, int o, bounds b, float cx, float cy, float cz)
{
	long NI = 1 + b.iMax - b.iMin, NJ = 1 + b.jMax - b.jMin, NK = 1 + b.kMax - b.kMin;
	float *f = malloc(3 * NI * NJ * NK * sizeof *f);
	if (!f || !alis_be_vox_fill(vox, o, &b.iMin, f, f + NI*NJ*NK, f + 2*NI*NJ*NK)) {
		free(f);
		return 0;
	}
	float *fx = f, *fy = f + NI*NJ*NK, *fz = f + 2*NI*NJ*NK;
	#pragma omp parallel for
	for (int i = b.iMin; i <= b.iMax; i++) for (int j = b.jMin; j <= b.jMax; j++) for (int k = b.kMin; k <= b.kMax; k++) {
		long t = ((i - b.iMin) * NJ + (j - b.jMin)) * NK + (k - b.kMin);
		HARMONIC(C->x, i, j, k, cx, fx[t]);
		HARMONIC(C->y, i, j, k, cy, fy[t]);
		HARMONIC(C->z, i, j, k, cz, fz[t]);
	}
	/* the far plane of the staggered grid where the box touches the edge */
	if (b.iMax == W->iMAX) {
		int dev = alis_be_vox_fill_edge(vox, o, 0, b.iMax, b.jMin, b.jMax, b.kMin, b.kMax, f);
		for (int j = b.jMin; j <= b.jMax; j++) for (int k = b.kMin; k <= b.kMax; k++)
			HARMONIC(C->x, b.iMax+1, j, k, cx, dev ? f[(j - b.jMin) * NK + (k - b.kMin)] : fillFactor(W, O, o, b.iMax+0.5, j, k));
	}
	if (b.jMax == W->jMAX) {
		int dev = alis_be_vox_fill_edge(vox, o, 1, b.jMax, b.iMin, b.iMax, b.kMin, b.kMax, f);
		for (int i = b.iMin; i <= b.iMax; i++) for (int k = b.kMin; k <= b.kMax; k++)
			HARMONIC(C->y, i, b.jMax+1, k, cy, dev ? f[(i - b.iMin) * NK + (k - b.kMin)] : fillFactor(W, O, o, i, b.jMax+0.5, k));
	}
	if (b.kMax == W->kMAX) {
		int dev = alis_be_vox_fill_edge(vox, o, 2, b.kMax, b.iMin, b.iMax, b.jMin, b.jMax, f);
		for (int i = b.iMin; i <= b.iMax; i++) for (int j = b.jMin; j <= b.jMax; j++)
			HARMONIC(C->z, i, j, b.kMax+1, cz, dev ? f[(i - b.iMin) * NJ + (j - b.jMin)] : fillFactor(W, O, o, i, j, b.kMax+0.5));
	}
	free(f);
	return 1;
}

void putObjectArray(world W, matter *M, object *O)
{
	removeObjects(W);
	int N;
	for (N = 0; O[N].S; N++) if (alis_needs_currents(M[N])) W->CE->N++;
	printf("\rPreparing to put %d objects.\n", N);
	W->subN = W->Res.spec.subN = W->Res.spec.subN ? W->Res.spec.subN : W->CE->N ? 1 : 12;
	void *vox = alis_be_vox_begin(W, O, N);
	bounds *B = objectBounds(W, O, N, vox);
	coeffs *C = W->CE;
	alis_alloc_current_tables(W, W->E, C->N);
	allocCoeffTables(W, C);
	backgroundMaps(W, C, staticEps(W, M[N], 0), staticEps(W, M[N], 1), staticEps(W, M[N], 2));
	MALLOC(C->O, 0, N+1);
	MALLOC(C->M, 0, N+1);
	C->M[N] = M[N];

	for (int o = N-1, n = C->N; o >= 0; o--) {
		C->O[o] = O[o];
		C->M[o] = M[o];
		float cx = staticEps(W, M[o], 0) - staticEps(W, M[N], 0);
		float cy = staticEps(W, M[o], 1) - staticEps(W, M[N], 1);
		float cz = staticEps(W, M[o], 2) - staticEps(W, M[N], 2);
		printf("\rPutting objects: %d left.", o+1);
		fflush(stdout);
		bounds b = B[o];

		if (alis_needs_currents(M[o])) {
			n--;
			int m = M[o].e.y || M[o].e.z ? 1 : 0;
			for (int p = 0; p < MAXPOLES; p++) {
				if (M[o].P[p].w && !M[o].P[p].f && !M[o].P[p].g) C->NJ[n]++;
				if (M[o].P[p].w) C->NK[n]++;
			}
			if (m) C->NJ[n] /= 3, C->NK[n] /= 3;
			dispersiveBox(W, C, n, b);
			dispersiveCoeffs(W, C, M, O, n, o, m, vox);
			float ****fx = C->Jx, ****fy = C->Jy, ****fz = C->Jz;
			#pragma omp parallel for schedule(guided)
			for (int i = b.iMin; i <= b.iMax; i++) for (int j = b.jMin; j <= b.jMax; j++) for (int k = b.kMin; k <= b.kMax; k++) {
				HARMONIC(C->x, i, j, k, cx, fx[n][i][j][k]);
				HARMONIC(C->y, i, j, k, cy, fy[n][i][j][k]);
				HARMONIC(C->z, i, j, k, cz, fz[n][i][j][k]);
			}
			if (b.iMax == W->iMAX) for (int j = b.jMin; j <= b.jMax; j++) for (int k = b.kMin; k <= b.kMax; k++)
				HARMONIC(C->x, b.iMax+1, j, k, cx, fx[n][b.iMax+1][j][k]);
			if (b.jMax == W->jMAX) for (int i = b.iMin; i <= b.iMax; i++) for (int k = b.kMin; k <= b.kMax; k++)
				HARMONIC(C->y, i, b.jMax+1, k, cy, fy[n][i][b.jMax+1][k]);
			if (b.kMax == W->kMAX) for (int i = b.iMin; i <= b.iMax; i++) for (int j = b.jMin; j <= b.jMax; j++)
				HARMONIC(C->z, i, j, b.kMax+1, cz, fz[n][i][j][b.kMax+1]);
		} else if (vox && harmonicOnDevice(W, C, O, vox, o, b, cx, cy, cz)) {
		} else {
			#pragma omp parallel for schedule(guided)
			for (int i = b.iMin; i <= b.iMax; i++) for (int j = b.jMin; j <= b.jMax; j++) for (int k = b.kMin; k <= b.kMax; k++) {
				HARMONIC(C->x, i, j, k, cx, fillFactor(W, O, o, i-0.5, j, k));
				HARMONIC(C->y, i, j, k, cy, fillFactor(W, O, o, i, j-0.5, k));
				HARMONIC(C->z, i, j, k, cz, fillFactor(W, O, o, i, j, k-0.5));
			}
			if (b.iMax == W->iMAX) for (int j = b.jMin; j <= b.jMax; j++) for (int k = b.kMin; k <= b.kMax; k++)
				HARMONIC(C->x, b.iMax+1, j, k, cx, fillFactor(W, O, o, b.iMax+0.5, j, k));
			if (b.jMax == W->jMAX) for (int i = b.iMin; i <= b.iMax; i++) for (int k = b.kMin; k <= b.kMax; k++)
				HARMONIC(C->y, i, b.jMax+1, k, cy, fillFactor(W, O, o, i, b.jMax+0.5, k));
			if (b.kMax == W->kMAX) for (int i = b.iMin; i <= b.iMax; i++) for (int j = b.jMin; j <= b.jMax; j++)
				HARMONIC(C->z, i, j, b.kMax+1, cz, fillFactor(W, O, o, i, j, b.kMax+0.5));
		}
	}
	free(B);
	alis_be_vox_end(vox);
	printf("\rPutting objects: %d done.\n", N);
	fflush(stdout);
	alis_be_objects_changed(W);
}

void (putObjects)(world W, ...)
{
	int N = 0;
	va_list ap;
	matter *M;
	object *O;
	va_start(ap, W);
	while (va_arg(ap, matter), va_arg(ap, object).S) N++;
	va_end(ap);
	MALLOC(M, 0, N+1);
	MALLOC(O, 0, N+1);
	va_start(ap, W);
	for (int o = 0; o <= N; o++) {
		M[o] = va_arg(ap, matter);
		O[o] = va_arg(ap, object);
	}
	va_end(ap);
	putObjectArray(W, M, O);
	free(M);
	free(O);
}

static void freeCoeffs(world W, coeffs *C)
{
	for (int n = 0; n < C->N; n++) {
		removeField(C->Jx[n], C->iMin[n], C->jMin[n], C->kMin[n]);
		removeField(C->Jy[n], C->iMin[n], C->jMin[n], C->kMin[n]);
		removeField(C->Jz[n], C->iMin[n], C->jMin[n], C->kMin[n]);
		free(C->JJx[n]); free(C->JKx[n]); free(C->JEx[n]);
		free(C->JJy[n]); free(C->JKy[n]); free(C->JEy[n]);
		free(C->JJz[n]); free(C->JKz[n]); free(C->JEz[n]);
		free(C->KJx[n]+C->NJ[n]); free(C->KKx[n]+C->NJ[n]); free(C->KEx[n]+C->NJ[n]);
		free(C->KJy[n]+C->NJ[n]); free(C->KKy[n]+C->NJ[n]); free(C->KEy[n]+C->NJ[n]);
		free(C->KJz[n]+C->NJ[n]); free(C->KKz[n]+C->NJ[n]); free(C->KEz[n]+C->NJ[n]);
	}
	removeField(C->x, W->iMIN, W->jMIN, W->kMIN);
	removeField(C->y, W->iMIN, W->jMIN, W->kMIN);
	removeField(C->z, W->iMIN, W->jMIN, W->kMIN);
	free(C->NJ); free(C->NK);
	free(C->iMin); free(C->jMax); free(C->iMax); free(C->kMin); free(C->jMin); free(C->kMax);
	free(C->Jx); free(C->ax); free(C->Jy); free(C->ay); free(C->Jz); free(C->az);
	free(C->JJx); free(C->JKx); free(C->JEx); free(C->KJx); free(C->KKx); free(C->KEx);
	free(C->JJy); free(C->JKy); free(C->JEy); free(C->KJy); free(C->KKy); free(C->KEy);
	free(C->JJz); free(C->JKz); free(C->JEz); free(C->KJz); free(C->KKz); free(C->KEz);
	free(C->O); free(C->M);
	C->O = 0; C->M = 0; C->N = 0;
	C->NJ = C->NK = C->iMin = C->iMax = C->jMin = C->jMax = C->kMin = C->kMax = 0;
	C->Jx = C->Jy = C->Jz = 0;
}

void removeObjects(world W)
{
	if (W->CE->O && W->CE->M) {
		alis_free_currents(W, W->E, W->CE);
		freeCoeffs(W, W->CE);
		alis_be_objects_changed(W);
	}
}

/* scale the damping of every pole (reference src/object.c:500-507) */
matter LT(matter M, float T)
{
	for (int i = 0; i < MAXPOLES; i++) {
		M.P[i].r *= T;
		M.P[i].g *= T;
	}
	return M;
}

/* (n, k) table lookup with linear interpolation in wavelength, returning
 * the same conductive dielectric as the nk() macro (reference
 * src/object.c:510-549).  Columns may be separated by tab, space or comma. */
matter nkFile(char *name, float l, float f)
{
	FILE *file = fopen(name, "r");
	if (!file) {
		printf("The (n,k) file not found.\n");
		exit(0);
	}
	int N = 0, cap = 0;
	char line[1024];
	float *L = 0, *Nn = 0, *Kk = 0, n = 0, k = 0;
	while (fgets(line, 256, file)) {
		if (N >= cap) {
			cap += 256;
			L = realloc(L, cap*sizeof(float));
			Nn = realloc(Nn, cap*sizeof(float));
			Kk = realloc(Kk, cap*sizeof(float));
		}
		char *s = line;
		L[N] = atof(s);
		s = strchr(s,'\t') ? strchr(s,'\t')+1 : strchr(s,' ') ? strchr(s,' ')+1 : strchr(s,',')+1;
		Nn[N] = atof(s);
		s = strchr(s,'\t') ? strchr(s,'\t')+1 : strchr(s,' ') ? strchr(s,' ')+1 : strchr(s,',')+1;
		Kk[N] = atof(s);
		N++;
	}
	fclose(file);
	int i = 1;
	while (i < N-1 && l > L[i]) i++;
	n = (Nn[i-1]*(L[i]-l) + Nn[i]*(l-L[i-1])) / (L[i]-L[i-1]);
	k = (Kk[i-1]*(L[i]-l) + Kk[i]*(l-L[i-1])) / (L[i]-L[i-1]);
	free(L); free(Nn); free(Kk);
	return (matter) {{(n)*(n)-(k)*(k)},{{0,2*n*k*((float)f)}}};
}
