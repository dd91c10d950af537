/*
 * phaser.c -- running-DFT observers on the faces of a box.
 *
 * Host half of the reference src/phaser.c: frequency grids, source
 * normalisation, face geometry and the Poynting flux of the accumulated
 * DFT fields.  The per-step accumulation (updatePhaser) belongs to the
 * backend; on the GPU it is time-blocked (see the device DFT kernel) and
 * the host cfield arrays below are the mirrors that alis_be_sync_phaser
 * refreshes before any host-side reduction.
 */
#include <string.h>
#include "engine.h"

/* planar face arrays: the 4 tangential components of each PML-side face
 * (reference src/phaser.c:12-18, 57-62) */
static void faceArrays(phaser p, cfield *c, int i0, int i1, int j0, int j1, int k0, int k1, int which)
{
	/* which: 0 x-face (Ey, Ez, Hy, Hz), 1 y-face (Ez, Ex, Hz, Hx), 2 z-face (Ex, Ey, Hx, Hy) */
	float complex ****slot[3][4] = {
		{ &c->Ey, &c->Ez, &c->Hy, &c->Hz }, { &c->Ez, &c->Ex, &c->Hz, &c->Hx }, { &c->Ex, &c->Ey, &c->Hx, &c->Hy } };
	for (int q = 0; q < 4; q++) *slot[which][q] = makeComplexField(i0, i1, j0, j1, k0, k1);
	(void)p;
}

/* source whose duration set W->N: first an E or H source of W itself,
 * else one of the first TFSF world (reference src/phaser.c:25-26) */
source alis_reference_source(world W)
{
	source S = W->SE && W->N==W->SE->N ? W->SE : W->SH && W->N==W->SH->N ? W->SH : 0;
	for (world w = W; !S && w->S && w->S->W; S = w->SE && W->N==w->SE->N ? w->SE : w->SH && W->N==w->SH->N ? w->SH : 0)
		w = W->S->W;
	return S;
}

/* Geometry, normalisation and face arrays of phaser p at frequency f
 * (reference src/phaser.c:29-63). */
static void setupPhaser(world W, phaser P, phaser p, source S, float xMin, float xMax, float yMin, float yMax, float zMin, float zMax)
{
	p->W = W;
	p->A = 2.0 / (P->W->N ? P->W->N : P->N);
	p->iMin = MAX(W->iMin, W->xtoi(W, xMin)), p->iMax = MIN(W->iMax, W->xtoi(W, xMax));
	p->jMin = MAX(W->jMin, W->ytoj(W, yMin)), p->jMax = MIN(W->jMax, W->ytoj(W, yMax));
	p->kMin = MAX(W->kMin, W->ztok(W, zMin)), p->kMax = MIN(W->kMax, W->ztok(W, zMax));
	if (S && W->N) {
		/* 1 / |DFT of the source waveform| at f */
		float complex c = 0;
		float complex iwdt = 2 * PI * I * p->f * W->dt;
		for (int n = 1; n < W->N; n++) c += S->waveForm(W, S, W->dt*n, S->phase) * cexpf(iwdt*n);
		p->A = 1 / cabsf(c);
		if (W->sourceType == 2) p->A /= sqrtf(p->f * S->wavelength);
		if (W->sourceType == 3) p->A /= p->f * S->wavelength;
	}
	if ((xMax-xMin < INF && xMin < W->xMin && W->xMax < xMax) && (W->xMaxSur==SYM || W->xMaxSur==PBC || W->xMaxSur==BBC)) {
		p->xNUM = floor((xMax - xMin) / (W->xMax - W->xMin) + 0.5);
		p->expikx = (W->xMaxSur==BBC) ? (W->coskx+I*W->sinkx) : 1;
	}
	if ((yMax-yMin < INF && yMin < W->yMin && W->yMax < yMax) && (W->yMaxSur==SYM || W->yMaxSur==PBC || W->yMaxSur==BBC)) {
		p->yNUM = floor((yMax - yMin) / (W->yMax - W->yMin) + 0.5);
		p->expiky = (W->yMaxSur==BBC) ? (W->cosky+I*W->sinky) : 1;
	}
	if (W->xMinSur==PML && p->iMin != p->iMax) faceArrays(p, &p->xMin, p->iMin, p->iMin, p->jMin, p->jMax, p->kMin, p->kMax, 0);
	if (W->yMinSur==PML && p->jMin != p->jMax) faceArrays(p, &p->yMin, p->iMin, p->iMax, p->jMin, p->jMin, p->kMin, p->kMax, 1);
	if (W->zMinSur==PML && p->kMin != p->kMax) faceArrays(p, &p->zMin, p->iMin, p->iMax, p->jMin, p->jMax, p->kMin, p->kMin, 2);
	if (W->xMaxSur==PML) faceArrays(p, &p->xMax, p->iMax, p->iMax, p->jMin, p->jMax, p->kMin, p->kMax, 0);
	if (W->yMaxSur==PML) faceArrays(p, &p->yMax, p->iMin, p->iMax, p->jMax, p->jMax, p->kMin, p->kMax, 1);
	if (W->zMaxSur==PML) faceArrays(p, &p->zMax, p->iMin, p->iMax, p->jMin, p->jMax, p->kMax, p->kMax, 2);
}

/* Frequencies f_n = (nMax-n)/(dL nMin nMax), n = 0..nMax-nMin: uniform in
 * frequency between 1/LMax and 1/LMin, in decreasing order, closed by an
 * f = 0 sentinel (reference src/phaser.c:21-66).  The grid (its counts,
 * accumulation length and frequencies) is computed in single precision
 * (alis_f32), as the reference computes it. */
phaser (createPhasers)(world W, float LMin, float LMax, float dL, float xMin, float xMax, float yMin, float yMax, float zMin, float zMax, ...)
{
	alis_f32 lo = LMin, hi = LMax, step = dL, dt = W->dt;
	int nMin = floor(lo/step), nMax = ceil(hi/step);
	phaser P;
	source S = alis_reference_source(W);
	MALLOC(P, 0, 2-nMin+nMax);
	for (int n = 0; n <= nMax-nMin; n++) {
		P[n].N = nMin * nMax * step / dt;
		P[n].f = (alis_f32)((nMax-n) / (step * nMin * nMax));
		setupPhaser(W, P, P+n, S, xMin, xMax, yMin, yMax, zMin, zMax);
	}
	alis_be_phaser_created(P);
	return P;
}

phaser (createPhaser)(world W, float L, float xMin, float xMax, float yMin, float yMax, float zMin, float zMax, ...)
{
	return (createPhasers)(W, L, L, L, xMin, xMax, yMin, yMax, zMin, zMax);
}

/* Engine addition: phasers at an explicit wavelength list.  N (the
 * accumulation length) is that of the longest wavelength, as createPhaser
 * would give for it. */
phaser createPhasersList(world W, int count, const float *wavelengths, float xMin, float xMax, float yMin, float yMax, float zMin, float zMax)
{
	phaser P;
	source S = alis_reference_source(W);
	MALLOC(P, 0, count+1);
	alis_f32 Lmax = 0, dt = W->dt;
	for (int n = 0; n < count; n++) Lmax = MAX(Lmax, (alis_f32)wavelengths[n]);
	for (int n = 0; n < count; n++) {
		P[n].N = Lmax / dt;
		P[n].f = (alis_f32)(1 / (alis_f32)wavelengths[n]);
		setupPhaser(W, P, P+n, S, xMin, xMax, yMin, yMax, zMin, zMax);
	}
	alis_be_phaser_created(P);
	return P;
}

/* phaser of the set closest to a wavelength (reference src/phaser.c:75-80) */
phaser choosePhaser(phaser P, float wavelength)
{
	do P++;
	while (1/wavelength < P->f);
	return (1/wavelength - P->f < (P-1)->f - 1/wavelength) ? P : P-1;
}

static void freeFace(phaser P, cfield *c, int i0, int j0, int k0)
{
	if (c->Ex) removeField(c->Ex, i0, j0, k0);
	if (c->Ey) removeField(c->Ey, i0, j0, k0);
	if (c->Ez) removeField(c->Ez, i0, j0, k0);
	if (c->Hx) removeField(c->Hx, i0, j0, k0);
	if (c->Hy) removeField(c->Hy, i0, j0, k0);
	if (c->Hz) removeField(c->Hz, i0, j0, k0);
	(void)P;
}

void deletePhaser(phaser P)
{
	alis_be_phaser_deleted(P);
	phaser Q = P;
	do {
		freeFace(Q, &Q->xMin, Q->iMin, Q->jMin, Q->kMin);
		freeFace(Q, &Q->xMax, Q->iMax, Q->jMin, Q->kMin);
		freeFace(Q, &Q->yMin, Q->iMin, Q->jMin, Q->kMin);
		freeFace(Q, &Q->yMax, Q->iMin, Q->jMax, Q->kMin);
		freeFace(Q, &Q->zMin, Q->iMin, Q->jMin, Q->kMin);
		freeFace(Q, &Q->zMax, Q->iMin, Q->jMin, Q->kMax);
		if (Q->dE) free(&Q->dE[Q->kMIN]);
		if (Q->dH) free(&Q->dH[Q->kMIN]);
		if (Q->ex) free(&Q->ex[Q->kMIN]);
		if (Q->ez) free(&Q->ez[Q->kMIN]);
		Q++;
	} while (Q->f);
	free(P);
}


/* --- Poynting flux of the DFT fields (reference src/phaser.c:142-245) ---
 * 0.5 Re(E x H*) integrated over a face with the trapezoid rule on the
 * E grid and the H-grid spacing across.  Sums are sequential, which is
 * the reference's result with one OpenMP thread. */

static float fluxX(phaser P, cfield S, int i)
{
	float Sum = 0, Part = 0;
	coeffs *E = P->W->CE, *H = P->W->CH;
	if (S.Ey && S.Hz) for (int j = P->jMin+1; j <= P->jMax; j++) {
		float sum = 0;
		sum += 0.5 * E->dz[P->kMin] * S.Ey[i][j][P->kMin] * conjf(S.Hz[i][j][P->kMin]);
		sum += 0.5 * E->dz[P->kMax] * S.Ey[i][j][P->kMax] * conjf(S.Hz[i][j][P->kMax]);
		for (int k = P->kMin+1; k < P->kMax; k++) sum += E->dz[k] * S.Ey[i][j][k] * conjf(S.Hz[i][j][k]);
		Sum += H->dy[j] * sum;
	}
	if (S.Ez && S.Hy) for (int k = P->kMin+1; k <= P->kMax; k++) {
		float sum = 0;
		sum -= 0.5 * E->dy[P->jMin] * S.Ez[i][P->jMin][k] * conjf(S.Hy[i][P->jMin][k]);
		sum -= 0.5 * E->dy[P->jMax] * S.Ez[i][P->jMax][k] * conjf(S.Hy[i][P->jMax][k]);
		for (int j = P->jMin+1; j < P->jMax; j++) sum -= E->dy[j] * S.Ez[i][j][k] * conjf(S.Hy[i][j][k]);
		Part += H->dz[k] * sum;
	}
	Sum += Part;
	return Sum;
}

static float fluxY(phaser P, cfield S, int j)
{
	float Sum = 0, Part = 0;
	coeffs *E = P->W->CE, *H = P->W->CH;
	if (S.Ez && S.Hx) for (int k = P->kMin+1; k <= P->kMax; k++) {
		float sum = 0;
		sum += 0.5 * E->dx[P->iMin] * S.Ez[P->iMin][j][k] * conjf(S.Hx[P->iMin][j][k]);
		sum += 0.5 * E->dx[P->iMax] * S.Ez[P->iMax][j][k] * conjf(S.Hx[P->iMax][j][k]);
		for (int i = P->iMin+1; i < P->iMax; i++) sum += E->dx[i] * S.Ez[i][j][k] * conjf(S.Hx[i][j][k]);
		Sum += H->dz[k] * sum;
	}
	if (S.Ex && S.Hz) for (int i = P->iMin+1; i <= P->iMax; i++) {
		float sum = 0;
		sum -= 0.5 * E->dz[P->kMin] * S.Ex[i][j][P->kMin] * conjf(S.Hz[i][j][P->kMin]);
		sum -= 0.5 * E->dz[P->kMax] * S.Ex[i][j][P->kMax] * conjf(S.Hz[i][j][P->kMax]);
		for (int k = P->kMin+1; k < P->kMax; k++) sum -= E->dz[k] * S.Ex[i][j][k] * conjf(S.Hz[i][j][k]);
		Part += H->dx[i] * sum;
	}
	Sum += Part;
	return Sum;
}

static float fluxZ(phaser P, cfield S, int k)
{
	float Sum = 0, Part = 0;
	coeffs *E = P->W->CE, *H = P->W->CH;
	if (S.Ex && S.Hy) for (int i = P->iMin+1; i <= P->iMax; i++) {
		float sum = 0;
		sum += 0.5 * E->dy[P->jMin] * S.Ex[i][P->jMin][k] * conjf(S.Hy[i][P->jMin][k]);
		sum += 0.5 * E->dy[P->jMax] * S.Ex[i][P->jMax][k] * conjf(S.Hy[i][P->jMax][k]);
		for (int j = P->jMin+1; j < P->jMax; j++) sum += E->dy[j] * S.Ex[i][j][k] * conjf(S.Hy[i][j][k]);
		Sum += H->dx[i] * sum;
	}
	if (S.Ey && S.Hx) for (int j = P->jMin+1; j <= P->jMax; j++) {
		float sum = 0;
		sum -= 0.5 * E->dx[P->iMin] * S.Ey[P->iMin][j][k] * conjf(S.Hx[P->iMin][j][k]);
		sum -= 0.5 * E->dx[P->iMax] * S.Ey[P->iMax][j][k] * conjf(S.Hx[P->iMax][j][k]);
		for (int i = P->iMin+1; i < P->iMax; i++) sum -= E->dx[i] * S.Ey[i][j][k] * conjf(S.Hx[i][j][k]);
		Part += H->dy[j] * sum;
	}
	Sum += Part;
	return Sum;
}

float phaserPoynting(phaser P) { return fabsf(phaserPoyntingOut(P)); }
float phaserPoyntingIn(phaser P) { return -phaserPoyntingOut(P); }

float phaserPoyntingOut(phaser P)
{
	float Sum = 0, face[6];
	world W = P->W;
	if (alis_be_phaser_flux(P, face)) {
		/* the same face values, reduced where the accumulators live */
		Sum += face[1] - face[0];
		Sum += face[3] - face[2];
		Sum += face[5] - face[4];
	} else {
		alis_be_sync_phaser(P);
		Sum += fluxX(P, P->xMax, P->iMax) - fluxX(P, P->xMin, P->iMin);
		Sum += fluxY(P, P->yMax, P->jMax) - fluxY(P, P->yMin, P->jMin);
		Sum += fluxZ(P, P->zMax, P->kMax) - fluxZ(P, P->zMin, P->kMin);
	}
	if (W->Dom.x.Min==W->Dom.x.Max) Sum /= W->CH->dx[P->iMax]+W->CH->dx[P->iMax-1];
	if (W->Dom.y.Min==W->Dom.y.Max) Sum /= W->CH->dy[P->jMax]+W->CH->dy[P->jMax-1];
	if (W->Dom.z.Min==W->Dom.z.Max) Sum /= W->CH->dz[P->kMax]+W->CH->dz[P->kMax-1];
	if (W->xMinSur==SYM) Sum *= 2;
	if (W->yMinSur==SYM) Sum *= 2;
	if (W->zMinSur==SYM) Sum *= 2;
	return Sum * sq(P->A);
}


/* --- spectra to text (reference src/phaser.c:248-295) --- */

void (writePoyntingSpectrum)(world W, char *format, ...)
{
	int M = 0;
	char str[1024], filename[1024];
	va_list ap;
	va_start(ap, format);
	vsprintf(filename, format, ap);
	for (phaser p = va_arg(ap, phaser); p; M++) p = va_arg(ap, phaser);
	va_end(ap);
	phaser *P;
	MALLOC(P, 0, M);
	va_start(ap, format);
	vsprintf(filename, format, ap);
	for (int m = 0; m < M; m++) P[m] = va_arg(ap, phaser);
	va_end(ap);
	for (int n = 0; P[0][n].f; n++) {
		int s = sprintf(str, "%g", 1/P[0][n].f);
		for (int m = 0; m < M; m++) s += sprintf(str+s, "\t%g", phaserPoynting(P[m]+n));
		sprintf(str+s, "\n");
		writeTxt(W, filename, str);
	}
	free(P);
}

void (writeFarFieldSpectrum)(world W, tfield pol(phaser,float,float), float theta, float phi, char *format, ...)
{
	int M = 0;
	char str[1024], filename[1024];
	va_list ap;
	va_start(ap, format);
	vsprintf(filename, format, ap);
	for (phaser p = va_arg(ap, phaser); p; M++) p = va_arg(ap, phaser);
	va_end(ap);
	phaser *P;
	MALLOC(P, 0, M);
	va_start(ap, format);
	vsprintf(filename, format, ap);
	for (int m = 0; m < M; m++) P[m] = va_arg(ap, phaser);
	va_end(ap);
	for (int n = 0; P[0][n].f; n++) {
		int s = sprintf(str, "%g", 1/P[0][n].f);
		for (int m = 0; m < M; m++) s += sprintf(str+s, "\t%g", farFieldI(P[m]+n, pol, theta, phi));
		sprintf(str+s, "\n");
		writeTxt(W, filename, str);
	}
	free(P);
}
