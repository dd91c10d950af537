/*
 * cpu_step.c -- ORACLE (test infrastructure only).
 *
 * A CPU restatement of the ALiS time-stepping hot path, used by tests/,
 * smoke() and bench.py's CPU-baseline leg as the checker of the GPU
 * engine.  It is linked with the engine's host setup layer (world,
 * objects, sources, phasers: alis_gb300/csrc/host) in place of the GPU
 * backend, and steps the host arrays directly:
 *   updateE / updateH      reference src/update.c:48-341
 *   updatePhaser           reference src/phaser.c:83-110
 *   far-field face sums    reference src/farfld.c:248-459, 488-493
 * Floating-point operation order follows the reference line by line, so
 * that with FMA contraction disabled (-ffp-contract=off) the results are
 * bit-identical to the reference build.  The restatement is pinned by
 * tests/test_oracle_pin.py against outputs of the reference itself built
 * from its sources (oracle/build_ref.sh) and committed as golden
 * fixtures under tests/golden/.
 *
 * Never linked into the product library.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "engine.h"

#define LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) \
_Pragma("omp parallel for") for (int i=i0; i<=i1; i++) for (int j=j0; j<=j1; j++) for (int k=k0; k<=k1; k++)


/* --- CPML psi slabs (reference src/update.c:48-84) ---
 * psi = b psi + c (G - G[+Alt along the slab axis]); F += psi (* C). */

static void psiX(vfield F, vfield G, coeffs *C, float ***Py, float ***Pz, int Alt, int i0, int i1, int j0, int j1, int k0, int k1)
{
	int mat = C->y && C->z;
	LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) {
		Py[i][j][k] = C->xP[i] * Py[i][j][k] + C->xPy[i] * (G.z[i][j][k] - G.z[i+Alt][j][k]);
		Pz[i][j][k] = C->xP[i] * Pz[i][j][k] + C->xPz[i] * (G.y[i][j][k] - G.y[i+Alt][j][k]);
		if (mat) F.y[i][j][k] += Py[i][j][k] * C->y[i][j][k], F.z[i][j][k] += Pz[i][j][k] * C->z[i][j][k];
		else F.y[i][j][k] += Py[i][j][k], F.z[i][j][k] += Pz[i][j][k];
	}
}

static void psiY(vfield F, vfield G, coeffs *C, float ***Pz, float ***Px, int Alt, int i0, int i1, int j0, int j1, int k0, int k1)
{
	int mat = C->z && C->x;
	LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) {
		Pz[i][j][k] = C->yP[j] * Pz[i][j][k] + C->yPz[j] * (G.x[i][j][k] - G.x[i][j+Alt][k]);
		Px[i][j][k] = C->yP[j] * Px[i][j][k] + C->yPx[j] * (G.z[i][j][k] - G.z[i][j+Alt][k]);
		if (mat) F.z[i][j][k] += Pz[i][j][k] * C->z[i][j][k], F.x[i][j][k] += Px[i][j][k] * C->x[i][j][k];
		else F.z[i][j][k] += Pz[i][j][k], F.x[i][j][k] += Px[i][j][k];
	}
}

static void psiZ(vfield F, vfield G, coeffs *C, float ***Px, float ***Py, int Alt, int i0, int i1, int j0, int j1, int k0, int k1)
{
	int mat = C->x && C->y;
	LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) {
		Px[i][j][k] = C->zP[k] * Px[i][j][k] + C->zPx[k] * (G.y[i][j][k] - G.y[i][j][k+Alt]);
		Py[i][j][k] = C->zP[k] * Py[i][j][k] + C->zPy[k] * (G.x[i][j][k] - G.x[i][j][k+Alt]);
		if (mat) F.x[i][j][k] += Px[i][j][k] * C->x[i][j][k], F.y[i][j][k] += Py[i][j][k] * C->y[i][j][k];
		else F.x[i][j][k] += Px[i][j][k], F.y[i][j][k] += Py[i][j][k];
	}
}


/* --- curl half step with conduction, ADE currents and CPML
 * (reference src/update.c:87-125); Alt = +1 for E, -1 for H --- */

/* Conduction factor q = (1 - a u) / (1 + a u) of a cell with fill u.
 * The reference multiplies F by q, rounded to float, at every step: that
 * rounding is the same each step, so over n steps the field of a
 * conducting object drifts by n times it (2.85e-4 of the flux after 4000
 * steps of the benchmark's gold block).  With
 * ALIS_ORACLE_PRECISE_CONDUCTION=1 (the engine's
 * ALISGPU_PRECISE_CONDUCTION=1) F loses F b instead, b = 2 a u / (1 + a u)
 * = 1 - q: b's rounding moves the applied factor by b times as much.  Not
 * the reference's arithmetic: an opt-in precision mode. */
static int preciseConduction = -1;

static void curlStep(world W, vfield F, vfield G, coeffs *C, int Alt)
{
	int i0 = W->iMIN, i1 = W->iMAX, j0 = W->jMIN, j1 = W->jMAX, k0 = W->kMIN, k1 = W->kMAX;
	if (preciseConduction < 0) {
		const char *e = getenv("ALIS_ORACLE_PRECISE_CONDUCTION");
		preciseConduction = e && e[0] == '1';
	}
	for (int n = 0; n < C->N; n++) {
		int a0 = MAX(i0, C->iMin[n]), a1 = MIN(i1, C->iMax[n]);
		int b0 = MAX(j0, C->jMin[n]), b1 = MIN(j1, C->jMax[n]);
		int c0 = MAX(k0, C->kMin[n]), c1 = MIN(k1, C->kMax[n]);
		if (!(C->ax[n] || C->ay[n] || C->az[n])) continue;
		if (preciseConduction) LOOP3(i,a0,a1,j,b0,b1,k,c0,c1) {
			float px = C->ax[n] * C->Jx[n][i][j][k], py = C->ay[n] * C->Jy[n][i][j][k], pz = C->az[n] * C->Jz[n][i][j][k];
			F.x[i][j][k] -= F.x[i][j][k] * (2 * px / (1 + px));
			F.y[i][j][k] -= F.y[i][j][k] * (2 * py / (1 + py));
			F.z[i][j][k] -= F.z[i][j][k] * (2 * pz / (1 + pz));
		}
		else LOOP3(i,a0,a1,j,b0,b1,k,c0,c1) {
			F.x[i][j][k] *= (1 - C->ax[n] * C->Jx[n][i][j][k]) / (1 + C->ax[n] * C->Jx[n][i][j][k]);
			F.y[i][j][k] *= (1 - C->ay[n] * C->Jy[n][i][j][k]) / (1 + C->ay[n] * C->Jy[n][i][j][k]);
			F.z[i][j][k] *= (1 - C->az[n] * C->Jz[n][i][j][k]) / (1 + C->az[n] * C->Jz[n][i][j][k]);
		}
	}
	for (int n = 0; n < C->N; n++) {
		int a0 = MAX(i0, C->iMin[n]), a1 = MIN(i1, C->iMax[n]);
		int b0 = MAX(j0, C->jMin[n]), b1 = MIN(j1, C->jMax[n]);
		int c0 = MAX(k0, C->kMin[n]), c1 = MIN(k1, C->kMax[n]);
		for (int p = 0; p < C->NK[n]; p++) LOOP3(i,a0,a1,j,b0,b1,k,c0,c1) {
			F.x[i][j][k] -= F.Jx[n][p][i][j][k];
			F.y[i][j][k] -= F.Jy[n][p][i][j][k];
			F.z[i][j][k] -= F.Jz[n][p][i][j][k];
		}
	}
	if (C->x && C->y && C->z) LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) {
		F.x[i][j][k] += (C->dtdz[k] * (G.y[i][j][k] - G.y[i][j][k+Alt]) + C->dtdy[j] * (G.z[i][j+Alt][k] - G.z[i][j][k])) * C->x[i][j][k];
		F.y[i][j][k] += (C->dtdx[i] * (G.z[i][j][k] - G.z[i+Alt][j][k]) + C->dtdz[k] * (G.x[i][j][k+Alt] - G.x[i][j][k])) * C->y[i][j][k];
		F.z[i][j][k] += (C->dtdy[j] * (G.x[i][j][k] - G.x[i][j+Alt][k]) + C->dtdx[i] * (G.y[i+Alt][j][k] - G.y[i][j][k])) * C->z[i][j][k];
	}
	else LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) {
		F.x[i][j][k] += (C->dtdz[k] * (G.y[i][j][k] - G.y[i][j][k+Alt]) + C->dtdy[j] * (G.z[i][j+Alt][k] - G.z[i][j][k]));
		F.y[i][j][k] += (C->dtdx[i] * (G.z[i][j][k] - G.z[i+Alt][j][k]) + C->dtdz[k] * (G.x[i][j][k+Alt] - G.x[i][j][k]));
		F.z[i][j][k] += (C->dtdy[j] * (G.x[i][j][k] - G.x[i][j+Alt][k]) + C->dtdx[i] * (G.y[i+Alt][j][k] - G.y[i][j][k]));
	}
	/* slabs: xMin, yMin, zMin, xMax, yMax, zMax */
	int lo = -(Alt-1)/2, hi = -(Alt+3)/2;
	if (W->iMIN < W->iMin) psiX(F, G, C, F.xMinPy, F.xMinPz, Alt, W->iMIN+lo, W->iMin+hi, j0, j1, k0, k1);
	if (W->jMIN < W->jMin) psiY(F, G, C, F.yMinPz, F.yMinPx, Alt, i0, i1, W->jMIN+lo, W->jMin+hi, k0, k1);
	if (W->kMIN < W->kMin) psiZ(F, G, C, F.zMinPx, F.zMinPy, Alt, i0, i1, j0, j1, W->kMIN+lo, W->kMin+hi);
	if (W->iMAX > W->iMax) psiX(F, G, C, F.xMaxPy, F.xMaxPz, Alt, W->iMax+2, W->iMAX, j0, j1, k0, k1);
	if (W->jMAX > W->jMax) psiY(F, G, C, F.yMaxPz, F.yMaxPx, Alt, i0, i1, W->jMax+2, W->jMAX, k0, k1);
	if (W->kMAX > W->kMax) psiZ(F, G, C, F.zMaxPx, F.zMaxPy, Alt, i0, i1, j0, j1, W->kMax+2, W->kMAX);
}

/* ADE polarisation currents of every dispersive object, driven by F
 * (reference src/update.c:128-158): Drude J' = JJ J + JE fill F;
 * pair J' = JJ J + JK K + JE fill F then K' = KJ J' + KK K + KE fill F. */
static void currentStep(world W, vfield F, coeffs *C)
{
	for (int n = 0; n < C->N; n++) {
		int a0 = MAX(W->iMIN, C->iMin[n]), a1 = MIN(W->iMAX, C->iMax[n]);
		int b0 = MAX(W->jMIN, C->jMin[n]), b1 = MIN(W->jMAX, C->jMax[n]);
		int c0 = MAX(W->kMIN, C->kMin[n]), c1 = MIN(W->kMAX, C->kMax[n]);
		for (int p = 0; p < C->NJ[n]; p++) LOOP3(i,a0,a1,j,b0,b1,k,c0,c1) {
			F.Jx[n][p][i][j][k] = C->JJx[n][p] * F.Jx[n][p][i][j][k] + C->JEx[n][p] * C->Jx[n][i][j][k] * F.x[i][j][k];
			F.Jy[n][p][i][j][k] = C->JJy[n][p] * F.Jy[n][p][i][j][k] + C->JEy[n][p] * C->Jy[n][i][j][k] * F.y[i][j][k];
			F.Jz[n][p][i][j][k] = C->JJz[n][p] * F.Jz[n][p][i][j][k] + C->JEz[n][p] * C->Jz[n][i][j][k] * F.z[i][j][k];
		}
		float ***fill[3] = { C->Jx[n], C->Jy[n], C->Jz[n] };
		float ***Fc[3] = { F.x, F.y, F.z };
		float ****Jc[3] = { F.Jx[n], F.Jy[n], F.Jz[n] }, ****Kc[3] = { F.Kx[n], F.Ky[n], F.Kz[n] };
		float *JJ[3] = { C->JJx[n], C->JJy[n], C->JJz[n] }, *JK[3] = { C->JKx[n], C->JKy[n], C->JKz[n] }, *JE[3] = { C->JEx[n], C->JEy[n], C->JEz[n] };
		float *KJ[3] = { C->KJx[n], C->KJy[n], C->KJz[n] }, *KK[3] = { C->KKx[n], C->KKy[n], C->KKz[n] }, *KE[3] = { C->KEx[n], C->KEy[n], C->KEz[n] };
		for (int a = 0; a < 3; a++) for (int p = C->NJ[n]; p < C->NK[n]; p++) LOOP3(i,a0,a1,j,b0,b1,k,c0,c1) {
			float ***J = Jc[a][p], ***K = Kc[a][p];
			J[i][j][k] = JJ[a][p] * J[i][j][k] + JK[a][p] * K[i][j][k] + JE[a][p] * fill[a][i][j][k] * Fc[a][i][j][k];
			K[i][j][k] = KJ[a][p] * J[i][j][k] + KK[a][p] * K[i][j][k] + KE[a][p] * fill[a][i][j][k] * Fc[a][i][j][k];
		}
	}
}

/* soft sources along a chain (reference src/update.c:161-179) */
static void sourceStep(world W, source S, float t)
{
	for (; S; S = S->S) {
		if (!(W->n < S->N)) continue;
		if (S->Phase) {
			LOOP3(i,S->iMin,S->iMax,j,S->jMin,S->jMax,k,S->kMin,S->kMax)
				S->F[i][j][k] += (S->Amplitude ? S->Amplitude[i][j][k] : S->amplitude) * S->waveForm(W, S, t, S->Phase[i][j][k]);
		} else {
			float f = S->waveForm(W, S, t, S->phase);
			if (S->Amplitude) LOOP3(i,S->iMin,S->iMax,j,S->jMin,S->jMax,k,S->kMin,S->kMax) S->F[i][j][k] += S->Amplitude[i][j][k] * f;
			else LOOP3(i,S->iMin,S->iMax,j,S->jMin,S->jMax,k,S->kMin,S->kMax) S->F[i][j][k] += S->amplitude * f;
		}
	}
}

/* F += dtds G[+Alt] (* C) on one TFSF face plane (reference src/update.c:194-202) */
static void faceStep(float ***F, float ***G, float ***C, float dtds, int i0, int i1, int j0, int j1, int k0, int k1, int ia, int ja, int ka)
{
	if (C) LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) F[i][j][k] += dtds * G[i+ia][j+ja][k+ka] * C[i][j][k];
	else LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) F[i][j][k] += dtds * G[i+ia][j+ja][k+ka];
}

void updateE(world W);
void updateH(world W);

/* incident-field corrections on the 12 TFSF face planes after advancing
 * the auxiliary world (reference src/update.c:205-237) */
static void tfsfE(world W, tfsf S)
{
	for (; S; S = S->S) {
		updateE(S->W);
		coeffs *C = W->CE;
		for (int n = 0; n <= W->complexField; n++) {
			vfield *E = &W->E[n], *h = &S->W->H[n];
			if (S->iMin > W->iMIN) {
				faceStep(E->z, h->y, C->z, -C->dtdx[S->iMin], S->iMin, S->iMin, S->jMin, S->jMax, S->kMIN, S->kMAX, 0, 0, 0);
				faceStep(E->y, h->z, C->y, +C->dtdx[S->iMin], S->iMin, S->iMin, S->jMIN, S->jMAX, S->kMin, S->kMax, 0, 0, 0);
			}
			if (S->jMin > W->jMIN) {
				faceStep(E->x, h->z, C->x, -C->dtdy[S->jMin], S->iMIN, S->iMAX, S->jMin, S->jMin, S->kMin, S->kMax, 0, 0, 0);
				faceStep(E->z, h->x, C->z, +C->dtdy[S->jMin], S->iMin, S->iMax, S->jMin, S->jMin, S->kMIN, S->kMAX, 0, 0, 0);
			}
			if (S->kMin > W->kMIN) {
				faceStep(E->y, h->x, C->y, -C->dtdz[S->kMin], S->iMin, S->iMax, S->jMIN, S->jMAX, S->kMin, S->kMin, 0, 0, 0);
				faceStep(E->x, h->y, C->x, +C->dtdz[S->kMin], S->iMIN, S->iMAX, S->jMin, S->jMax, S->kMin, S->kMin, 0, 0, 0);
			}
			if (S->iMax < W->iMAX) {
				faceStep(E->z, h->y, C->z, +C->dtdx[S->iMax], S->iMax, S->iMax, S->jMin, S->jMax, S->kMIN, S->kMAX, 1, 0, 0);
				faceStep(E->y, h->z, C->y, -C->dtdx[S->iMax], S->iMax, S->iMax, S->jMIN, S->jMAX, S->kMin, S->kMax, 1, 0, 0);
			}
			if (S->jMax < W->jMAX) {
				faceStep(E->x, h->z, C->x, +C->dtdy[S->jMax], S->iMIN, S->iMAX, S->jMax, S->jMax, S->kMin, S->kMax, 0, 1, 0);
				faceStep(E->z, h->x, C->z, -C->dtdy[S->jMax], S->iMin, S->iMax, S->jMax, S->jMax, S->kMIN, S->kMAX, 0, 1, 0);
			}
			if (S->kMax < W->kMAX) {
				faceStep(E->y, h->x, C->y, +C->dtdz[S->kMax], S->iMin, S->iMax, S->jMIN, S->jMAX, S->kMax, S->kMax, 0, 0, 1);
				faceStep(E->x, h->y, C->x, -C->dtdz[S->kMax], S->iMIN, S->iMAX, S->jMin, S->jMax, S->kMax, S->kMax, 0, 0, 1);
			}
		}
	}
}

/* (reference src/update.c:240-272) */
static void tfsfH(world W, tfsf S)
{
	for (; S; S = S->S) {
		updateH(S->W);
		coeffs *C = W->CH;
		for (int n = 0; n <= W->complexField; n++) {
			vfield *H = &W->H[n], *e = &S->W->E[n];
			if (S->iMin > W->iMIN) {
				faceStep(H->z, e->y, C->z, +C->dtdx[S->iMin], S->iMin, S->iMin, S->jMIN, S->jMAX, S->kMin, S->kMax, 0, 0, 0);
				faceStep(H->y, e->z, C->y, -C->dtdx[S->iMin], S->iMin, S->iMin, S->jMin, S->jMax, S->kMIN, S->kMAX, 0, 0, 0);
			}
			if (S->jMin > W->jMIN) {
				faceStep(H->x, e->z, C->x, +C->dtdy[S->jMin], S->iMin, S->iMax, S->jMin, S->jMin, S->kMIN, S->kMAX, 0, 0, 0);
				faceStep(H->z, e->x, C->z, -C->dtdy[S->jMin], S->iMIN, S->iMAX, S->jMin, S->jMin, S->kMin, S->kMax, 0, 0, 0);
			}
			if (S->kMin > W->kMIN) {
				faceStep(H->y, e->x, C->y, +C->dtdz[S->kMin], S->iMIN, S->iMAX, S->jMin, S->jMax, S->kMin, S->kMin, 0, 0, 0);
				faceStep(H->x, e->y, C->x, -C->dtdz[S->kMin], S->iMin, S->iMax, S->jMIN, S->jMAX, S->kMin, S->kMin, 0, 0, 0);
			}
			if (S->iMax < W->iMAX) {
				faceStep(H->z, e->y, C->z, -C->dtdx[S->iMax+1], S->iMax+1, S->iMax+1, S->jMIN, S->jMAX, S->kMin, S->kMax, -1, 0, 0);
				faceStep(H->y, e->z, C->y, +C->dtdx[S->iMax+1], S->iMax+1, S->iMax+1, S->jMin, S->jMax, S->kMIN, S->kMAX, -1, 0, 0);
			}
			if (S->jMax < W->jMAX) {
				faceStep(H->x, e->z, C->x, -C->dtdy[S->jMax+1], S->iMin, S->iMax, S->jMax+1, S->jMax+1, S->kMIN, S->kMAX, 0, -1, 0);
				faceStep(H->z, e->x, C->z, +C->dtdy[S->jMax+1], S->iMIN, S->iMAX, S->jMax+1, S->jMax+1, S->kMin, S->kMax, 0, -1, 0);
			}
			if (S->kMax < W->kMAX) {
				faceStep(H->y, e->x, C->y, -C->dtdz[S->kMax+1], S->iMIN, S->iMAX, S->jMin, S->jMax, S->kMax+1, S->kMax+1, 0, 0, -1);
				faceStep(H->x, e->y, C->x, +C->dtdz[S->kMax+1], S->iMin, S->iMax, S->jMIN, S->jMAX, S->kMax+1, S->kMax+1, 0, 0, -1);
			}
		}
	}
}

#define GHOST(W, F, c, ...) (copyBoundary)(W->F[0].c, W->complexField ? W->F[1].c : 0, __VA_ARGS__)

/* FP16 field storage (environment ALIS_ORACLE_FP16_STORAGE=1; the
 * engine's half storage, alisgpu_world_set_storage): the E and H
 * components of a real world stepped by the user (not its TFSF auxiliary
 * columns, not worlds with complex fields) are held as IEEE half values
 * times 2^e, one exponent e per
 * component and x plane.  A half step takes e from the largest magnitude
 * M the plane's cells of that component reached in the previous half step
 * of the field, before rounding: e = x - 11 for M = f 2^x, f in [0.5, 1)
 * (M 2^-e in [2^10, 2^11): 32 times headroom below the half maximum
 * 65504), e = -11 while M = 0, e = 100 for M infinite or NaN, clamped to
 * [-100, 100].  The step rounds every cell it updates (after the curl,
 * currents, CPML and TFSF corrections) to v = half(v 2^-e) 2^e, with
 * round-to-nearest-even and values beyond the half range saturated at
 * +-65504 2^e; the source patches then add to the rounded values and
 * their cells are rounded again with the same e.  Ghost copies move the
 * rounded values unchanged.  ADE currents, CPML psi and the auxiliary
 * columns stay float.  M is taken over the float bits of |v| as unsigned
 * integers (the order of magnitudes, NaN above infinity). */
#define HALF_E0 (-11)
#define HALF_EMIN (-100)
#define HALF_EMAX 100
static int fp16Storage = -1, stepDepth;

typedef struct HalfState {
	world W;
	int ni;
	unsigned *M[2][2];                     /* [E/H][previous/current] 3 x ni */
	struct HalfState *next;
} HalfState;
static HalfState *halfStates;

static int halfExponent(unsigned mbits)
{
	if (mbits == 0) return HALF_E0;
	if (mbits >= 0x7f800000u) return HALF_EMAX;
	float m;
	memcpy(&m, &mbits, 4);
	int x;
	frexpf(m, &x);
	int e = x - 11;
	return e < HALF_EMIN ? HALF_EMIN : e > HALF_EMAX ? HALF_EMAX : e;
}

static float roundHalf(float v, int e)
{
	float x = v * ldexpf(1.0f, -e);
	if (x > 65504.0f) x = 65504.0f;
	else if (x < -65504.0f) x = -65504.0f;
	return (float)(_Float16)x * ldexpf(1.0f, e);
}

static HalfState *halfState(world W)
{
	HalfState *h = halfStates;
	while (h && h->W != W) h = h->next;
	if (!h) {
		h = calloc(1, sizeof *h);
		h->W = W, h->ni = W->iMAX - W->iMIN + 1;
		for (int f = 0; f < 2; f++) for (int q = 0; q < 2; q++) h->M[f][q] = calloc(3 * (size_t)h->ni, sizeof(unsigned));
		h->next = halfStates, halfStates = h;
	}
	return h;
}

/* a rebooted world starts again from M = 0 */
static void halfForget(world W)
{
	for (HalfState *h = halfStates; h; h = h->next)
		if (h->W == W)
			for (int f = 0; f < 2; f++) for (int q = 0; q < 2; q++) memset(h->M[f][q], 0, 3 * (size_t)h->ni * sizeof(unsigned));
}

static int halfOn(void)
{
	if (fp16Storage < 0) {
		const char *e = getenv("ALIS_ORACLE_FP16_STORAGE");
		fp16Storage = e && e[0] == '1';
#ifdef ALIS_ORACLE_FP64_H
		fp16Storage = 0;                   /* a float storage form: not in the FP64 build */
#endif
	}
	return fp16Storage && stepDepth == 1;
}

/* the half step's rounding of the cells it updated (field f: 0 E, 1 H);
 * worlds with complex fields stay float */
static void storeStep(world W, vfield F, int f)
{
	if (!halfOn() || W->complexField) return;
	HalfState *h = halfState(W);
	float ***c[3] = { F.x, F.y, F.z };
	unsigned *prev = h->M[f][0], *cur = h->M[f][1];
	for (int q = 0; q < 3; q++) {
		_Pragma("omp parallel for")
		for (int i = W->iMIN; i <= W->iMAX; i++) {
			int e = halfExponent(prev[q * h->ni + (i - W->iMIN)]);
			unsigned m = 0;
			for (int j = W->jMIN; j <= W->jMAX; j++) for (int k = W->kMIN; k <= W->kMAX; k++) {
				float a = fabsf(c[q][i][j][k]);
				unsigned bits;
				memcpy(&bits, &a, 4);
				if (bits > m) m = bits;
				c[q][i][j][k] = roundHalf(c[q][i][j][k], e);
			}
			cur[q * h->ni + (i - W->iMIN)] = m;
		}
	}
	h->M[f][0] = cur, h->M[f][1] = prev;
}

/* the source patches' cells, rounded again with the exponents of the step
 * (storeStep has made them the previous ones) */
static void storeSources(world W, vfield F, int f, source S)
{
	if (!halfOn() || W->complexField) return;
	HalfState *h = halfState(W);
	const unsigned *used = h->M[f][1];
	float ***c[3] = { F.x, F.y, F.z };
	for (; S; S = S->S) {
		if (!(W->n < S->N)) continue;
		int q = S->F == F.x ? 0 : S->F == F.y ? 1 : S->F == F.z ? 2 : -1;
		if (q < 0 || S->iMin < W->iMIN || S->iMax > W->iMAX || S->jMin < W->jMIN || S->jMax > W->jMAX ||
		    S->kMin < W->kMIN || S->kMax > W->kMAX) {
			fprintf(stderr, "oracle: FP16 storage needs source patches inside the updated cells\n");
			exit(1);
		}
		for (int i = S->iMin; i <= S->iMax; i++) {
			int e = halfExponent(used[q * h->ni + (i - W->iMIN)]);
			for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
				c[q][i][j][k] = roundHalf(c[q][i][j][k], e);
		}
	}
}

/* reference src/update.c:275-299 */
void updateE(world W)
{
	stepDepth++;
	for (int m = 0; m <= W->complexField; m++) {
		curlStep(W, W->E[m], W->H[m], W->CE, 1);
		currentStep(W, W->H[m], W->CH);
	}
	if (W->S) tfsfE(W, W->S);
	storeStep(W, W->E[0], 0);
	if (W->SE) sourceStep(W, W->SE, W->H->t), storeSources(W, W->E[0], 0, W->SE);
	int iAlt = (W->xMinSur==PBC || W->xMinSur==BBC ? W->iNUM-1 : 1);
	int jAlt = (W->yMinSur==PBC || W->yMinSur==BBC ? W->jNUM-1 : 1);
	int kAlt = (W->zMinSur==PBC || W->zMinSur==BBC ? W->kNUM-1 : 1);
	GHOST(W, E, x, W->coskx, -W->sinkx, W->iMAX+1, W->iMAX+1, W->jMIN, W->jMAX, W->kMIN, W->kMAX, -iAlt, 0, 0);
	GHOST(W, E, z, W->coskz, -W->sinkz, W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMAX+1, W->kMAX+1, 0, 0, -kAlt);
	if (W->yMinSur==HBC) {
		GHOST(W, E, y, W->coskym, -W->sinkym, W->iMIN, 0, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMAX, 1-W->jNUM, 0);
		GHOST(W, E, y, W->coskyp, -W->sinkyp, 1, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMIN, 1-W->jNUM, 0);
	} else {
		GHOST(W, E, y, W->cosky, -W->sinky, W->iMIN, W->iMAX, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, 0, -jAlt, 0);
	}
	W->t = W->E->t = ++W->n * W->dt;
	stepDepth--;
}

/* reference src/update.c:302-341 */
void updateH(world W)
{
	stepDepth++;
	for (int m = 0; m <= W->complexField; m++) {
		curlStep(W, W->H[m], W->E[m], W->CH, -1);
		currentStep(W, W->E[m], W->CE);
	}
	if (W->S) tfsfH(W, W->S);
	storeStep(W, W->H[0], 1);
	if (W->SH) sourceStep(W, W->SH, W->E->t), storeSources(W, W->H[0], 1, W->SH);
	int iAlt = (W->xMinSur==PBC || W->xMinSur==BBC ? W->iNUM-1 : 1);
	int jAlt = (W->yMinSur==PBC || W->yMinSur==BBC ? W->jNUM-1 : 1);
	int kAlt = (W->zMinSur==PBC || W->zMinSur==BBC ? W->kNUM-1 : 1);
	GHOST(W, H, y, W->xMaxSur==PEC?1:W->coskx, -W->sinkx, W->iMAX+1, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, -iAlt, 0, 0);
	GHOST(W, H, z, W->xMaxSur==PEC?1:W->coskx, -W->sinkx, W->iMAX+1, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, -iAlt, 0, 0);
	GHOST(W, H, x, W->zMaxSur==PEC?1:W->coskz, -W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMAX+1, W->kMAX+1, 0, 0, -kAlt);
	GHOST(W, H, y, W->zMaxSur==PEC?1:W->coskz, -W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMAX+1, W->kMAX+1, 0, 0, -kAlt);
	GHOST(W, H, y, W->coskx, W->sinkx, W->iMIN, W->iMIN, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, iAlt, 0, 0);
	GHOST(W, H, z, W->coskx, W->sinkx, W->iMIN, W->iMIN, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, iAlt, 0, 0);
	GHOST(W, H, x, W->coskz, W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMIN, 0, 0, kAlt);
	GHOST(W, H, y, W->coskz, W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMIN, 0, 0, kAlt);
	if (W->yMinSur==HBC) {
		GHOST(W, H, x, W->coskyp, W->sinkyp, W->iMIN, 0, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMAX, W->jNUM-1, 0);
		GHOST(W, H, z, W->coskyp, W->sinkyp, W->iMIN, 0, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMAX, W->jNUM-1, 0);
		GHOST(W, H, x, W->coskym, -W->sinkym, W->iMIN, 0, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMAX, 1-W->jNUM, 0);
		GHOST(W, H, z, W->coskym, -W->sinkym, W->iMIN, 0, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMAX, 1-W->jNUM, 0);
		GHOST(W, H, x, W->coskym, W->sinkym, 1, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMIN, W->jNUM-1, 0);
		GHOST(W, H, z, W->coskym, W->sinkym, 1, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMIN, W->jNUM-1, 0);
		GHOST(W, H, x, W->coskyp, -W->sinkyp, 1, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMIN, 1-W->jNUM, 0);
		GHOST(W, H, z, W->coskyp, -W->sinkyp, 1, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMIN, 1-W->jNUM, 0);
	} else {
		GHOST(W, H, z, W->yMaxSur==PEC?1:W->cosky, -W->sinky, W->iMIN, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX+1, 0, -jAlt, 0);
		GHOST(W, H, x, W->yMaxSur==PEC?1:W->cosky, -W->sinky, W->iMIN, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX+1, 0, -jAlt, 0);
		GHOST(W, H, z, W->cosky, W->sinky, W->iMIN, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX+1, 0, jAlt, 0);
		GHOST(W, H, x, W->cosky, W->sinky, W->iMIN, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX+1, 0, jAlt, 0);
	}
	W->t = W->H->t = W->E->t + 0.5 * W->dt;
	stepDepth--;
}


/* --- running DFT on phaser faces (reference src/phaser.c:83-110) --- */

/* FP64 accumulation (environment ALIS_ORACLE_DFT64=1): the same float
 * fields and float phase factors, summed in double complex in shadow
 * arrays; alis_be_sync_phasers_of rounds them into the face arrays.  The
 * GPU's compensated (Kahan) accumulation is checked against it. */
typedef struct Shadow {
	float complex ***A;
	int i0, j0, k0, ni, nj, nk;
	double complex *v;
	struct Shadow *next;
} Shadow;
static Shadow *shadows;
static int dft64 = -1;

static double complex *shadowOf(float complex ***A, int i0, int i1, int j0, int j1, int k0, int k1)
{
	for (Shadow *s = shadows; s; s = s->next) if (s->A == A) return s->v;
	Shadow *s = calloc(1, sizeof *s);
	s->A = A, s->i0 = i0, s->j0 = j0, s->k0 = k0, s->ni = 1 + i1 - i0, s->nj = 1 + j1 - j0, s->nk = 1 + k1 - k0;
	s->v = calloc((size_t)(1 + i1 - i0) * s->nj * s->nk, sizeof(double complex));
	s->next = shadows;
	shadows = s;
	return s->v;
}

static void dftFace64(cfield *c, float ***e1, float ***e2, float ***h1, float ***h2,
                      float complex pE, float complex pH, int axis, int i0, int i1, int j0, int j1, int k0, int k1)
{
	float complex ***E1, ***E2, ***H1, ***H2;
	if (axis == 0) E1 = c->Ey, E2 = c->Ez, H1 = c->Hy, H2 = c->Hz;
	else if (axis == 1) E1 = c->Ez, E2 = c->Ex, H1 = c->Hz, H2 = c->Hx;
	else E1 = c->Ex, E2 = c->Ey, H1 = c->Hx, H2 = c->Hy;
	if (!(E1 && E2 && H1 && H2)) return;
	double complex *s1 = shadowOf(E1, i0, i1, j0, j1, k0, k1), *s2 = shadowOf(E2, i0, i1, j0, j1, k0, k1);
	double complex *s3 = shadowOf(H1, i0, i1, j0, j1, k0, k1), *s4 = shadowOf(H2, i0, i1, j0, j1, k0, k1);
	int di = axis==0, dj = axis==1, dk = axis==2, nj = 1 + j1 - j0, nk = 1 + k1 - k0;
	double complex qE = pE, qH = pH;
	for (int i = i0; i <= i1; i++) for (int j = j0; j <= j1; j++) for (int k = k0; k <= k1; k++) {
		size_t o = ((size_t)(i - i0) * nj + (j - j0)) * nk + (k - k0);
		s1[o] += qE * (double)e1[i][j][k];
		s2[o] += qE * (double)e2[i][j][k];
		s3[o] += qH * ((double)h1[i][j][k] + (double)h1[i+di][j+dj][k+dk]) * 0.5;
		s4[o] += qH * ((double)h2[i][j][k] + (double)h2[i+di][j+dj][k+dk]) * 0.5;
	}
}

static void dftFace(world W, cfield *c, float ***e1, float ***e2, float ***h1, float ***h2,
                    float complex pE, float complex pH, int axis, int i0, int i1, int j0, int j1, int k0, int k1)
{
	if (!(c->Ex || c->Ey || c->Ez)) return;
	if (dft64 < 0) { const char *e = getenv("ALIS_ORACLE_DFT64"); dft64 = e && e[0] == '1'; }
	if (dft64) { dftFace64(c, e1, e2, h1, h2, pE, pH, axis, i0, i1, j0, j1, k0, k1); return; }
	float complex ***E1, ***E2, ***H1, ***H2;
	if (axis == 0) E1 = c->Ey, E2 = c->Ez, H1 = c->Hy, H2 = c->Hz;
	else if (axis == 1) E1 = c->Ez, E2 = c->Ex, H1 = c->Hz, H2 = c->Hx;
	else E1 = c->Ex, E2 = c->Ey, H1 = c->Hx, H2 = c->Hy;
	if (!(E1 && E2 && H1 && H2)) return;
	int di = axis==0, dj = axis==1, dk = axis==2;
	LOOP3(i,i0,i1,j,j0,j1,k,k0,k1) {
		E1[i][j][k] += pE * e1[i][j][k];
		E2[i][j][k] += pE * e2[i][j][k];
		H1[i][j][k] += pH * (h1[i][j][k] + h1[i+di][j+dj][k+dk]) * 0.5;
		H2[i][j][k] += pH * (h2[i][j][k] + h2[i+di][j+dj][k+dk]) * 0.5;
	}
	(void)W;
}

void updatePhaser(world W, phaser P)
{
	do {
		float complex pE = cexpf(2 * PI * I * P->f * W->E->t);
		float complex pH = cexpf(2 * PI * I * P->f * W->H->t);
		vfield *E = W->E, *H = W->H;
		dftFace(W, &P->xMin, E->y, E->z, H->y, H->z, pE, pH, 0, P->iMin, P->iMin, P->jMin, P->jMax, P->kMin, P->kMax);
		dftFace(W, &P->xMax, E->y, E->z, H->y, H->z, pE, pH, 0, P->iMax, P->iMax, P->jMin, P->jMax, P->kMin, P->kMax);
		dftFace(W, &P->yMin, E->z, E->x, H->z, H->x, pE, pH, 1, P->iMin, P->iMax, P->jMin, P->jMin, P->kMin, P->kMax);
		dftFace(W, &P->yMax, E->z, E->x, H->z, H->x, pE, pH, 1, P->iMin, P->iMax, P->jMax, P->jMax, P->kMin, P->kMax);
		dftFace(W, &P->zMin, E->x, E->y, H->x, H->y, pE, pH, 2, P->iMin, P->iMax, P->jMin, P->jMax, P->kMin, P->kMin);
		dftFace(W, &P->zMax, E->x, E->y, H->x, H->y, pE, pH, 2, P->iMin, P->iMax, P->jMin, P->jMax, P->kMax, P->kMax);
		P++;
	} while (P->f);
}


/* --- far-field face sums (reference src/farfld.c:248-459) ---
 * REAL is float for the reference-precision restatement and double for
 * the FP64 oracle (environment ALIS_ORACLE_FF64=1), against which the
 * GPU's FP64 projection is also checked. */

#define DEFINE_FF(REAL, CPLX, CEXP, CONJ, NAME) \
static CPLX NAME##X(phaser P, cfield S, int i, tfield T, REAL kx, REAL ky) \
{ \
	world W = P->W; \
	CPLX *Y = (CPLX*)calloc(1-P->jMin+P->jMax, sizeof(CPLX)) - P->jMin, *Z = (CPLX*)calloc(1-P->kMin+P->kMax, sizeof(CPLX)) - P->kMin; \
	CPLX EyHz = 0, EzHy = 0, HyEz = 0, HzEy = 0, Sum = 0; \
	if (T.Hz || T.Ey) { \
		for (int j = P->jMin+1; j <= P->jMax; j++) Y[j] = W->CH->dy[j] * CEXP(I*ky*(REAL)W->jtoy(W, j-0.5)); \
		if (W->yMinSur==SYM) for (int j = P->jMin+1; j <= P->jMax; j++) Y[j] += CONJ(Y[j]) * W->cosky; \
	} \
	if (T.Hz) { \
		for (int k = P->kMin; k <= P->kMax; k++) Z[k] = W->CE->dz[k] * (CPLX)T.Hz[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin; k <= P->kMax; k++) Z[k] -= W->CE->dz[k] * (CPLX)T.Hz[-k] * W->coskz; \
		for (int j = P->jMin+1; j <= P->jMax; j++) { \
			CPLX sum = 0.5 * ((CPLX)S.Ey[i][j][P->kMin] * Z[P->kMin] + (CPLX)S.Ey[i][j][P->kMax] * Z[P->kMax]); \
			for (int k = P->kMin+1; k < P->kMax; k++) sum += (CPLX)S.Ey[i][j][k] * Z[k]; \
			EyHz += Y[j] * sum; \
		} \
	} \
	if (T.Ey) { \
		for (int k = P->kMin; k <= P->kMax; k++) Z[k] = W->CE->dz[k] * (CPLX)T.Ey[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin; k <= P->kMax; k++) Z[k] -= W->CE->dz[k] * (CPLX)T.Ey[-k] * W->coskz; \
		for (int j = P->jMin+1; j <= P->jMax; j++) { \
			CPLX sum = 0.5 * ((CPLX)S.Hz[i][j][P->kMin] * Z[P->kMin] + (CPLX)S.Hz[i][j][P->kMax] * Z[P->kMax]); \
			for (int k = P->kMin+1; k < P->kMax; k++) sum += (CPLX)S.Hz[i][j][k] * Z[k]; \
			HzEy += Y[j] * sum; \
		} \
	} \
	if (T.Hy || T.Ez) { \
		for (int j = P->jMin; j <= P->jMax; j++) Y[j] = W->CE->dy[j] * CEXP(I*ky*(REAL)W->jtoy(W, j)); \
		if (W->yMinSur==SYM) for (int j = P->jMin; j <= P->jMax; j++) Y[j] -= CONJ(Y[j]) * W->cosky; \
	} \
	if (T.Hy) { \
		for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] = W->CH->dz[k] * (CPLX)T.Hy[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] += W->CH->dz[k] * (CPLX)T.Hy[1-k] * W->coskz; \
		for (int k = P->kMin+1; k <= P->kMax; k++) { \
			CPLX sum = 0.5 * ((CPLX)S.Ez[i][P->jMin][k] * Y[P->jMin] + (CPLX)S.Ez[i][P->jMax][k] * Y[P->jMax]); \
			for (int j = P->jMin+1; j < P->jMax; j++) sum += (CPLX)S.Ez[i][j][k] * Y[j]; \
			EzHy += Z[k] * sum; \
		} \
	} \
	if (T.Ez) { \
		for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] = W->CH->dz[k] * (CPLX)T.Ez[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] += W->CH->dz[k] * (CPLX)T.Ez[1-k] * W->coskz; \
		for (int k = P->kMin+1; k <= P->kMax; k++) { \
			CPLX sum = 0.5 * ((CPLX)S.Hy[i][P->jMin][k] * Y[P->jMin] + (CPLX)S.Hy[i][P->jMax][k] * Y[P->jMax]); \
			for (int j = P->jMin+1; j < P->jMax; j++) sum += (CPLX)S.Hy[i][j][k] * Y[j]; \
			HyEz += Z[k] * sum; \
		} \
	} \
	Sum += (EyHz-HzEy-EzHy+HyEz) * CEXP(I*kx*(REAL)W->itox(W, i)); \
	if (W->xMinSur==SYM) Sum += (EyHz+HzEy-EzHy-HyEz) * CEXP(-I*kx*(REAL)W->itox(W, i)) * W->coskx; \
	free(Y + P->jMin); free(Z + P->kMin); \
	return Sum; \
} \
static CPLX NAME##Y(phaser P, cfield S, int j, tfield T, REAL kx, REAL ky) \
{ \
	world W = P->W; \
	CPLX *X = (CPLX*)calloc(1-P->iMin+P->iMax, sizeof(CPLX)) - P->iMin, *Z = (CPLX*)calloc(1-P->kMin+P->kMax, sizeof(CPLX)) - P->kMin; \
	CPLX ExHz = 0, EzHx = 0, HxEz = 0, HzEx = 0, Sum = 0; \
	if (T.Hx || T.Ez) { \
		for (int i = P->iMin; i <= P->iMax; i++) X[i] = W->CE->dx[i] * CEXP(I*kx*(REAL)W->itox(W, i)); \
		if (W->xMinSur==SYM) for (int i = P->iMin; i <= P->iMax; i++) X[i] -= CONJ(X[i]) * W->coskx; \
	} \
	if (T.Hx) { \
		for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] = W->CH->dz[k] * (CPLX)T.Hx[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] += W->CH->dz[k] * (CPLX)T.Hx[1-k] * W->coskz; \
		for (int k = P->kMin+1; k <= P->kMax; k++) { \
			CPLX sum = 0.5 * ((CPLX)S.Ez[P->iMin][j][k] * X[P->iMin] + (CPLX)S.Ez[P->iMax][j][k] * X[P->iMax]); \
			for (int i = P->iMin+1; i < P->iMax; i++) sum += (CPLX)S.Ez[i][j][k] * X[i]; \
			EzHx += Z[k] * sum; \
		} \
	} \
	if (T.Ez) { \
		for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] = W->CH->dz[k] * (CPLX)T.Ez[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin+1; k <= P->kMax; k++) Z[k] += W->CH->dz[k] * (CPLX)T.Ez[1-k] * W->coskz; \
		for (int k = P->kMin+1; k <= P->kMax; k++) { \
			CPLX sum = 0.5 * ((CPLX)S.Hx[P->iMin][j][k] * X[P->iMin] + (CPLX)S.Hx[P->iMax][j][k] * X[P->iMax]); \
			for (int i = P->iMin+1; i < P->iMax; i++) sum += (CPLX)S.Hx[i][j][k] * X[i]; \
			HxEz += Z[k] * sum; \
		} \
	} \
	if (T.Hz || T.Ex) { \
		for (int i = P->iMin+1; i <= P->iMax; i++) X[i] = W->CH->dx[i] * CEXP(I*kx*(REAL)W->itox(W, i-0.5)); \
		if (W->xMinSur==SYM) for (int i = P->iMin+1; i <= P->iMax; i++) X[i] += CONJ(X[i]) * W->coskx; \
	} \
	if (T.Hz) { \
		for (int k = P->kMin; k <= P->kMax; k++) Z[k] = W->CE->dz[k] * (CPLX)T.Hz[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin; k <= P->kMax; k++) Z[k] -= W->CE->dz[k] * (CPLX)T.Hz[-k] * W->coskz; \
		for (int i = P->iMin+1; i <= P->iMax; i++) { \
			CPLX sum = 0.5 * ((CPLX)S.Ex[i][j][P->kMin] * Z[P->kMin] + (CPLX)S.Ex[i][j][P->kMax] * Z[P->kMax]); \
			for (int k = P->kMin+1; k < P->kMax; k++) sum += (CPLX)S.Ex[i][j][k] * Z[k]; \
			ExHz += X[i] * sum; \
		} \
	} \
	if (T.Ex) { \
		for (int k = P->kMin; k <= P->kMax; k++) Z[k] = W->CE->dz[k] * (CPLX)T.Ex[k]; \
		if (W->zMinSur==SYM) for (int k = P->kMin; k <= P->kMax; k++) Z[k] -= W->CE->dz[k] * (CPLX)T.Ex[-k] * W->coskz; \
		for (int i = P->iMin+1; i <= P->iMax; i++) { \
			CPLX sum = 0.5 * ((CPLX)S.Hz[i][j][P->kMin] * Z[P->kMin] + (CPLX)S.Hz[i][j][P->kMax] * Z[P->kMax]); \
			for (int k = P->kMin+1; k < P->kMax; k++) sum += (CPLX)S.Hz[i][j][k] * Z[k]; \
			HzEx += X[i] * sum; \
		} \
	} \
	Sum += (EzHx-HxEz-ExHz+HzEx) * CEXP(I*ky*(REAL)W->jtoy(W, j)); \
	if (W->yMinSur==SYM) Sum += (EzHx+HxEz-ExHz-HzEx) * CEXP(-I*ky*(REAL)W->jtoy(W, j)) * W->cosky; \
	free(X + P->iMin); free(Z + P->kMin); \
	return Sum; \
} \
static CPLX NAME##Z(phaser P, cfield S, int k, tfield T, REAL kx, REAL ky) \
{ \
	world W = P->W; \
	CPLX *X = (CPLX*)calloc(1-P->iMin+P->iMax, sizeof(CPLX)) - P->iMin, *Y = (CPLX*)calloc(1-P->jMin+P->jMax, sizeof(CPLX)) - P->jMin; \
	CPLX ExHy = 0, EyHx = 0, HxEy = 0, HyEx = 0, Sum = 0; \
	if (T.Hy || T.Ex) { \
		for (int i = P->iMin+1; i <= P->iMax; i++) X[i] = W->CH->dx[i] * CEXP(I*kx*(REAL)W->itox(W, i-0.5)); \
		if (W->xMinSur==SYM) for (int i = P->iMin+1; i <= P->iMax; i++) X[i] += CONJ(X[i]) * W->coskx; \
		for (int j = P->jMin; j <= P->jMax; j++) Y[j] = W->CE->dy[j] * CEXP(I*ky*(REAL)W->jtoy(W, j)); \
		if (W->yMinSur==SYM) for (int j = P->jMin; j <= P->jMax; j++) Y[j] -= CONJ(Y[j]) * W->cosky; \
	} \
	if (T.Hy) { \
		for (int i = P->iMin+1; i <= P->iMax; i++) { \
			CPLX sum = 0.5 * ((CPLX)S.Ex[i][P->jMin][k] * Y[P->jMin] + (CPLX)S.Ex[i][P->jMax][k] * Y[P->jMax]); \
			for (int j = P->jMin+1; j < P->jMax; j++) sum += (CPLX)S.Ex[i][j][k] * Y[j]; \
			ExHy += X[i] * sum; \
		} \
		Sum += ExHy * 0.5 * ((CPLX)T.Hy[k]+(CPLX)T.Hy[k+1]); \
		if (W->zMinSur==SYM) Sum += ExHy * 0.5 * ((CPLX)T.Hy[1-k]+(CPLX)T.Hy[-k]) * W->coskz; \
	} \
	if (T.Ex) { \
		for (int i = P->iMin+1; i <= P->iMax; i++) { \
			CPLX sum = 0.5 * ((CPLX)S.Hy[i][P->jMin][k] * Y[P->jMin] + (CPLX)S.Hy[i][P->jMax][k] * Y[P->jMax]); \
			for (int j = P->jMin+1; j < P->jMax; j++) sum += (CPLX)S.Hy[i][j][k] * Y[j]; \
			HyEx += X[i] * sum; \
		} \
		Sum -= HyEx * (CPLX)T.Ex[k]; \
		if (W->zMinSur==SYM) Sum += HyEx * (CPLX)T.Ex[-k] * W->coskz; \
	} \
	if (T.Hx || T.Ey) { \
		for (int i = P->iMin; i <= P->iMax; i++) X[i] = W->CE->dx[i] * CEXP(I*kx*(REAL)W->itox(W, i)); \
		if (W->xMinSur==SYM) for (int i = P->iMin; i <= P->iMax; i++) X[i] -= CONJ(X[i]) * W->coskx; \
		for (int j = P->jMin+1; j <= P->jMax; j++) Y[j] = W->CH->dy[j] * CEXP(I*ky*(REAL)W->jtoy(W, j-0.5)); \
		if (W->yMinSur==SYM) for (int j = P->jMin+1; j <= P->jMax; j++) Y[j] += CONJ(Y[j]) * W->cosky; \
	} \
	if (T.Hx) { \
		for (int j = P->jMin+1; j <= P->jMax; j++) { \
			CPLX sum = 0.5 * ((CPLX)S.Ey[P->iMin][j][k] * X[P->iMin] + (CPLX)S.Ey[P->iMax][j][k] * X[P->iMax]); \
			for (int i = P->iMin+1; i < P->iMax; i++) sum += (CPLX)S.Ey[i][j][k] * X[i]; \
			EyHx += Y[j] * sum; \
		} \
		Sum -= EyHx * 0.5 * ((CPLX)T.Hx[k]+(CPLX)T.Hx[k+1]); \
		if (W->zMinSur==SYM) Sum -= EyHx * 0.5 * ((CPLX)T.Hx[1-k]+(CPLX)T.Hx[-k]) * W->coskz; \
	} \
	if (T.Ey) { \
		for (int j = P->jMin+1; j <= P->jMax; j++) { \
			CPLX sum = 0.5 * ((CPLX)S.Hx[P->iMin][j][k] * X[P->iMin] + (CPLX)S.Hx[P->iMax][j][k] * X[P->iMax]); \
			for (int i = P->iMin+1; i < P->iMax; i++) sum += (CPLX)S.Hx[i][j][k] * X[i]; \
			HxEy += Y[j] * sum; \
		} \
		Sum += HxEy * (CPLX)T.Ey[k]; \
		if (W->zMinSur==SYM) Sum -= HxEy * (CPLX)T.Ey[-k] * W->coskz; \
	} \
	free(X + P->iMin); free(Y + P->jMin); \
	return Sum; \
}

DEFINE_FF(float, float complex, cexpf, conjf, ff32)
DEFINE_FF(double, double complex, cexp, conj, ff64)

void alis_be_farfield_sums(phaser P, int nA, const tfield *T, const float *kx, const float *ky, double complex *out)
{
	const char *env = getenv("ALIS_ORACLE_FF64");
	int wide = env && env[0] == '1';
	world W = P->W;
	for (int a = 0; a < nA; a++) {
		if (wide) {
			double complex Sum = 0;
			if (W->xMinSur==PML) Sum -= ff64X(P, P->xMin, P->iMin, T[a], kx[a], ky[a]);
			if (W->xMaxSur==PML) Sum += ff64X(P, P->xMax, P->iMax, T[a], kx[a], ky[a]);
			if (W->yMinSur==PML) Sum -= ff64Y(P, P->yMin, P->jMin, T[a], kx[a], ky[a]);
			if (W->yMaxSur==PML) Sum += ff64Y(P, P->yMax, P->jMax, T[a], kx[a], ky[a]);
			if (W->zMinSur==PML) Sum -= ff64Z(P, P->zMin, P->kMin, T[a], kx[a], ky[a]);
			if (W->zMaxSur==PML) Sum += ff64Z(P, P->zMax, P->kMax, T[a], kx[a], ky[a]);
			out[a] = Sum;
		} else {
			float complex Sum = 0;
			if (W->xMinSur==PML) Sum -= ff32X(P, P->xMin, P->iMin, T[a], kx[a], ky[a]);
			if (W->xMaxSur==PML) Sum += ff32X(P, P->xMax, P->iMax, T[a], kx[a], ky[a]);
			if (W->yMinSur==PML) Sum -= ff32Y(P, P->yMin, P->jMin, T[a], kx[a], ky[a]);
			if (W->yMaxSur==PML) Sum += ff32Y(P, P->yMax, P->jMax, T[a], kx[a], ky[a]);
			if (W->zMinSur==PML) Sum -= ff32Z(P, P->zMin, P->kMin, T[a], kx[a], ky[a]);
			if (W->zMaxSur==PML) Sum += ff32Z(P, P->zMax, P->kMax, T[a], kx[a], ky[a]);
			out[a] = Sum;
		}
	}
}


/* --- backend hooks: the oracle steps the host arrays themselves --- */

void alis_be_world_created(world W) { (void)W; }
void alis_be_world_deleted(world W)
{
	for (HalfState **pp = &halfStates; *pp; pp = &(*pp)->next)
		if ((*pp)->W == W) {
			HalfState *h = *pp;
			*pp = h->next;
			for (int f = 0; f < 2; f++) for (int q = 0; q < 2; q++) free(h->M[f][q]);
			free(h);
			break;
		}
}
void alis_be_objects_changed(world W) { (void)W; }
void alis_be_sources_changed(world W) { (void)W; }
void alis_be_world_reset(world W) { halfForget(W); }
void alis_be_sync_world(world W) { (void)W; }
void alis_be_phaser_created(phaser P) { (void)P; }
void alis_be_phaser_deleted(phaser P) { (void)P; }
void alis_be_sync_phaser(phaser P) { (void)P; }
int alis_be_phaser_flux(phaser P, float face[6]) { (void)P; (void)face; return 0; }
int alis_be_plane_flux(world W, int axis, int pos, int uLo, int uHi, int vLo, int vHi, float *out)
{
	(void)W, (void)axis, (void)pos, (void)uLo, (void)uHi, (void)vLo, (void)vHi, (void)out;
	return 0;
}
void alis_be_sync_phasers_of(world W)
{
	/* FP64 mode: the double sums rounded into the face arrays */
	(void)W;
	for (Shadow *s = shadows; s; s = s->next)
		for (int i = s->i0; i < s->i0 + s->ni; i++)
			for (int j = s->j0; j < s->j0 + s->nj; j++) for (int k = s->k0; k < s->k0 + s->nk; k++)
				s->A[i][j][k] = (float complex)s->v[((size_t)(i - s->i0) * s->nj + (j - s->j0)) * s->nk + (k - s->k0)];
}
int alis_be_sync_near(world W, int i, int j, int k) { (void)W, (void)i, (void)j, (void)k; return 0; }
int alis_be_sync_box(world W, int i0, int i1, int j0, int j1, int k0, int k1)
{
	(void)W, (void)i0, (void)i1, (void)j0, (void)j1, (void)k0, (void)k1;
	return 0;
}
void alis_be_hold_sync(world W) { (void)W; }
int alis_be_object_absorption(world W, int n, float *out) { (void)W, (void)n, (void)out; return 0; }
void alis_be_world_streams(world W) { (void)W; }
void *alis_be_slice_dft_begin(world W, const int b[6]) { (void)W, (void)b; return NULL; }
int alis_be_slice_dft_add(void *h, world W, field *f, float re, float im) { (void)h, (void)W, (void)f, (void)re, (void)im; return 0; }
int alis_be_slice_dft_read(void *h, float *F, float *G) { (void)h, (void)F, (void)G; return 0; }
void alis_be_slice_dft_end(void *h) { (void)h; }
void *alis_be_vox_begin(world W, object *O, int N) { (void)W, (void)O, (void)N; return NULL; }
int alis_be_vox_bounds(void *v, int N, int *box) { (void)v, (void)N, (void)box; return 0; }
int alis_be_vox_fill(void *v, int o, const int *b, float *fx, float *fy, float *fz) { (void)v, (void)o, (void)b, (void)fx, (void)fy, (void)fz; return 0; }
int alis_be_vox_fill_edge(void *v, int o, int axis, int n, int u0, int u1, int v0, int v1, float *out)
{ (void)v, (void)o, (void)axis, (void)n, (void)u0, (void)u1, (void)v0, (void)v1, (void)out; return 0; }
void alis_be_vox_end(void *v) { (void)v; }
/* --- second-order coupling (reference src/update.c:343-411) ---
 * term by term over the box of dispersive object n (less its last plane
 * on every axis): E_a += 2 Alt d C_a fill_a (G1 G2), the pump components
 * averaged onto the a-grid with 0.25 x a 4-cell sum where they sit
 * elsewhere (a double product, as the reference's 0.25 literal makes it) */
#define PAT(G, c, i, j, k) ((G)[c][i][j][k])
static double pumpOn(float ***G[3], int c, int a, int i, int j, int k, int *isD)
{
	*isD = c != a;
	if (c == a) return PAT(G, c, i, j, k);
	if (a == 0 && c == 1) return 0.25 * (PAT(G,1,i,j,k) + PAT(G,1,i-1,j,k) + PAT(G,1,i,j+1,k) + PAT(G,1,i-1,j+1,k));
	if (a == 0 && c == 2) return 0.25 * (PAT(G,2,i,j,k) + PAT(G,2,i-1,j,k) + PAT(G,2,i,j,k+1) + PAT(G,2,i-1,j,k+1));
	if (a == 1 && c == 2) return 0.25 * (PAT(G,2,i,j,k) + PAT(G,2,i,j-1,k) + PAT(G,2,i,j,k+1) + PAT(G,2,i,j-1,k+1));
	if (a == 1 && c == 0) return 0.25 * (PAT(G,0,i,j,k) + PAT(G,0,i,j-1,k) + PAT(G,0,i+1,j,k) + PAT(G,0,i+1,j-1,k));
	if (a == 2 && c == 0) return 0.25 * (PAT(G,0,i,j,k) + PAT(G,0,i,j,k-1) + PAT(G,0,i+1,j,k) + PAT(G,0,i+1,j,k-1));
	return 0.25 * (PAT(G,1,i,j,k) + PAT(G,1,i,j,k-1) + PAT(G,1,i,j+1,k) + PAT(G,1,i,j+1,k-1));
}

static void couple(coeffs *C, vfield F, vfield G1, vfield G2, int n, float Alt)
{
	static const int T[9][3] = {{0,0,0},{1,1,1},{2,2,2},{3,1,2},{3,2,1},{4,2,0},{4,0,2},{5,0,1},{5,1,0}};
	float ***f[3] = { F.x, F.y, F.z }, ***g1[3] = { G1.x, G1.y, G1.z }, ***g2[3] = { G2.x, G2.y, G2.z };
	float ***cm[3] = { C->x, C->y, C->z }, ****fill[3] = { C->Jx, C->Jy, C->Jz };
	for (int a = 0; a < 3; a++)
		for (int q = 0; q < 9; q++) {
			float d = C->M[n].d[a][T[q][0]];
			if (!d) continue;
			for (int i = C->iMin[n]; i <= C->iMax[n]-1; i++) for (int j = C->jMin[n]; j <= C->jMax[n]-1; j++)
				for (int k = C->kMin[n]; k <= C->kMax[n]-1; k++) {
					int d1, d2;
					double v1 = pumpOn(g1, T[q][1], a, i, j, k, &d1), v2 = pumpOn(g2, T[q][2], a, i, j, k, &d2);
					float lead = 2 * Alt * d * cm[a][i][j][k] * fill[a][n][i][j][k];
					if (!d1 && !d2) f[a][i][j][k] += lead * ((float)v1 * (float)v2);
					else f[a][i][j][k] += lead * (v1 * v2);
				}
		}
}

void alis_be_nonlinear(world WS, world WP1, world WP2, float Alt)
{
	for (int n = 0; n < WS->CE->N; n++)
		for (int m = 0; m <= WS->complexField; m++) couple(WS->CE, WS->E[m], WP1->E[m], WP2->E[m], n, Alt);
}

void alis_be_sync_all(void) {}
void alis_be_batch(int begin) { (void)begin; }
