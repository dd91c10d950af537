/*
 * fields.c -- pointwise derived quantities, float F(world, i, j, k).
 *
 * The observer-side field functions of the reference src/fields.c: Yee
 * components averaged to the cell centre, energy densities, Poynting
 * vector, currents, Maxwell stress, forces, effective permittivity and
 * the incident / scattered split of TFSF runs.  A symmetry plane at
 * index 0 (xMinSur == SYM etc.) is handled by mirroring negative
 * indices with the parity held in W->cosk*.  They read the host mirrors,
 * which each call refreshes if the device is ahead.  Function identity
 * matters: sources compare F == Ex etc.
 */
#include "engine.h"

int alis_needs_currents(matter M);

/* mirror a negative index across a symmetry plane: idx -> -idx (or
 * 1-idx on the staggered axis) and multiply the parity factor */
#define MIR(W, a, v, s, par) if ((v) < 0 && W->a##MinSur == SYM) (v) = (s) - (v), p *= (par)
#define MIRN(W, a, v, s) if ((v) < 0 && W->a##MinSur == SYM) (v) = (s) - (v)

/* real part of the pole susceptibility and its frequency derivative
 * (reference src/fields.c:17-35) */
static float poleRe(matter M, float w, int p)
{
	if (M.P[p].f || M.P[p].g)
		return 0.5
			*((M.P[p].f * M.P[p].w - M.P[p].g * M.P[p].r + I * M.P[p].g * M.P[p].w) / (M.P[p].w + w + I * M.P[p].r)
			+ (M.P[p].f * M.P[p].w - M.P[p].g * M.P[p].r - I * M.P[p].g * M.P[p].w) / (M.P[p].w - w - I * M.P[p].r));
	if (M.P[p].w) return - sq(M.P[p].w) / (sq(w) + I * w * M.P[p].r);
	return 0;
}

static float dpoleRe(matter M, float w, int p)
{
	if (M.P[p].f || M.P[p].g)
		return 0.5
			*((M.P[p].f * M.P[p].w - M.P[p].g * M.P[p].r + I * M.P[p].g * M.P[p].w) / sq(M.P[p].w - w - I * M.P[p].r)
			- (M.P[p].f * M.P[p].w - M.P[p].g * M.P[p].r - I * M.P[p].g * M.P[p].w) / sq(M.P[p].w + w + I * M.P[p].r));
	if (M.P[p].w) return (2 * w + I * M.P[p].r) * sq(M.P[p].w) / sq(sq(w) + I * w * M.P[p].r);
	return 0;
}


/* --- effective permittivity and index (reference src/fields.c:40-125) --- */

/* energy-weighted permittivity of axis a at the source frequency W->f */
static float effEps(world W, int a, int i, int j, int k)
{
	coeffs *C = W->CE;
	float ***map = a==0 ? C->x : a==1 ? C->y : C->z;
	float ****fill = a==0 ? C->Jx : a==1 ? C->Jy : C->Jz;
	float *cond = a==0 ? C->ax : a==1 ? C->ay : C->az;
	float f = 1 / map[i][j][k];
	for (int n = 0, o = 0; n < C->N; n++, o++) {
		while (!alis_needs_currents(C->M[o])) o++;
		if (C->iMin[n]<=i && i<=C->iMax[n] && C->jMin[n]<=j && j<=C->jMax[n] && C->kMin[n]<=k && k<=C->kMax[n]) {
			matter M = C->M[o];
			int m = M.e.y || M.e.z ? 1 : 0;
			float e = a==0 ? (M.e.x ? M.e.x : M.e.x) : a==1 ? (M.e.y ? M.e.y : M.e.x) : (M.e.z ? M.e.z : M.e.x);
			f -= cond[n] * e * fill[n][i][j][k];
			for (int p = 0; p < MAXPOLES; p += 1+2*m)
				f += (poleRe(M, W->f*W->eV, p+a*m) + W->f*W->eV * dpoleRe(M, W->f*W->eV, p+a*m)) * fill[n][i][j][k];
		}
	}
	return f;
}

float raweEffx(world W, int i, int j, int k)
{
	ALIS_SYNC(W);
	if (!W->CE->x) return 1;
	MIRN(W, x, i, 1); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	return effEps(W, 0, i, j, k);
}

float raweEffy(world W, int i, int j, int k)
{
	ALIS_SYNC(W);
	if (!W->CE->y) return 1;
	MIRN(W, x, i, 0); MIRN(W, y, j, 1); MIRN(W, z, k, 0);
	return effEps(W, 1, i, j, k);
}

float raweEffz(world W, int i, int j, int k)
{
	ALIS_SYNC(W);
	if (!W->CE->z) return 1;
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 1);
	return effEps(W, 2, i, j, k);
}

float eEff(world W, int i, int j, int k)
{
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	return (raweEffx(W,i,j,k) + raweEffx(W,i+1,j,k) + raweEffy(W,i,j,k) + raweEffy(W,i,j+1,k) + raweEffz(W,i,j,k) + raweEffz(W,i,j,k+1)) / 6;
}

float RI(world W, int i, int j, int k)
{
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	return sqrtf(fabsf(eEff(W,i,j,k)));
}

float ContourRI(world W, int i, int j, int k)
{
	float x, y, z;
	i = W->xtoi(W, i*W->dx), j = W->ytoj(W, j*W->dy), k = W->ztok(W, k*W->dz);
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	x = log10f(1+sqrtf(fabsf(raweEffx(W, i+1, j, k)))) - log10f(1+sqrtf(fabsf(raweEffx(W, i, j, k))));
	y = log10f(1+sqrtf(fabsf(raweEffy(W, i, j+1, k)))) - log10f(1+sqrtf(fabsf(raweEffy(W, i, j, k))));
	z = log10f(1+sqrtf(fabsf(raweEffz(W, i, j, k+1)))) - log10f(1+sqrtf(fabsf(raweEffz(W, i, j, k))));
	return sqrt(x*x+y*y+z*z);
}

float LogRI(world W, int i, int j, int k) { return log10f(RI(W, i, j, k)); }
float Contour(world W, int i, int j, int k) { return ContourRI(W, i, j, k) ? 1 : 0; }


/* --- E and H (reference src/fields.c:130-291) ---
 * Parities on a symmetry plane: E tangential to the plane flips with
 * -cos, the normal component keeps cos; H the opposite. */

#define RAW(name, G, c, sx, sy, sz) \
float name(world W, int i, int j, int k) { \
	float p = 1; \
	ALIS_SYNC(W); \
	MIR(W, x, i, 0, (sx)*W->coskx); MIR(W, y, j, 0, (sy)*W->cosky); MIR(W, z, k, 0, (sz)*W->coskz); \
	return p * W->G->c[i][j][k]; \
}
RAW(rawEx, E, x,  1, -1, -1)
RAW(rawEy, E, y, -1,  1, -1)
RAW(rawEz, E, z, -1, -1,  1)
RAW(rawHx, H, x, -1,  1,  1)
RAW(rawHy, H, y,  1, -1,  1)
RAW(rawHz, H, z,  1,  1, -1)

/* E averaged over its two samples along its own axis */
#define EAVG(name, m, c, di, dj, dk, sx, sy, sz) \
float name(world W, int i, int j, int k) { \
	float p = 0.5; \
	ALIS_SYNC(W); \
	if ((m) && !W->complexField) return 0; \
	MIR(W, x, i, 0, (sx)*W->coskx); MIR(W, y, j, 0, (sy)*W->cosky); MIR(W, z, k, 0, (sz)*W->coskz); \
	return p * (W->E[m].c[i][j][k] + W->E[m].c[i+(di)][j+(dj)][k+(dk)]); \
}
EAVG(Ex, 0, x, 1, 0, 0,  1, -1, -1)
EAVG(Ey, 0, y, 0, 1, 0, -1,  1, -1)
EAVG(Ez, 0, z, 0, 0, 1, -1, -1,  1)
EAVG(iEx, 1, x, 1, 0, 0,  1, -1, -1)
EAVG(iEy, 1, y, 0, 1, 0, -1,  1, -1)
EAVG(iEz, 1, z, 0, 0, 1, -1, -1,  1)

/* H averaged over the four samples around the cell centre line */
#define HAVG(name, m, c, a1, b1, c1, a2, b2, c2, sx, sy, sz) \
float name(world W, int i, int j, int k) { \
	float p = 0.25; \
	ALIS_SYNC(W); \
	if ((m) && !W->complexField) return 0; \
	MIR(W, x, i, 0, (sx)*W->coskx); MIR(W, y, j, 0, (sy)*W->cosky); MIR(W, z, k, 0, (sz)*W->coskz); \
	return p * (W->H[m].c[i][j][k] + W->H[m].c[i+(a1)][j+(b1)][k+(c1)] + W->H[m].c[i+(a2)][j+(b2)][k+(c2)] + W->H[m].c[i+(a1)+(a2)][j+(b1)+(b2)][k+(c1)+(c2)]); \
}
HAVG(Hx, 0, x, 0, 1, 0, 0, 0, 1, -1,  1,  1)
HAVG(Hy, 0, y, 0, 0, 1, 1, 0, 0,  1, -1,  1)
HAVG(Hz, 0, z, 1, 0, 0, 0, 1, 0,  1,  1, -1)
HAVG(iHx, 1, x, 0, 1, 0, 0, 0, 1, -1,  1,  1)
HAVG(iHy, 1, y, 0, 0, 1, 1, 0, 0,  1, -1,  1)
HAVG(iHz, 1, z, 1, 0, 0, 0, 1, 0,  1,  1, -1)


/* --- current density (reference src/fields.c:296-376) ---
 * Polarisation plus conduction current that the update subtracts, read
 * back from the curl residual (1 - C) dt curl H, the ADE currents and the
 * soft sources acting on E in this half step. */

static float currentAt(world W, int a, int i, int j, int k)
{
	float f = 0;
	coeffs *C = W->CE;
	float ***map = a==0 ? C->x : a==1 ? C->y : C->z;
	if (map) {
		vfield *H = W->H;
		if (a == 0)
			f += (C->dtdz[k] * (H->y[i][j][k] - H->y[i][j][k+1]) + C->dtdy[j] * (H->z[i][j+1][k] - H->z[i][j][k])) * (1 - C->x[i][j][k]);
		else if (a == 1)
			f += (C->dtdx[i] * (H->z[i][j][k] - H->z[i+1][j][k]) + C->dtdz[k] * (H->x[i][j][k+1] - H->x[i][j][k])) * (1 - C->y[i][j][k]);
		else
			f += (C->dtdy[j] * (H->x[i][j][k] - H->x[i][j+1][k]) + C->dtdx[i] * (H->y[i+1][j][k] - H->y[i][j][k])) * (1 - C->z[i][j][k]);
		for (int n = 0; n < C->N; n++) {
			int in = C->iMin[n]<=i && (a==0 ? i<=C->iMax[n] : i<C->iMax[n])
			      && C->jMin[n]<=j && (a==1 ? j<=C->jMax[n] : j<C->jMax[n])
			      && C->kMin[n]<=k && (a==2 ? k<=C->kMax[n] : k<C->kMax[n]);
			if (!in) continue;
			float *ax = a==0 ? C->ax : a==1 ? C->ay : C->az;
			float ****fill = a==0 ? C->Jx : a==1 ? C->Jy : C->Jz;
			float ***e = a==0 ? W->E->x : a==1 ? W->E->y : W->E->z;
			float *****J = a==0 ? W->E->Jx : a==1 ? W->E->Jy : W->E->Jz;
			if (ax[n]) f += 2 * fill[n][i][j][k] * e[i][j][k] / (1 + 1 / ax[n]);
			for (int p = 0; p < C->NK[n]; p++) if (J[n][p]) f += J[n][p][i][j][k];
		}
	}
	float ***tgt = a==0 ? W->E->x : a==1 ? W->E->y : W->E->z;
	for (source S = W->SE; S; S = S->S)
		if (S->F == tgt && W->n < S->N && S->iMin <= i && i <= S->iMax && S->jMin <= j && j <= S->jMax && S->kMin <= k && k <= S->kMax)
			f -= (S->Amplitude ? S->Amplitude[i][j][k] : S->amplitude) * S->waveForm(W, S, W->H->t, S->Phase ? S->Phase[i][j][k] : S->phase);
	return f;
}

float rawJx(world W, int i, int j, int k)
{
	float p = 1;
	ALIS_SYNC(W);
	MIR(W, x, i, 1, W->coskx); MIR(W, y, j, 0, -W->cosky); MIR(W, z, k, 0, -W->coskz);
	return p * currentAt(W, 0, i, j, k) / W->dt;
}

float rawJy(world W, int i, int j, int k)
{
	float p = 1;
	ALIS_SYNC(W);
	MIR(W, x, i, 0, -W->coskx); MIR(W, y, j, 1, W->cosky); MIR(W, z, k, 0, -W->coskz);
	return p * currentAt(W, 1, i, j, k) / W->dt;
}

float rawJz(world W, int i, int j, int k)
{
	float p = 1;
	ALIS_SYNC(W);
	MIR(W, x, i, 0, -W->coskx); MIR(W, y, j, 0, -W->cosky); MIR(W, z, k, 1, W->coskz);
	return p * currentAt(W, 2, i, j, k) / W->dt;
}

float Jx(world W, int i, int j, int k) { return 0.5 * (rawJx(W,i,j,k) + rawJx(W,i+1,j,k)); }
float Jy(world W, int i, int j, int k) { return 0.5 * (rawJy(W,i,j,k) + rawJy(W,i,j+1,k)); }
float Jz(world W, int i, int j, int k) { return 0.5 * (rawJz(W,i,j,k) + rawJz(W,i,j,k+1)); }


/* --- products of E, J and H (reference src/fields.c:381-550) --- */

/* A[i] (H at i + H at i+o) + A[i+d] (H at i+d + H at i+d+o) / 4, with
 * fixed symmetry signs (the product's parity does not depend on cos) */
#define EH(name, A, c, da, db, dc, Hc, oa, ob, oc, sx, sy, sz) \
float name(world W, int i, int j, int k) { \
	float p = 0.25; \
	ALIS_SYNC(W); \
	MIR(W, x, i, 0, sx); MIR(W, y, j, 0, sy); MIR(W, z, k, 0, sz); \
	return p * (A(W, c, i, j, k) * (W->H->Hc[i][j][k] + W->H->Hc[i+(oa)][j+(ob)][k+(oc)]) \
	          + A(W, c, i+(da), j+(db), k+(dc)) * (W->H->Hc[i+(da)][j+(db)][k+(dc)] + W->H->Hc[i+(da)+(oa)][j+(db)+(ob)][k+(dc)+(oc)])); \
}
#define EFIELD(W, c, i, j, k) (W->E->c[i][j][k])
#define JFIELD(W, c, i, j, k) (c == 0 ? rawJx(W, i, j, k) : c == 1 ? rawJy(W, i, j, k) : rawJz(W, i, j, k))
static const int cx = 0, cy = 1, cz = 2;
EH(ExHy, EFIELD, x, 1, 0, 0, y, 0, 0, 1,  1,  1, -1)
EH(ExHz, EFIELD, x, 1, 0, 0, z, 0, 1, 0,  1, -1,  1)
EH(EyHz, EFIELD, y, 0, 1, 0, z, 1, 0, 0, -1,  1,  1)
EH(EyHx, EFIELD, y, 0, 1, 0, x, 0, 0, 1,  1,  1, -1)
EH(EzHx, EFIELD, z, 0, 0, 1, x, 0, 1, 0,  1, -1,  1)
EH(EzHy, EFIELD, z, 0, 0, 1, y, 1, 0, 0, -1,  1,  1)
EH(JxHy, JFIELD, cx, 1, 0, 0, y, 0, 0, 1,  1,  1, -1)
EH(JxHz, JFIELD, cx, 1, 0, 0, z, 0, 1, 0,  1, -1,  1)
EH(JyHz, JFIELD, cy, 0, 1, 0, z, 1, 0, 0, -1,  1,  1)
EH(JyHx, JFIELD, cy, 0, 1, 0, x, 0, 0, 1,  1,  1, -1)
EH(JzHx, JFIELD, cz, 0, 0, 1, x, 0, 1, 0,  1, -1,  1)
EH(JzHy, JFIELD, cz, 0, 0, 1, y, 1, 0, 0, -1,  1,  1)

float JE(world W, int i, int j, int k)
{
	float f = 0;
	ALIS_SYNC(W);
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	f += W->E->x[i][j][k] * rawJx(W,i,j,k) + W->E->x[i+1][j][k] * rawJx(W,i+1,j,k);
	f += W->E->y[i][j][k] * rawJy(W,i,j,k) + W->E->y[i][j+1][k] * rawJy(W,i,j+1,k);
	f += W->E->z[i][j][k] * rawJz(W,i,j,k) + W->E->z[i][j][k+1] * rawJz(W,i,j,k+1);
	return 0.5 * f;
}

/* sums of squares of the E samples and of the H samples of a cell */
static float sumE2(world W, int c, int i, int j, int k)
{
	vfield *E = W->E;
	if (c == 0) return sq(E->x[i][j][k]) + sq(E->x[i+1][j][k]);
	if (c == 1) return sq(E->y[i][j][k]) + sq(E->y[i][j+1][k]);
	return sq(E->z[i][j][k]) + sq(E->z[i][j][k+1]);
}

static float sumH2(world W, int c, int i, int j, int k)
{
	vfield *H = W->H;
	if (c == 0) return sq(H->x[i][j][k]) + sq(H->x[i][j+1][k]) + sq(H->x[i][j][k+1]) + sq(H->x[i][j+1][k+1]);
	if (c == 1) return sq(H->y[i][j][k]) + sq(H->y[i][j][k+1]) + sq(H->y[i+1][j][k]) + sq(H->y[i+1][j][k+1]);
	return sq(H->z[i][j][k]) + sq(H->z[i+1][j][k]) + sq(H->z[i][j+1][k]) + sq(H->z[i+1][j+1][k]);
}

float EE(world W, int i, int j, int k)
{
	float f = 0;
	ALIS_SYNC(W);
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	f += sumE2(W, 0, i, j, k);
	f += sumE2(W, 1, i, j, k);
	f += sumE2(W, 2, i, j, k);
	return 0.5 * f;
}

float UE(world W, int i, int j, int k)
{
	float f = 0;
	ALIS_SYNC(W);
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	vfield *E = W->E;
	f += sq(E->x[i][j][k]) * raweEffx(W, i, j, k) + sq(E->x[i+1][j][k]) * raweEffx(W, i+1, j, k);
	f += sq(E->y[i][j][k]) * raweEffy(W, i, j, k) + sq(E->y[i][j+1][k]) * raweEffy(W, i, j+1, k);
	f += sq(E->z[i][j][k]) * raweEffz(W, i, j, k) + sq(E->z[i][j][k+1]) * raweEffz(W, i, j, k+1);
	return 0.25 * f;
}

float HH(world W, int i, int j, int k)
{
	float f = 0;
	ALIS_SYNC(W);
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	f += sumH2(W, 0, i, j, k);
	f += sumH2(W, 1, i, j, k);
	f += sumH2(W, 2, i, j, k);
	return 0.25 * f;
}

float Sx(world W, int i, int j, int k) { return EyHz(W,i,j,k) - EzHy(W,i,j,k); }
float Sy(world W, int i, int j, int k) { return EzHx(W,i,j,k) - ExHz(W,i,j,k); }
float Sz(world W, int i, int j, int k) { return ExHy(W,i,j,k) - EyHx(W,i,j,k); }
float UH(world W, int i, int j, int k) { return 0.5*HH(W, i, j, k); }
float U(world W, int i, int j, int k) { return UE(W, i, j, k)+UH(W, i, j, k); }
float LogJE(world W, int i, int j, int k) { return log10f(JE(W, i, j, k)); }
float LogEE(world W, int i, int j, int k) { return log10f(EE(W, i, j, k)); }
float LogUE(world W, int i, int j, int k) { return log10f(UE(W, i, j, k)); }
float LogHH(world W, int i, int j, int k) { return log10f(HH(W, i, j, k)); }
float LogUH(world W, int i, int j, int k) { return log10f(HH(W, i, j, k)); }
float LogU(world W, int i, int j, int k) { return log10f(U(W, i, j, k)); }

float DivE(world W, int i, int j, int k)
{
	float p = 1;
	ALIS_SYNC(W);
	MIR(W, x, i, 0, -W->coskx); MIR(W, y, j, 0, -W->cosky); MIR(W, z, k, 0, -W->coskz);
	vfield *E = W->E;
	return ((E->x[i+1][j][k] - E->x[i][j][k]) * W->CE->dtdx[i] +
	        (E->y[i][j+1][k] - E->y[i][j][k]) * W->CE->dtdy[j] +
	        (E->z[i][j][k+1] - E->z[i][j][k]) * W->CE->dtdz[k]) * p / W->dt;
}


/* --- Maxwell stress (reference src/fields.c:563-681) --- */

/* diagonal: (+own -others) of H squares, halved, plus the same of E */
static float stressDiag(world W, int a, int i, int j, int k)
{
	float f = 0;
	ALIS_SYNC(W);
	MIRN(W, x, i, 0); MIRN(W, y, j, 0); MIRN(W, z, k, 0);
	for (int c = 0; c < 3; c++) { if (c == a) f += sumH2(W, c, i, j, k); else f -= sumH2(W, c, i, j, k); }
	f *= 0.5;
	for (int c = 0; c < 3; c++) { if (c == a) f += sumE2(W, c, i, j, k); else f -= sumE2(W, c, i, j, k); }
	return 0.25 * f;
}
float Txx(world W, int i, int j, int k) { return stressDiag(W, 0, i, j, k); }
float Tyy(world W, int i, int j, int k) { return stressDiag(W, 1, i, j, k); }
float Tzz(world W, int i, int j, int k) { return stressDiag(W, 2, i, j, k); }

/* pair sums of the E and H samples of a cell */
static float pairE(world W, int c, int i, int j, int k)
{
	vfield *E = W->E;
	if (c == 0) return E->x[i][j][k] + E->x[i+1][j][k];
	if (c == 1) return E->y[i][j][k] + E->y[i][j+1][k];
	return E->z[i][j][k] + E->z[i][j][k+1];
}

static float quadH(world W, int c, int i, int j, int k)
{
	vfield *H = W->H;
	if (c == 0) return H->x[i][j][k] + H->x[i][j+1][k] + H->x[i][j][k+1] + H->x[i][j+1][k+1];
	if (c == 1) return H->y[i][j][k] + H->y[i][j][k+1] + H->y[i+1][j][k] + H->y[i+1][j][k+1];
	return H->z[i][j][k] + H->z[i+1][j][k] + H->z[i][j+1][k] + H->z[i+1][j+1][k];
}

/* off-diagonal T_ab: components (a, b) in the reference's operand order */
#define TOFF(name, a, b, sx, sy, sz) \
float name(world W, int i, int j, int k) { \
	float f = 0, p = 0.25; \
	ALIS_SYNC(W); \
	MIR(W, x, i, 0, sx); MIR(W, y, j, 0, sy); MIR(W, z, k, 0, sz); \
	f += pairE(W, a, i, j, k) * pairE(W, b, i, j, k); \
	f += quadH(W, a, i, j, k) * quadH(W, b, i, j, k) * 0.25; \
	return p * f; \
}
TOFF(Txy, 0, 1, -1, -1,  1)
TOFF(Tyx, 0, 1, -1, -1,  1)
TOFF(Txz, 2, 0, -1,  1, -1)
TOFF(Tzx, 2, 0, -1,  1, -1)
TOFF(Tyz, 1, 2,  1, -1, -1)
TOFF(Tzy, 1, 2,  1, -1, -1)

float Fx(world W, int i, int j, int k) { return DivE(W, i, j, k) * Ex(W, i, j, k) + (JyHz(W, i, j, k) - JzHy(W, i, j, k)); }
float Fy(world W, int i, int j, int k) { return DivE(W, i, j, k) * Ey(W, i, j, k) + (JzHx(W, i, j, k) - JxHz(W, i, j, k)); }
float Fz(world W, int i, int j, int k) { return DivE(W, i, j, k) * Ez(W, i, j, k) + (JxHy(W, i, j, k) - JyHx(W, i, j, k)); }


/* --- incident and scattered fields of TFSF runs (reference src/fields.c:690-791) --- */

#define SOE(name, c, di, dj, dk, sx, sy, sz) \
float name(world W, int i, int j, int k) { \
	float f = 0, p = 0.5; \
	ALIS_SYNC(W); \
	MIR(W, x, i, 0, (sx)*W->coskx); MIR(W, y, j, 0, (sy)*W->cosky); MIR(W, z, k, 0, (sz)*W->coskz); \
	for (tfsf S = W->S; S; S = S->S) { ALIS_SYNC(S->W); f += S->W->E->c[i][j][k] + S->W->E->c[i+(di)][j+(dj)][k+(dk)]; } \
	return p * f; \
}
SOE(SoEx, x, 1, 0, 0,  1, -1, -1)
SOE(SoEy, y, 0, 1, 0, -1,  1, -1)
SOE(SoEz, z, 0, 0, 1, -1, -1,  1)
float SoEE(world W, int i, int j, int k) { return sq(SoEx(W,i,j,k))+sq(SoEy(W,i,j,k))+sq(SoEz(W,i,j,k)); }

/* total minus incident inside the TFSF box */
float ScEx(world W, int i, int j, int k)
{
	float f, p = 0.5;
	ALIS_SYNC(W);
	MIR(W, x, i, 0, W->coskx); MIR(W, y, j, 0, -W->cosky); MIR(W, z, k, 0, -W->coskz);
	f = W->E->x[i][j][k] + W->E->x[i+1][j][k];
	for (tfsf S = W->S; S; S = S->S) {
		ALIS_SYNC(S->W);
		if (S->jMin <= j && j <= S->jMax && S->kMin <= k && k <= S->kMax) {
			if (S->iMIN <= i && i <= S->iMAX) f -= S->W->E->x[i][j][k];
			if (S->iMIN <= i+1 && i+1 <= S->iMAX) f -= S->W->E->x[i+1][j][k];
		}
	}
	return p * f;
}

float ScEy(world W, int i, int j, int k)
{
	float f, p = 0.5;
	ALIS_SYNC(W);
	MIR(W, x, i, 0, -W->coskx); MIR(W, y, j, 0, W->cosky); MIR(W, z, k, 0, -W->coskz);
	f = W->E->y[i][j][k] + W->E->y[i][j+1][k];
	for (tfsf S = W->S; S; S = S->S) {
		ALIS_SYNC(S->W);
		if (S->iMin <= i && i <= S->iMax && S->kMin <= k && k <= S->kMax) {
			if (S->jMIN <= j && j <= S->jMAX) f -= S->W->E->y[i][j][k];
			if (S->jMIN <= j+1 && j+1 <= S->jMAX) f -= S->W->E->y[i][j+1][k];
		}
	}
	return p * f;
}

float ScEz(world W, int i, int j, int k)
{
	float f, p = 0.5;
	ALIS_SYNC(W);
	MIR(W, x, i, 0, -W->coskx); MIR(W, y, j, 0, -W->cosky); MIR(W, z, k, 0, W->coskz);
	f = W->E->z[i][j][k] + W->E->z[i][j][k+1];
	for (tfsf S = W->S; S; S = S->S) {
		ALIS_SYNC(S->W);
		if (S->iMin <= i && i <= S->iMax && S->jMin <= j && j <= S->jMax) {
			if (S->kMIN <= k && k <= S->kMAX) f -= S->W->E->z[i][j][k];
			if (S->kMIN <= k+1 && k+1 <= S->kMAX) f -= S->W->E->z[i][j][k+1];
		}
	}
	return p * f;
}

float ScEE(world W, int i, int j, int k) { return sq(ScEx(W,i,j,k))+sq(ScEy(W,i,j,k))+sq(ScEz(W,i,j,k)); }
