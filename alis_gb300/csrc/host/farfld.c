/*
 * farfld.c -- near-to-far-field projection of phaser data.
 *
 * Host half of the reference src/farfld.c: projection maps, the layered
 * background seen by the phaser column, the 1-D reciprocity test field
 * (Ppol/Spol transfer recursion along z), angle handling, lattice
 * factors and the image/flux drivers.  The face sums, which carry the
 * cost (every face cell times every direction), are computed by the
 * backend: in FP64 on the GPU, in the reference's FP32 by the oracle.
 * farFieldProfile/Theta/Phi/Flux hand the backend whole batches of
 * directions at once.
 */
#include <sys/stat.h>
#include <string.h>
#include "engine.h"

/* --- projection maps (reference src/farfld.c:14-41) ---
 * Pixel (x, y) of an X x Y image to a direction (theta, phi) in degrees;
 * INF marks a pixel outside the map.  The arithmetic (double ratios,
 * float square root and arc tangent) is the reference's, so the same
 * pixel gives the same float angles. */

void CylindericalMap(int x, int y, int X, int Y, float angle[2])
{
	angle[0] = 180.0 - 180.0 * y / Y;
	angle[1] = 360.0 * x / X;
}

/* one hemisphere seen from its pole: the polar angle grows with the
 * distance from the image centre, 90 degrees at the inscribed circle */
static void hemisphereMap(int x, int y, int X, int Y, int south, float angle[2])
{
	const double u = x / (X - 1.0) - 0.5, v = y / (Y - 1.0) - 0.5;
	const float fromPole = 180 * sqrtf(u * u + v * v);
	const float polar = south ? 180 - fromPole : fromPole;
	angle[1] = 180 * atan2f(v, u) / PI;
	angle[0] = (south ? polar < 90 : polar > 90) ? INF : polar;
}

void NorthernAzimuthalMap(int x, int y, int X, int Y, float angle[2])
{
	hemisphereMap(x, y, X, Y, 0, angle);
}

void SouthernAzimuthalMap(int x, int y, int X, int Y, float angle[2])
{
	hemisphereMap(x, y, X, Y, 1, angle);
}

/* the two hemispheres side by side; a middle column of an odd width
 * belongs to both, the southern one written last */
void AzimuthalMap(int x, int y, int X, int Y, float angle[2])
{
	const int half = (X + 1) / 2;
	if (x < half) hemisphereMap(x, y, half, Y, 0, angle);
	if (x > X / 2) hemisphereMap(x - X / 2, y, half, Y, 1, angle);
}

/* direction (a, b) rotated by theta about y (reference src/farfld.c:44-52) */
static float rotateA(float theta, float a, float b)
{
	return acosf(cosf(a*PI/180)*cosf(theta*PI/180)-(sinf(a*PI/180)*cosf(b*PI/180))*sinf(theta*PI/180))*180/PI;
}

static float rotateB(float theta, float a, float b)
{
	return atan2f(sinf(a*PI/180)*sinf(b*PI/180), (sinf(a*PI/180)*cosf(b*PI/180))*cosf(theta*PI/180)+cosf(a*PI/180)*sinf(theta*PI/180))*180/PI;
}

int alis_needs_currents(matter M);

/* susceptibility of pole p at photon energy w (eV) (reference
 * src/farfld.c:63-71) */
static float complex poleResponse(matter M, float w, int p)
{
	if (M.P[p].f || M.P[p].g)
		return 0.5
			*((M.P[p].f * M.P[p].w - M.P[p].g * M.P[p].r + I * M.P[p].g * M.P[p].w) / (M.P[p].w + w + I * M.P[p].r)
			+ (M.P[p].f * M.P[p].w - M.P[p].g * M.P[p].r - I * M.P[p].g * M.P[p].w) / (M.P[p].w - w - I * M.P[p].r));
	if (M.P[p].w) return - sq(M.P[p].w) / (sq(w) + I * w * M.P[p].r);
	return -I * M.P[p].r / w;
}

/* Layer profile along z at the phaser's (iMax, jMax) column: dz tables
 * and the complex permittivity at the phaser frequency, mirrored for a
 * z symmetry plane (reference src/farfld.c:74-117). */
void alis_farfield_profile(phaser P, world W)
{
	P->kMIN = (W->zMinSur==SYM) ? -P->kMax : P->kMin;
	MALLOC(P->dE, P->kMIN, 2-P->kMIN+P->kMax);
	MALLOC(P->dH, P->kMIN, 2-P->kMIN+P->kMax);
	MALLOC(P->ex, P->kMIN, 2-P->kMIN+P->kMax);
	MALLOC(P->ez, P->kMIN, 2-P->kMIN+P->kMax);
	for (int k = P->kMin; k <= P->kMax+1; k++) {
		P->dE[k] = 1 / W->CE->dtdz[k];
		P->dH[k] = 1 / W->CH->dtdz[k];
		P->ex[k] = W->CE->x ? 1/W->CE->x[P->iMax][P->jMax][k] : 1;
		P->ez[k] = W->CE->z ? 1/W->CE->z[P->iMax][P->jMax][k] : 1;
		for (int n = 0, o = 0; n < W->CE->N; n++, o++) {
			while (!alis_needs_currents(W->CE->M[o])) o++;
			coeffs *C = W->CE;
			if (C->iMin[n]<=P->iMax && P->iMax<=C->iMax[n] && C->jMin[n]<=P->jMax && P->jMax<=C->jMax[n] && C->kMin[n]<=k && k<=C->kMax[n]) {
				matter M = C->M[o];
				int m = M.e.y || M.e.z ? 1 : 0;
				P->ex[k] += -C->ax[n] * (M.e.x ? M.e.x : M.e.x) * C->Jx[n][P->iMax][P->jMax][k];
				P->ez[k] += -C->az[n] * (M.e.z ? M.e.z : M.e.x) * C->Jz[n][P->iMax][P->jMax][k];
				for (int p = 0; p < MAXPOLES; p += 1+2*m) {
					P->ex[k] += poleResponse(M, W->eV * P->f, p+0*m) * C->Jx[n][P->iMax][P->jMax][k];
					P->ez[k] += poleResponse(M, W->eV * P->f, p+2*m) * C->Jz[n][P->iMax][P->jMax][k];
				}
			}
		}
	}
	if (W->zMinSur==SYM) for (int k = P->kMIN; k < P->kMin; k++) {
		P->dE[k] = P->dE[-k];
		P->dH[k] = P->dH[1-k];
		P->ex[k] = P->ex[-k];
		P->ez[k] = P->ez[1-k];
	}
}


/* --- reciprocity test fields (reference src/farfld.c:120-245) ---
 * A unit plane wave arriving from direction (theta, phi) is propagated
 * through the discrete layer stack along z with the FDTD dispersion
 * (sin(pi f dt) factors); rows are rescaled by 1e10 whenever they grow
 * past 1e10.  T.A is the normalisation at the exit layer. */

tfield Unpol(phaser P, float theta, float phi)
{
	(void)P; (void)theta; (void)phi;
	return (tfield) {0};
}

tfield Ppol(phaser P, float theta, float phi)
{
	tfield T = {0};
	float sinth = 0, sin2th = 0, sinphi = sinf(phi*PI/180), cosphi = cosf(phi*PI/180);
	float s = sinf(PI*P->f*P->W->dt);
	MALLOC(T.Ex, P->kMIN, 2-P->kMIN+P->kMax);
	MALLOC(T.Hy, P->kMIN, 2-P->kMIN+P->kMax);
	if (theta < 90 || 270 < theta) {
		sinth = sinf(theta*PI/180) * sqrtf(crealf(P->ex[P->kMax])), sin2th = sq(sinth);
		T.Hy[P->kMIN] = -1;
		T.Ex[P->kMIN] = csqrtf((1-sin2th/P->ez[P->kMIN]) / P->ex[P->kMIN]);
		T.Ex[P->kMIN] *= cexpf(-I * casinf(sinf(PI*P->f*P->W->dt) * csqrtf(P->ex[P->kMIN]-sin2th) * P->dE[P->kMIN]));
		for (int k = P->kMIN; k <= P->kMax; k++) {
			T.Hy[k+1] = T.Hy[k] + 2 * I * sinf(PI*P->f*P->W->dt) * P->dE[k] * T.Ex[k] * P->ex[k];
			T.Ex[k+1] = T.Ex[k] + 2 * I * sinf(PI*P->f*P->W->dt) * P->dH[k+1] * T.Hy[k+1] * (1-sin2th/P->ez[k+1]);
			if (cabsf(T.Hy[k+1])>1E10) for (int kk = P->kMIN; kk <= k+1; kk++) T.Ex[kk]/=1E10, T.Hy[kk]/=1E10;
		}
		T.A = sqrtf(sqrtf(P->ex[P->kMax]));
		T.A /= cabsf(0.5*(T.Hy[P->kMax]+T.Hy[P->kMax+1]) / sqrtf(P->ex[P->kMax]) - T.Ex[P->kMax] / cosf(theta*PI/180));
	}
	if (90 < theta && theta < 270) {
		sinth = sinf(theta*PI/180) * sqrtf(crealf(P->ex[P->kMIN])), sin2th = sq(sinth);
		T.Hy[P->kMax+1] = 1;
		T.Ex[P->kMax+1] = csqrtf((1-sin2th/P->ez[P->kMax+1]) / P->ex[P->kMax+1]);
		T.Ex[P->kMax+1] *= cexpf(I * casinf(sinf(PI*P->f*P->W->dt) * csqrtf(P->ex[P->kMax+1]-sin2th) * P->dE[P->kMax+1]));
		for (int k = P->kMax; k >= P->kMIN; k--) {
			T.Ex[k] = T.Ex[k+1] - 2 * I * sinf(PI*P->f*P->W->dt) * P->dH[k+1] * T.Hy[k+1] * (1-sin2th/P->ez[k+1]);
			T.Hy[k] = T.Hy[k+1] - 2 * I * sinf(PI*P->f*P->W->dt) * P->dE[k] * T.Ex[k] * P->ex[k];
			if (cabsf(T.Hy[k+1])>1E10) for (int kk = P->kMax; kk >= k; kk--) T.Ex[kk]/=1E10, T.Hy[kk]/=1E10;
		}
		T.A = sqrtf(sqrtf(P->ex[P->kMIN]));
		T.A /= cabsf(0.5*(T.Hy[P->kMIN]+T.Hy[P->kMIN+1]) / sqrtf(P->ex[P->kMIN]) - T.Ex[P->kMIN] / cosf(theta*PI/180));
	}
	(void)s;
	if (theta) {
		MALLOC(T.Ez, P->kMIN, 2-P->kMIN+P->kMax);
		for (int k = P->kMIN; k <= P->kMax+1; k++) T.Ez[k] = T.Hy[k] * sinth/P->ez[k];
	}
	if (phi) {
		MALLOC(T.Hx, P->kMIN, 2-P->kMIN+P->kMax);
		MALLOC(T.Ey, P->kMIN, 2-P->kMIN+P->kMax);
		for (int k = P->kMIN; k <= P->kMax+1; k++) {
			T.Ey[k] = T.Ex[k] * sinphi;
			T.Ex[k] = T.Ex[k] * cosphi;
			T.Hx[k] =-T.Hy[k] * sinphi;
			T.Hy[k] = T.Hy[k] * cosphi;
		}
	}
	return T;
}

tfield Spol(phaser P, float theta, float phi)
{
	tfield T = {0};
	float sinth = 0, sin2th = 0, sinphi = sinf(phi*PI/180), cosphi = cosf(phi*PI/180);
	MALLOC(T.Hx, P->kMIN, 2-P->kMIN+P->kMax);
	MALLOC(T.Ey, P->kMIN, 2-P->kMIN+P->kMax);
	if (theta < 90 || 270 < theta) {
		sinth = sinf(theta*PI/180) * sqrtf(crealf(P->ex[P->kMax])), sin2th = sq(sinth);
		T.Hx[P->kMIN] = csqrtf(P->ex[P->kMIN] - sin2th);
		T.Ey[P->kMIN] = cexpf(-I * casinf(sinf(PI*P->f*P->W->dt) * csqrtf(P->ex[P->kMIN]-sin2th) * P->dE[P->kMIN]));
		for (int k = P->kMIN; k <= P->kMax; k++) {
			T.Hx[k+1] = T.Hx[k] - 2 * I * sinf(PI*P->f*P->W->dt) * P->dE[k] * T.Ey[k] * (P->ex[k] - sin2th);
			T.Ey[k+1] = T.Ey[k] - 2 * I * sinf(PI*P->f*P->W->dt) * P->dH[k+1] * T.Hx[k+1];
			if (cabsf(T.Hx[k+1])>1E10) for (int kk = P->kMIN; kk <= k+1; kk++) T.Ey[kk]/=1E10, T.Hx[kk]/=1E10;
		}
		T.A = sqrtf(sqrtf(P->ex[P->kMax]));
		T.A /= cabsf(T.Ey[P->kMax] + 0.5*(T.Hx[P->kMax]+T.Hx[P->kMax+1]) / (sqrtf(P->ex[P->kMax]) * cosf(theta*PI/180)));
	}
	if (90 < theta && theta < 270) {
		sinth = sinf(theta*PI/180) * sqrtf(crealf(P->ex[P->kMIN])), sin2th = sq(sinth);
		T.Ey[P->kMax+1] = cexpf(I * casinf(sinf(PI*P->f*P->W->dt) * csqrtf(P->ex[P->kMax+1]-sin2th) * P->dE[P->kMax+1]));
		T.Hx[P->kMax+1] = -csqrtf(P->ex[P->kMax+1] - sin2th);
		for (int k = P->kMax; k >= P->kMIN; k--) {
			T.Ey[k] = T.Ey[k+1] + 2 * I * sinf(PI*P->f*P->W->dt) * P->dH[k+1] * T.Hx[k+1];
			T.Hx[k] = T.Hx[k+1] + 2 * I * sinf(PI*P->f*P->W->dt) * P->dE[k] * T.Ey[k] * (P->ex[k] - sin2th);
			if (cabsf(T.Hx[k+1])>1E10) for (int kk = P->kMax; kk >= k; kk--) T.Ey[kk]/=1E10, T.Hx[kk]/=1E10;
		}
		T.A = sqrtf(sqrtf(P->ex[P->kMIN]));
		T.A /= cabsf(T.Ey[P->kMIN] + 0.5*(T.Hx[P->kMIN]+T.Hx[P->kMIN+1]) / (sqrtf(P->ex[P->kMIN]) * cosf(theta*PI/180)));
	}
	if (theta) {
		MALLOC(T.Hz, P->kMIN, 2-P->kMIN+P->kMax);
		for (int k = P->kMIN; k <= P->kMax+1; k++) T.Hz[k] = -T.Ey[k] * sinth;
	}
	if (phi) {
		MALLOC(T.Ex, P->kMIN, 2-P->kMIN+P->kMax);
		MALLOC(T.Hy, P->kMIN, 2-P->kMIN+P->kMax);
		for (int k = P->kMIN; k <= P->kMax+1; k++) {
			T.Ex[k] =-T.Ey[k] * sinphi;
			T.Ey[k] = T.Ey[k] * cosphi;
			T.Hy[k] = T.Hx[k] * sinphi;
			T.Hx[k] = T.Hx[k] * cosphi;
		}
	}
	return T;
}

static void freeTfield(phaser P, tfield T)
{
	if (T.Ex) free(&T.Ex[P->kMIN]);
	if (T.Ey) free(&T.Ey[P->kMIN]);
	if (T.Ez) free(&T.Ez[P->kMIN]);
	if (T.Hx) free(&T.Hx[P->kMIN]);
	if (T.Hy) free(&T.Hy[P->kMIN]);
	if (T.Hz) free(&T.Hz[P->kMIN]);
}


/* --- one direction, split in host prologue / backend sums / epilogue --- */

typedef struct {
	int kind;          /* 0: zero, 1: average of two directions, 2: direct */
	float theta, phi;  /* normalised angles */
	float kx, ky;
	tfield T;
} ffDir;

/* angle normalisation, the 89-91 / 269-271 degree averaging, evanescent
 * exits, test field and lateral wave numbers (reference
 * src/farfld.c:462-487) */
static void prepareDirection(phaser P, tfield pol(phaser,float,float), float theta, float phi, ffDir *d)
{
	memset(d, 0, sizeof *d);
	if (!P->dE) alis_farfield_profile(P, P->W);
	if (theta == INF || phi == INF) return;
	while (theta < 0) theta += 360;
	while (theta >= 360) theta -= 360;
	while (phi < 0) phi += 360;
	while (phi >= 360) phi -= 360;
	d->theta = theta, d->phi = phi;
	if ((89 < theta && theta < 91) || (269 < theta && theta < 271)) { d->kind = 1; return; }
	float sinth = 0;
	if (theta < 90 || 270 < theta) {
		if (cimagf(P->ex[P->kMax])) return;
		sinth = sinf(theta*PI/180) * sqrtf(crealf(P->ex[P->kMax]));
	}
	if (90 < theta && theta < 270) {
		if (cimagf(P->ex[P->kMIN])) return;
		sinth = sinf(theta*PI/180) * sqrtf(crealf(P->ex[P->kMIN]));
	}
	d->kind = 2;
	d->T = pol(P, theta, phi);
	d->kx = - 2 * PI * P->f * sinth * cosf(phi*PI/180);
	d->ky = - 2 * PI * P->f * sinth * sinf(phi*PI/180);
}

/* lattice factor and normalisation (reference src/farfld.c:502-513) */
static float complex finishDirection(phaser P, ffDir *d, float complex Sum)
{
	if (P->xNUM) {
		float complex s = 0, q = 1, p = P->expikx * cexpf(I*d->kx*(P->W->xMax-P->W->xMin));
		for (int x = 0; x < P->xNUM; x++) s += (q *= p);
		Sum *= s / P->xNUM;
	}
	if (P->yNUM) {
		float complex s = 0, q = 1, p = P->expiky * cexpf(I*d->ky*(P->W->yMax-P->W->yMin));
		for (int y = 0; y < P->yNUM; y++) s += (q *= p);
		Sum *= s / P->yNUM;
	}
	return Sum * d->T.A * P->A * P->f;
}

/* Far field of a batch of directions of one phaser.  Directions between
 * 89 and 91 (269 and 271) degrees are the mean of the 89 and 91 (269 and
 * 271) degree results, as in the reference. */
static void farFieldBatch(phaser P, tfield pol(phaser,float,float), int n, const float *theta, const float *phi, float complex *out)
{
	alis_be_sync_phaser(P);
	int cap = 2*n;
	ffDir *d = calloc(cap, sizeof *d);
	int *slot = calloc(2*n, sizeof(int));
	int m = 0;
	for (int a = 0; a < n; a++) {
		ffDir tmp;
		prepareDirection(P, pol, theta[a], phi[a], &tmp);
		if (tmp.kind == 1) {
			float t0 = tmp.theta < 180 ? 89 : 269, t1 = tmp.theta < 180 ? 91 : 271;
			prepareDirection(P, pol, t0, tmp.phi, &d[m]); slot[2*a] = m++;
			prepareDirection(P, pol, t1, tmp.phi, &d[m]); slot[2*a+1] = m++;
		} else {
			d[m] = tmp; slot[2*a] = m++; slot[2*a+1] = -1;
		}
	}
	tfield *T = calloc(m, sizeof *T);
	float *kx = calloc(m, sizeof(float)), *ky = calloc(m, sizeof(float));
	int *live = calloc(m, sizeof(int));
	int L = 0;
	for (int q = 0; q < m; q++) if (d[q].kind == 2) T[L] = d[q].T, kx[L] = d[q].kx, ky[L] = d[q].ky, live[q] = L++;
	double complex *sums = calloc(L ? L : 1, sizeof(double complex));
	if (L) alis_be_farfield_sums(P, L, T, kx, ky, sums);
	float complex *res = calloc(m, sizeof(float complex));
	for (int q = 0; q < m; q++) {
		if (d[q].kind != 2) { res[q] = 0; continue; }
		res[q] = finishDirection(P, &d[q], (float complex)sums[live[q]]);
		freeTfield(P, d[q].T);
	}
	for (int a = 0; a < n; a++) {
		if (slot[2*a+1] < 0) out[a] = res[slot[2*a]];
		else out[a] = 0.5 * (res[slot[2*a]] + res[slot[2*a+1]]);
	}
	free(d); free(slot); free(T); free(kx); free(ky); free(live); free(sums); free(res);
}

float complex farField(phaser P, tfield pol(phaser,float,float), float theta, float phi)
{
	float complex r;
	farFieldBatch(P, pol, 1, &theta, &phi, &r);
	return r;
}

float farFieldI(phaser P, tfield pol(phaser,float,float), float theta, float phi)
{
	if (pol == Unpol) return farFieldI(P, Ppol, theta, phi) + farFieldI(P, Spol, theta, phi);
	float complex f = farField(P, pol, theta, phi);
	return conjf(f) * f;
}

/* The seven intensities of one direction from its P and S amplitudes:
 * X and Y (the frame rotated by phi), circular left and right, P, S and
 * unpolarised (reference src/farfld.c:563-580); log10 of each when asked. */
enum { IMG_X, IMG_Y, IMG_CL, IMG_CR, IMG_P, IMG_S, IMG_UNPOL, IMG_COUNT };

static void polarisations(float complex p, float complex s, float phi, int logScale, float v[IMG_COUNT])
{
	const float complex x = p*cosf(phi*PI/180)-s*sinf(phi*PI/180);
	const float complex y = s*cosf(phi*PI/180)+p*sinf(phi*PI/180);
	v[IMG_X] = conjf(x)*x;
	v[IMG_Y] = conjf(y)*y;
	v[IMG_CL] = sq(crealf(p)+cimagf(s))+sq(cimagf(p)-crealf(s));
	v[IMG_CR] = sq(crealf(p)-cimagf(s))+sq(cimagf(p)+crealf(s));
	v[IMG_P] = conjf(p)*p;
	v[IMG_S] = conjf(s)*s;
	if (!logScale) {
		v[IMG_UNPOL] = v[IMG_P] + v[IMG_S];
		return;
	}
	for (int q = 0; q < IMG_UNPOL; q++) v[q] = log10f(v[q]);
	v[IMG_UNPOL] = log10f(conjf(p)*p+conjf(s)*s);
}

/* Where an image writer puts its files: W->ID followed by the caller's
 * formatted name; a name starting with '/' puts them in the directory
 * W->ID, and a full name ending with '/' is itself a directory. */
static void outputName(world W, const char *name, char *full, size_t cap)
{
	snprintf(full, cap, "%s%s", W->ID, name);
	if (name[0] == '/') mkdir(W->ID, 0755);
	size_t n = strlen(full);
	if (n && full[n-1] == '/') mkdir(full, 0755);
}

/* a one-plane slice of X x Y pixels, the shape the image writers take */
static slice imageSlice(int X, int Y)
{
	slice S = calloc(1, sizeof *S);
	S->jMax = S->jMAX = X - 1, S->jNUM = X;
	S->kMax = S->kMAX = Y - 1, S->kNUM = Y;
	return S;
}

/* Seven polarisation images of the far field over an X x Y projection
 * map (reference src/farfld.c:525-594).  The variable arguments are the
 * writer, its colour map and scale when it is png, and a printf-style
 * file name; a name containing "Log" writes log10 intensities.  Every
 * direction of the map goes to the backend in one batch per
 * polarisation. */
void farFieldProfile(world W, phaser P, projmap projMap, int X, int Y, ...)
{
	va_list ap;
	va_start(ap, Y);
	const method M = va_arg(ap, method);
	unsigned long int *cmap = 0;
	float scale = 1;
	if (M == png) {
		cmap = va_arg(ap, unsigned long int *);
		scale = va_arg(ap, double);
	}
	const char *format = va_arg(ap, const char *);
	char name[1024], base[1024], file[1100];
	vsnprintf(name, sizeof name, format, ap);
	va_end(ap);
	outputName(W, name, base, sizeof base);
	char logTag[4] = "";
	if (strstr(name, "Log")) strcpy(logTag, "Log");

	const int pixels = X * Y;
	float *theta = malloc(pixels * sizeof(float)), *phi = malloc(pixels * sizeof(float));
	float complex *ampP = malloc(pixels * sizeof(float complex)), *ampS = malloc(pixels * sizeof(float complex));
	/* pixels in the reference's order; a pixel the map leaves untouched
	 * (the middle column of an even-width AzimuthalMap) repeats the
	 * direction of the pixel before it */
	float a[2] = { 0, 0 };
	for (int q = 0; q < pixels; q++) {
		projMap(q / Y, q % Y, X, Y, a);
		theta[q] = a[0], phi[q] = a[1];
	}
	farFieldBatch(P, Ppol, pixels, theta, phi, ampP);
	farFieldBatch(P, Spol, pixels, theta, phi, ampS);

	slice S = imageSlice(X, Y);
	float ***img[IMG_COUNT];
	for (int q = 0; q < IMG_COUNT; q++) img[q] = makeField(0, 0, 0, X-1, 0, Y-1);
	float brightest = 0;
	for (int q = 0; q < pixels; q++) {
		float v[IMG_COUNT];
		polarisations(ampP[q], ampS[q], phi[q], logTag[0] != 0, v);
		for (int c = 0; c < IMG_COUNT; c++) img[c][0][q / Y][q % Y] = v[c];
		brightest = MAX(brightest, v[IMG_UNPOL]);
	}
	free(theta); free(phi); free(ampP); free(ampS);
	if (scale <= 0) scale = brightest;
	static const char *const suffix[IMG_COUNT] = { "X-pol", "Y-pol", "CL-pol", "CR-pol", "P-pol", "S-pol", "Unpol" };
	for (int c = 0; c < IMG_COUNT; c++) {
		snprintf(file, sizeof file, "%s%s", base, suffix[c]);
		S->F = img[c];
		M(W, S, scale, logTag, file, cmap);
		if (c < IMG_UNPOL) removeField(img[c], 0, 0, 0);
	}
	deleteSlice(S);
}

/* A 360-degree cut through the far field, one degree apart: theta at
 * fixed phi, or phi at fixed theta.  One row per degree: the angle, the
 * unpolarised, P and S intensities (reference src/farfld.c:597-624). */
static void farFieldCut(world W, phaser P, int alongTheta, float fixed, const char *name)
{
	float theta[360], phi[360];
	float complex ampP[360], ampS[360];
	for (int a = 0; a < 360; a++) {
		theta[a] = alongTheta ? a : fixed;
		phi[a] = alongTheta ? fixed : a;
	}
	farFieldBatch(P, Ppol, 360, theta, phi, ampP);
	farFieldBatch(P, Spol, 360, theta, phi, ampS);
	for (int a = 0; a < 360; a++) {
		const float ip = sq(cabsf(ampP[a])), is = sq(cabsf(ampS[a]));
		writeRow(W, (char *)name, (float)a, ip + is, ip, is);
	}
}

void farFieldTheta(world W, phaser P, float phi, char *format, ...)
{
	char name[1024];
	va_list ap;
	va_start(ap, format);
	vsnprintf(name, sizeof name, format, ap);
	va_end(ap);
	farFieldCut(W, P, 1, phi, name);
}

void farFieldPhi(world W, phaser P, float theta, char *format, ...)
{
	char name[1024];
	va_list ap;
	va_start(ap, format);
	vsnprintf(name, sizeof name, format, ap);
	va_end(ap);
	farFieldCut(W, P, 0, theta, name);
}

/* One ring of farFieldFlux: its index n around the axis, its sample
 * count and its solid-angle weight (a difference of cosines). */
typedef struct { int n, samples; float weight; } fluxRing;

/* Power into a cone of half-angle aMax (a ring aMin..aMax when aMin > 0)
 * around the direction (theta, phi), in the reference's quadrature
 * (src/farfld.c:627-662): a polar cap below delta/2 from farFieldI, then
 * rings of width delta with 6n samples each (at most 360 samples, from 60
 * degrees on).  Every ring sample goes to the backend in one batch per
 * polarisation; the float sum is formed in the reference's order. */
float (farFieldFlux)(phaser P, tfield pol(phaser,float,float), float theta, float phi, float aMin, float aMax, float delta, ...)
{
	if (!delta) delta = 1;
	if (!aMax) aMax = aMin, aMin = 0;
	float Sum = 0;
	int first = floor(aMin/delta+0.5);
	const int last = ceil(aMax/delta-0.5);
	if (!first) {
		Sum = 2 * PI * (cosf(aMin*PI/180) - cosf(MIN(aMax,0.5*delta)*PI/180)) * farFieldI(P,pol,theta,phi);
		aMin = 0.5 * delta;
		first = 1;
	}
	if (!last || last < first) return Sum;
	const int rings = 1 + last - first;
	const int widest = floor(60/delta+0.5);
	fluxRing *ring = malloc(rings * sizeof *ring);
	int total = 0;
	for (int r = 0; r < rings; r++) {
		const int n = first + r;
		ring[r].n = n;
		ring[r].samples = n < widest ? n*6 : widest*6;
		ring[r].weight = cosf(MAX(aMin,delta*(n-0.5))*PI/180) - cosf(MIN(aMax,delta*(n+0.5))*PI/180);
		total += ring[r].samples;
	}
	/* sample m of ring n: the direction at polar angle delta n and azimuth
	 * 360 m / N about the axis, and the angle c that turns its P/S frame
	 * into the frame of the axis */
	float *a = malloc(total * sizeof(float)), *b = malloc(total * sizeof(float)), *c = malloc(total * sizeof(float));
	float complex *ampP = malloc(total * sizeof(float complex)), *ampS = malloc(total * sizeof(float complex));
	for (int r = 0, q = 0; r < rings; r++) {
		const int n = ring[r].n, N = ring[r].samples;
		for (int m = 0; m < N; m++, q++) {
			a[q] = rotateA(theta, delta*n, 360.0*m/N);
			b[q] = rotateB(theta, delta*n, 360.0*m/N)+phi;
			c[q] = rotateB(-a[q], theta, phi-b[q])+180-360.0*m/N;
		}
	}
	farFieldBatch(P, Ppol, total, a, b, ampP);
	farFieldBatch(P, Spol, total, a, b, ampS);
	for (int r = 0, q = 0; r < rings; r++) {
		const int N = ring[r].samples;
		const float dth = ring[r].weight, arc = PI/N, chord = sinf(PI/N);
		for (int m = 0; m < N; m++, q++) {
			const float complex p = ampP[q], s = ampS[q];
			const float pp = sq(cabsf((p * cosf(c[q]*PI/180) - s * sinf(c[q]*PI/180))));
			const float ss = sq(cabsf((s * cosf(c[q]*PI/180) + p * sinf(c[q]*PI/180))));
			if (pol == Ppol) Sum += dth * (pp * (arc + chord) + ss * (arc - chord));
			if (pol == Spol) Sum += dth * (pp * (arc - chord) + ss * (arc + chord));
			if (pol == Unpol) Sum += 2 * arc * dth * (pp + ss);
		}
	}
	free(ring); free(a); free(b); free(c); free(ampP); free(ampS);
	return Sum;
}
