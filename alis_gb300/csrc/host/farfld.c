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

/* --- projection maps (reference src/farfld.c:14-41) --- */

void CylindericalMap(int x, int y, int X, int Y, float angle[2])
{
	angle[0] = 180.0 - 180.0 * y / Y;
	angle[1] = 360.0 * x / X;
}

void NorthernAzimuthalMap(int x, int y, int X, int Y, float angle[2])
{
	angle[0] = 180 * sqrtf(sq(x/(X-1.0)-0.5) + sq(y/(Y-1.0)-0.5));
	angle[1] = 180 * atan2f(y/(Y-1.0)-0.5, x/(X-1.0)-0.5) / PI;
	if (angle[0] > 90) angle[0] = INF;
}

void SouthernAzimuthalMap(int x, int y, int X, int Y, float angle[2])
{
	angle[0] = 180 - 180 * sqrtf(sq(x/(X-1.0)-0.5) + sq(y/(Y-1.0)-0.5));
	angle[1] = 180 * atan2f(y/(Y-1.0)-0.5, x/(X-1.0)-0.5) / PI;
	if (angle[0] < 90) angle[0] = INF;
}

void AzimuthalMap(int x, int y, int X, int Y, float angle[2])
{
	if (x < (X+1)/2) NorthernAzimuthalMap(x, y, (X+1)/2, Y, angle);
	if (x > X/2) SouthernAzimuthalMap(x-X/2, y, (X+1)/2, Y, angle);
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

/* Seven polarisation images (X, Y, CL, CR, P, S, unpolarised) of the far
 * field over an X x Y projection map (reference src/farfld.c:525-594).
 * All directions go to the backend as two batches. */
void farFieldProfile(world W, phaser P, projmap projMap, int X, int Y, ...)
{
	char *format, fieldname[4], filename[1024], fullname[1024];
	va_list ap;
	va_start(ap, Y);
	method M = va_arg(ap, method);
	unsigned long int *cmap = (M == png) ? va_arg(ap, unsigned long int *) : 0;
	float Max = (M == png) ? va_arg(ap, double) : 1;
	float max = 0, angle[2];
	format = va_arg(ap, char*);
	vsprintf(filename, format, ap);
	va_end(ap);
	strcat(strcpy(fullname, W->ID), filename);
	strcpy(fieldname, strstr(filename, "Log") ? "Log" : "");
	if (filename[0]=='/') mkdir(W->ID, 0755);
	if (fullname[strlen(fullname)-1]=='/') mkdir(fullname, 0755);

	slice S;
	MALLOC(S, 0, 1);
	*S = (struct slice) {0, 0, 0, X-1, 0, Y-1, 0, 0, 0, 0, X-1, X, 0, Y-1, Y};
	float ***img[7];
	for (int q = 0; q < 7; q++) img[q] = makeField(S->iMIN, S->iMAX, S->jMIN, S->jMAX, S->kMIN, S->kMAX);
	float ***Xp = img[0], ***Yp = img[1], ***Lp = img[2], ***Rp = img[3], ***Pp = img[4], ***Sp = img[5], ***Up = img[6];

	int NA = X*Y;
	float *th = calloc(NA, sizeof(float)), *ph = calloc(NA, sizeof(float));
	float complex *pv = calloc(NA, sizeof(float complex)), *sv = calloc(NA, sizeof(float complex));
	for (int x = 0; x < X; x++) for (int y = 0; y < Y; y++) {
		projMap(x, y, X, Y, angle);
		th[x*Y+y] = angle[0], ph[x*Y+y] = angle[1];
	}
	printf("Performing Near-to-Far-Field Transformation.\n");
	farFieldBatch(P, Ppol, NA, th, ph, pv);
	farFieldBatch(P, Spol, NA, th, ph, sv);
	int log = fieldname[0] != 0;
	for (int x = 0; x < X; x++) for (int y = 0; y < Y; y++) {
		float complex p = pv[x*Y+y], s = sv[x*Y+y];
		float a1 = ph[x*Y+y];
		float vx = conjf(p*cosf(a1*PI/180)-s*sinf(a1*PI/180))*(p*cosf(a1*PI/180)-s*sinf(a1*PI/180));
		float vy = conjf(s*cosf(a1*PI/180)+p*sinf(a1*PI/180))*(s*cosf(a1*PI/180)+p*sinf(a1*PI/180));
		float vl = sq(crealf(p)+cimagf(s))+sq(cimagf(p)-crealf(s));
		float vr = sq(crealf(p)-cimagf(s))+sq(cimagf(p)+crealf(s));
		float vp = conjf(p)*p, vs = conjf(s)*s;
		if (log) {
			Xp[0][x][y] = log10f(vx), Yp[0][x][y] = log10f(vy), Lp[0][x][y] = log10f(vl), Rp[0][x][y] = log10f(vr);
			Pp[0][x][y] = log10f(vp), Sp[0][x][y] = log10f(vs), Up[0][x][y] = log10f(conjf(p)*p+conjf(s)*s);
		} else {
			Xp[0][x][y] = vx, Yp[0][x][y] = vy, Lp[0][x][y] = vl, Rp[0][x][y] = vr;
			Pp[0][x][y] = vp, Sp[0][x][y] = vs, Up[0][x][y] = Pp[0][x][y]+Sp[0][x][y];
		}
		max = MAX(max, Up[0][x][y]);
	}
	free(th); free(ph); free(pv); free(sv);
	if (Max <= 0) Max = max;
	const char *tag[7] = { "X-pol", "Y-pol", "CL-pol", "CR-pol", "P-pol", "S-pol", "Unpol" };
	for (int q = 0; q < 7; q++) {
		S->F = img[q];
		M(W, S, Max, fieldname, strcat(strcpy(filename, fullname), tag[q]), cmap);
		if (q < 6) removeField(img[q], 0, 0, 0);
	}
	deleteSlice(S);
}

void farFieldTheta(world W, phaser P, float phi, char *format, ...)
{
	char filename[1024];
	va_list ap;
	va_start(ap, format);
	vsprintf(filename, format, ap);
	va_end(ap);
	float th[360], ph[360];
	float complex p[360], s[360];
	for (int a = 0; a < 360; a++) th[a] = a, ph[a] = phi;
	farFieldBatch(P, Ppol, 360, th, ph, p);
	farFieldBatch(P, Spol, 360, th, ph, s);
	for (int a = 0; a < 360; a++)
		writeRow(W, filename, th[a], sq(cabsf(p[a]))+sq(cabsf(s[a])), sq(cabsf(p[a])), sq(cabsf(s[a])));
}

void farFieldPhi(world W, phaser P, float theta, char *format, ...)
{
	char filename[1024];
	va_list ap;
	va_start(ap, format);
	vsprintf(filename, format, ap);
	va_end(ap);
	float th[360], ph[360];
	float complex p[360], s[360];
	for (int a = 0; a < 360; a++) th[a] = theta, ph[a] = a;
	farFieldBatch(P, Ppol, 360, th, ph, p);
	farFieldBatch(P, Spol, 360, th, ph, s);
	for (int a = 0; a < 360; a++)
		writeRow(W, filename, ph[a], sq(cabsf(p[a]))+sq(cabsf(s[a])), sq(cabsf(p[a])), sq(cabsf(s[a])));
}

/* power into a cone of half-angle aMax (or a ring aMin..aMax) around
 * (theta, phi), integrated on rings of width delta with 6n samples
 * (reference src/farfld.c:627-662) */
float (farFieldFlux)(phaser P, tfield pol(phaser,float,float), float theta, float phi, float aMin, float aMax, float delta, ...)
{
	if (!delta) delta = 1;
	if (!aMax) aMax = aMin, aMin = 0;
	float Sum = 0;
	int nMin = floor(aMin/delta+0.5);
	int nMax = ceil(aMax/delta-0.5);
	if (!nMin) {
		Sum = 2 * PI * (cosf(aMin*PI/180) - cosf(MIN(aMax,0.5*delta)*PI/180)) * farFieldI(P,pol,theta,phi);
		aMin = 0.5 * delta;
		nMin++;
	}
	if (!nMax) return Sum;
	for (int n = nMin; n <= nMax; n++) {
		int N = n<floor(60/delta+0.5) ? n*6 : floor(60/delta+0.5)*6;
		float dth = cosf(MAX(aMin,delta*(n-0.5))*PI/180) - cosf(MIN(aMax,delta*(n+0.5))*PI/180);
		float *a = calloc(N, sizeof(float)), *b = calloc(N, sizeof(float)), *c = calloc(N, sizeof(float));
		float complex *pv = calloc(N, sizeof(float complex)), *sv = calloc(N, sizeof(float complex));
		for (int m = 0; m < N; m++) {
			a[m] = rotateA(theta, delta*n, 360.0*m/N);
			b[m] = rotateB(theta, delta*n, 360.0*m/N)+phi;
			c[m] = rotateB(-a[m], theta, phi-b[m])+180-360.0*m/N;
		}
		farFieldBatch(P, Ppol, N, a, b, pv);
		farFieldBatch(P, Spol, N, a, b, sv);
		for (int m = 0; m < N; m++) {
			float complex p = pv[m], s = sv[m];
			float pp = sq(cabsf((p * cosf(c[m]*PI/180) - s * sinf(c[m]*PI/180))));
			float ss = sq(cabsf((s * cosf(c[m]*PI/180) + p * sinf(c[m]*PI/180))));
			if (pol == Ppol) Sum += dth * (pp * (PI/N + sinf(PI/N)) + ss * (PI/N - sinf(PI/N)));
			if (pol == Spol) Sum += dth * (pp * (PI/N - sinf(PI/N)) + ss * (PI/N + sinf(PI/N)));
			if (pol == Unpol) Sum += 2 * PI/N * dth * (pp + ss);
		}
		free(a); free(b); free(c); free(pv); free(sv);
	}
	return Sum;
}
