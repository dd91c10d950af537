/*
 * output.c -- point probes, volume reductions, Poynting flux through
 * planes and boxes, object absorption, and text output.
 *
 * Host observers of the reference src/output.c.  They read host mirrors
 * and refresh them first.  Reductions are sequential (the reference's
 * result with one OpenMP thread).
 */
#include <sys/time.h>
#include <sys/stat.h>
#include <string.h>
#include "engine.h"

int alis_needs_currents(matter M);

/* --- output files keyed by (world, name) (reference src/output.c:104-174) --- */

typedef struct outfile {
	world W;
	char *name;
	FILE *file;
	unsigned long N;
	unsigned long long stamp;
	float complex **spectrum;
	struct outfile *next;
} outfile;

/* find or open the record of (W, ID); on return ID holds W->ID + name
 * and the directory it names exists */
static outfile *lookup(world W, char *ID, outfile **head)
{
	outfile *q;
	for (q = *head; q; q = q->next) if (q->W == W && !strcmp(q->name, ID)) break;
	if (!q) {
		q = calloc(1, sizeof *q);
		q->W = W;
		q->name = strdup(ID);
		q->next = *head;
		*head = q;
		strcat(strcpy(ID, W->ID), q->name);
		if (q->name[0]=='/') mkdir(W->ID, 0755);
		if (ID[0] && ID[strlen(ID)-1]=='/') mkdir(ID, 0755);
	} else {
		strcat(strcpy(ID, W->ID), q->name);
	}
	q->N++;
	return q;
}

static unsigned long long nowMicro(void)
{
	struct timeval now;
	gettimeofday(&now, 0);
	return now.tv_sec * 1000000ULL + now.tv_usec;
}

/* append text to <ID><name>.txt, flushed at most every 300 s */
void (writeTxt)(world W, char *format, ...)
{
	static outfile *head;
	char str[4096], filename[1024];
	va_list ap;
	va_start(ap, format);
	vsnprintf(filename, sizeof filename, format, ap);
	format = va_arg(ap, char*);
	vsnprintf(str, sizeof str, format, ap);
	va_end(ap);
	outfile *q = lookup(W, filename, &head);
	unsigned long long t = nowMicro();
	if (!q->stamp) {
		q->file = fopen(strcat(filename, ".txt"), "w");
		q->stamp = t;
	}
	if (q->file) fputs(str, q->file);
	if (q->file && t - q->stamp >= 300*1000000ULL) fflush(q->file), q->stamp = t;
}

/* one tab-separated row of doubles, terminated by the INT2NAN sentinel */
void (writeRow)(world W, char *format, ...)
{
	char str[4096], filename[1024];
	va_list ap;
	va_start(ap, format);
	vsnprintf(filename, sizeof filename, format, ap);
	double f = va_arg(ap, double);
	if (!NAN2INT(f)) {
		int n = sprintf(str, "%g", f);
		for (f = va_arg(ap, double); !NAN2INT(f); f = va_arg(ap, double)) n += sprintf(str+n, "\t%g", f);
		sprintf(str+n, "\n");
		writeTxt(W, filename, str);
	}
	va_end(ap);
}

source alis_reference_source(world W);

/* Running DFT of point values over N calls on the createPhasers grid of
 * (LMin, LMax, dL = LMin LMax / (N dt)); on the N-th call writes
 * |value / source spectrum| and its phase per wavelength
 * (reference src/output.c:177-230). */
void (writeSpectrum)(world W, int N, float LMin, float LMax, char *format, ...)
{
	static outfile *head;
	char filename[1024];
	double d;
	float dL = LMin * LMax / (N * W->dt);
	int M = 0, nMin = floor(LMin/dL), nMax = ceil(LMax/dL);
	va_list ap;
	va_start(ap, format);
	vsnprintf(filename, sizeof filename, format, ap);
	do d = va_arg(ap, double), M++;
	while (!NAN2INT(d));
	va_end(ap);
	va_start(ap, format);
	vsnprintf(filename, sizeof filename, format, ap);
	outfile *q = lookup(W, filename, &head);
	int nf = 1-nMin+nMax;
	if (!q->spectrum) {
		source S = alis_reference_source(W);
		MALLOC(q->spectrum, 0, M);
		MALLOC(q->spectrum[0], 0, M*nf);
		for (int m = 1; m < M; m++) q->spectrum[m] = q->spectrum[0]+m*nf;
		if (S && W->N) for (int n = 0; n <= nMax-nMin; n++) {
			float f = (nMax-n) / (dL * nMin * nMax);
			for (int m = 1; m < W->N; m++) q->spectrum[0][n] += S->waveForm(W, S, W->dt*m, S->phase) * cexpf(2*PI*I*f*W->dt*m);
			if (cabsf(q->spectrum[0][n]) < 1E-3) q->spectrum[0][n] = 0;
			else if (W->sourceType == 2) q->spectrum[0][n] *= sqrtf(f * S->wavelength);
			else if (W->sourceType == 3) q->spectrum[0][n] *= f * S->wavelength;
		}
	}
	for (int m = 1; m < M; m++) {
		float t = W->t / (dL * nMin * nMax);
		d = va_arg(ap, double);
		for (int n = 0; n <= nMax-nMin; n++) q->spectrum[m][n] += (float) d * cexpf(2*PI*I*t*(nMax-n));
	}
	va_end(ap);
	if (q->N == (unsigned long)N) {
		q->file = fopen(strcat(filename, ".txt"), "w");
		if (!q->file) return;
		for (int n = 0; n <= nMax-nMin; n++) {
			fprintf(q->file, "%g", (dL * nMin * nMax) / (nMax-n));
			for (int m = 1; m < M; m++) fprintf(q->file, "\t%g", q->spectrum[0][n] ? cabsf(q->spectrum[m][n]/q->spectrum[0][n]) : 0);
			for (int m = 1; m < M; m++) fprintf(q->file, "\t%g", q->spectrum[0][n] ? cargf(q->spectrum[m][n]/q->spectrum[0][n])/PI : 0);
			fprintf(q->file, "\n");
		}
		fclose(q->file);
		q->file = 0;
	}
}


/* --- probes and volume reductions (reference src/output.c:50-101) --- */

float get(world W, field F, float x, float y, float z)
{
	int i = W->xtoi(W, x), j = W->ytoj(W, y), k = W->ztok(W, z);
	if (alis_be_sync_near(W, i, j, k)) {
		/* the host mirrors are current around the probe */
		alis_be_hold_sync(W);
		float v = F(W, i, j, k);
		alis_be_hold_sync(0);
		return v;
	}
	alis_be_sync_world(W);
	return F(W, i, j, k);
}

float worldMax(world W, field F)
{
	alis_be_sync_world(W);
	float Max = 0, f;
	for (int i = W->iMin; i < W->iMax; i++) for (int j = W->jMin; j < W->jMax; j++) for (int k = W->kMin; k < W->kMax; k++)
		if (Max < (f = fabsf(F(W, i, j, k)))) Max = f;
	return Max;
}

/* trapezoid integral over the domain (reference src/output.c:72-101) */
static float sumZ(world W, field F, int i, int j)
{
	float Sum = 0;
	for (int k = W->kMin+1; k < W->kMax; k++) Sum += W->CE->dz[k] * F(W, i, j, k);
	Sum += 0.5 * W->CE->dz[W->kMin] * F(W, i, j, W->kMin);
	Sum += 0.5 * W->CE->dz[W->kMax] * F(W, i, j, W->kMax);
	return Sum;
}

static float sumY(world W, field F, int i)
{
	float Sum = 0;
	for (int j = W->jMin+1; j < W->jMax; j++) Sum += W->CE->dy[j] * sumZ(W, F, i, j);
	Sum += 0.5 * W->CE->dy[W->jMin] * sumZ(W, F, i, W->jMin);
	Sum += 0.5 * W->CE->dy[W->jMax] * sumZ(W, F, i, W->jMax);
	return Sum;
}

float worldSum(world W, field F)
{
	alis_be_sync_world(W);
	float Sum = 0;
	for (int i = W->iMin+1; i < W->iMax; i++) Sum += W->CE->dx[i] * sumY(W, F, i);
	Sum += 0.5 * W->CE->dx[W->iMin] * sumY(W, F, W->iMin);
	Sum += 0.5 * W->CE->dx[W->iMax] * sumY(W, F, W->iMax);
	if (W->xMinSur==SYM) Sum *= 2;
	if (W->yMinSur==SYM) Sum *= 2;
	if (W->zMinSur==SYM) Sum *= 2;
	return Sum;
}


/* --- Poynting flux through planes (reference src/output.c:233-356) ---
 * Instantaneous E x H through an axis-normal plane clipped to the domain;
 * H is averaged across the plane.  A zero-width range in a transverse
 * axis (or a 2-D world) becomes a line density. */

/* index range of [lo, hi] along an axis: a point widens to +-1 cell */
static void span(int (*toIdx)(world, float), world W, float lo, float hi, int minI, int maxI, int *a, int *b)
{
	*a = lo==hi ? MAX(minI, toIdx(W, lo)-1) : MAX(minI, toIdx(W, lo));
	*b = lo==hi ? MIN(maxI, toIdx(W, hi)+1) : MIN(maxI, toIdx(W, hi));
}

float (poyntingX)(world W, float x, float yMin, float yMax, float zMin, float zMax, ...)
{
	float Sum = 0, Part = 0;
	int i = W->xtoi(W, x<0 && W->xMinSur==SYM ? -x : x), jMin, jMax, kMin, kMax;
	span(W->ytoj, W, yMin, yMax, W->jMin, W->jMax, &jMin, &jMax);
	span(W->ztok, W, zMin, zMax, W->kMin, W->kMax, &kMin, &kMax);
	vfield *E = W->E, *H = W->H;
	if (alis_be_plane_flux(W, 0, i, jMin, jMax, kMin, kMax, &Sum)) goto scale;
	alis_be_sync_world(W);
	for (int j = jMin+1; j <= jMax; j++) {
		float sum = 0;
		sum += 0.5 * W->CE->dz[kMin] * E->y[i][j][kMin] * (H->z[i][j][kMin] + H->z[i+1][j][kMin]);
		sum += 0.5 * W->CE->dz[kMax] * E->y[i][j][kMax] * (H->z[i][j][kMax] + H->z[i+1][j][kMax]);
		for (int k = kMin+1; k < kMax; k++) sum += W->CE->dz[k] * E->y[i][j][k] * (H->z[i][j][k] + H->z[i+1][j][k]);
		Sum += W->CH->dy[j] * sum;
	}
	for (int k = kMin+1; k <= kMax; k++) {
		float sum = 0;
		sum -= 0.5 * W->CE->dy[jMin] * E->z[i][jMin][k] * (H->y[i][jMin][k] + H->y[i+1][jMin][k]);
		sum -= 0.5 * W->CE->dy[jMax] * E->z[i][jMax][k] * (H->y[i][jMax][k] + H->y[i+1][jMax][k]);
		for (int j = jMin+1; j < jMax; j++) sum -= W->CE->dy[j] * E->z[i][j][k] * (H->y[i][j][k] + H->y[i+1][j][k]);
		Part += W->CH->dz[k] * sum;
	}
	Sum += Part;
scale:
	if (yMin==yMax || W->Dom.y.Min==W->Dom.y.Max) Sum /= W->CH->dy[jMax]+W->CH->dy[jMax-1];
	if (zMin==zMax || W->Dom.z.Min==W->Dom.z.Max) Sum /= W->CH->dz[kMax]+W->CH->dz[kMax-1];
	if (W->yMinSur==SYM) Sum *= 2;
	if (W->zMinSur==SYM) Sum *= 2;
	return (x<0 && W->xMinSur==SYM ? -0.5 : 0.5) * Sum;
}

float (poyntingY)(world W, float y, float xMin, float xMax, float zMin, float zMax, ...)
{
	float Sum = 0, Part = 0;
	int j = W->ytoj(W, y<0 && W->yMinSur==SYM ? -y : y), iMin, iMax, kMin, kMax;
	span(W->xtoi, W, xMin, xMax, W->iMin, W->iMax, &iMin, &iMax);
	span(W->ztok, W, zMin, zMax, W->kMin, W->kMax, &kMin, &kMax);
	vfield *E = W->E, *H = W->H;
	if (alis_be_plane_flux(W, 1, j, iMin, iMax, kMin, kMax, &Sum)) goto scale;
	alis_be_sync_world(W);
	for (int k = kMin+1; k <= kMax; k++) {
		float sum = 0;
		sum += 0.5 * W->CE->dx[iMin] * E->z[iMin][j][k] * (H->x[iMin][j][k] + H->x[iMin][j+1][k]);
		sum += 0.5 * W->CE->dx[iMax] * E->z[iMax][j][k] * (H->x[iMax][j][k] + H->x[iMax][j+1][k]);
		for (int i = iMin+1; i < iMax; i++) sum += W->CE->dx[i] * E->z[i][j][k] * (H->x[i][j][k] + H->x[i][j+1][k]);
		Sum += W->CH->dz[k] * sum;
	}
	for (int i = iMin+1; i <= iMax; i++) {
		float sum = 0;
		sum -= 0.5 * W->CE->dz[kMin] * E->x[i][j][kMin] * (H->z[i][j][kMin] + H->z[i][j+1][kMin]);
		sum -= 0.5 * W->CE->dz[kMax] * E->x[i][j][kMax] * (H->z[i][j][kMax] + H->z[i][j+1][kMax]);
		for (int k = kMin+1; k < kMax; k++) sum -= W->CE->dz[k] * E->x[i][j][k] * (H->z[i][j][k] + H->z[i][j+1][k]);
		Part += W->CH->dx[i] * sum;
	}
	Sum += Part;
scale:
	if (xMin==xMax || W->Dom.x.Min==W->Dom.x.Max) Sum /= W->CH->dx[iMax]+W->CH->dx[iMax-1];
	if (zMin==zMax || W->Dom.z.Min==W->Dom.z.Max) Sum /= W->CH->dz[kMax]+W->CH->dz[kMax-1];
	if (W->xMinSur==SYM) Sum *= 2;
	if (W->zMinSur==SYM) Sum *= 2;
	return (y<0 && W->yMinSur==SYM ? -0.5 : 0.5) * Sum;
}

float (poyntingZ)(world W, float z, float xMin, float xMax, float yMin, float yMax, ...)
{
	float Sum = 0, Part = 0;
	int k = W->ztok(W, z<0 && W->zMinSur==SYM ? -z : z), iMin, iMax, jMin, jMax;
	span(W->xtoi, W, xMin, xMax, W->iMin, W->iMax, &iMin, &iMax);
	span(W->ytoj, W, yMin, yMax, W->jMin, W->jMax, &jMin, &jMax);
	vfield *E = W->E, *H = W->H;
	if (alis_be_plane_flux(W, 2, k, iMin, iMax, jMin, jMax, &Sum)) goto scale;
	alis_be_sync_world(W);
	for (int i = iMin+1; i <= iMax; i++) {
		float sum = 0;
		sum += 0.5 * W->CE->dy[jMin] * E->x[i][jMin][k] * (H->y[i][jMin][k] + H->y[i][jMin][k+1]);
		sum += 0.5 * W->CE->dy[jMax] * E->x[i][jMax][k] * (H->y[i][jMax][k] + H->y[i][jMax][k+1]);
		for (int j = jMin+1; j < jMax; j++) sum += W->CE->dy[j] * E->x[i][j][k] * (H->y[i][j][k] + H->y[i][j][k+1]);
		Sum += W->CH->dx[i] * sum;
	}
	for (int j = jMin+1; j <= jMax; j++) {
		float sum = 0;
		sum -= 0.5 * W->CE->dx[iMin] * E->y[iMin][j][k] * (H->x[iMin][j][k] + H->x[iMin][j][k+1]);
		sum -= 0.5 * W->CE->dx[iMax] * E->y[iMax][j][k] * (H->x[iMax][j][k] + H->x[iMax][j][k+1]);
		for (int i = iMin+1; i < iMax; i++) sum -= W->CE->dx[i] * E->y[i][j][k] * (H->x[i][j][k] + H->x[i][j][k+1]);
		Part += W->CH->dy[j] * sum;
	}
	Sum += Part;
scale:
	if (xMin==xMax || W->Dom.x.Min==W->Dom.x.Max) Sum /= W->CH->dx[iMax]+W->CH->dx[iMax-1];
	if (yMin==yMax || W->Dom.y.Min==W->Dom.y.Max) Sum /= W->CH->dy[jMax]+W->CH->dy[jMax-1];
	if (W->xMinSur==SYM) Sum *= 2;
	if (W->yMinSur==SYM) Sum *= 2;
	return (z<0 && W->zMinSur==SYM ? -0.5 : 0.5) * Sum;
}

float poyntingOut(world W, float xMin, float xMax, float yMin, float yMax, float zMin, float zMax)
{
	float Sx = 0, Sy = 0, Sz = 0;
	if (xMin > W->xMin || xMax < W->xMax || W->xMinSur != BBC) {
		Sx = (poyntingX)(W, xMax, yMin, yMax, zMin, zMax);
		if (xMin < 0 && W->xMinSur==SYM) Sx *= 2;
		else Sx -= (poyntingX)(W, xMin, yMin, yMax, zMin, zMax);
	}
	if (yMin > W->yMin || yMax < W->yMax || W->yMinSur != BBC) {
		Sy = (poyntingY)(W, yMax, xMin, xMax, zMin, zMax);
		if (yMin < 0 && W->yMinSur==SYM) Sy *= 2;
		else Sy -= (poyntingY)(W, yMin, xMin, xMax, zMin, zMax);
	}
	if (zMin > W->zMin || zMax < W->zMax || W->zMinSur != BBC) {
		Sz = (poyntingZ)(W, zMax, xMin, xMax, yMin, yMax);
		if (zMin < 0 && W->zMinSur==SYM) Sz *= 2;
		else Sz -= (poyntingZ)(W, zMin, xMin, xMax, yMin, yMax);
	}
	return Sx + Sy + Sz;
}


/* --- absorption in a dispersive object (reference src/output.c:25-47, 359-435) --- */

/* polarisation + conduction current density of dispersive object n */
static float objCurrent(world W, int a, int n, int i, int j, int k)
{
	coeffs *C = W->CE;
	float *ax = a==0 ? C->ax : a==1 ? C->ay : C->az;
	float ****fill = a==0 ? C->Jx : a==1 ? C->Jy : C->Jz;
	float ***e = a==0 ? W->E->x : a==1 ? W->E->y : W->E->z;
	float *****J = a==0 ? W->E->Jx : a==1 ? W->E->Jy : W->E->Jz;
	float ***map = a==0 ? C->x : a==1 ? C->y : C->z;
	float f = 0;
	if (ax[n]) f += 2 * fill[n][i][j][k] * e[i][j][k] / (1 + 1 / ax[n]);
	for (int p = 0; p < C->NK[n]; p++) if (J[n][p]) f += J[n][p][i][j][k];
	return f / map[i][j][k];
}

static int sameObject(object a, object b)
{
	if (a.S != b.S || a.p != b.p) return 0;
	for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) if (a.f[i][j] != b.f[i][j]) return 0;
	return 1;
}

static float columnAbsorption(world W, int n, int i, int j, float x, float y, float z)
{
	float Sum = 0, xsum = 0, ysum = 0, zsum = 0;
	coeffs *C = W->CE;
	int kMinJ = MAX(W->kMIN, C->kMin[n]), kMaxJ = MIN(W->kMAX, C->kMax[n]);
	for (int k = kMinJ; k <= kMaxJ; k++) {
		if (C->x[i][j][k]) xsum += C->dz[k] * W->E->x[i][j][k] * objCurrent(W, 0, n, i, j, k);
		if (C->y[i][j][k]) ysum += C->dz[k] * W->E->y[i][j][k] * objCurrent(W, 1, n, i, j, k);
		if (C->z[i][j][k]) zsum += W->CH->dz[k] * W->E->z[i][j][k] * objCurrent(W, 2, n, i, j, k);
	}
	if (kMinJ == W->kMIN) {
		if (C->x[i][j][W->kMIN]) xsum -= C->dz[W->kMIN] * W->E->x[i][j][W->kMIN] * objCurrent(W, 0, n, i, j, W->kMIN) * 0.5;
		if (C->y[i][j][W->kMIN]) ysum -= C->dz[W->kMIN] * W->E->y[i][j][W->kMIN] * objCurrent(W, 1, n, i, j, W->kMIN) * 0.5;
		if (C->z[i][j][W->kMIN]) zsum -= W->CH->dz[W->kMIN] * W->E->z[i][j][W->kMIN] * objCurrent(W, 2, n, i, j, W->kMIN);
	}
	if (kMaxJ == W->kMAX) {
		if (C->x[i][j][W->kMAX]) xsum -= C->dz[W->kMAX] * W->E->x[i][j][W->kMAX] * objCurrent(W, 0, n, i, j, W->kMAX) * 0.5;
		if (C->y[i][j][W->kMAX]) ysum -= C->dz[W->kMAX] * W->E->y[i][j][W->kMAX] * objCurrent(W, 1, n, i, j, W->kMAX) * 0.5;
	}
	Sum += x * xsum * W->CH->dx[i] * C->dy[j];
	Sum += y * ysum * C->dx[i] * W->CH->dy[j];
	Sum += z * zsum * C->dx[i] * C->dy[j];
	return Sum;
}

/* power absorbed by the dispersive object O: J . E summed over its box
 * with half weights on the grid edges */
float objectAbsorption(world W, object O)
{
	float Sum = 0;
	int n = 0;
	for (int o = 0; !sameObject(O, W->CE->O[o]); o++) if (alis_needs_currents(W->CE->M[o])) n++;
	coeffs *C = W->CE;
	if (alis_be_object_absorption(W, n, &Sum)) goto scale;
	alis_be_sync_world(W);
	int iMinJ = MAX(W->iMIN, C->iMin[n]), iMaxJ = MIN(W->iMAX, C->iMax[n]);
	int jMinJ = MAX(W->jMIN, C->jMin[n]), jMaxJ = MIN(W->jMAX, C->jMax[n]);
	for (int i = iMinJ; i <= iMaxJ; i++) {
		for (int j = jMinJ; j <= jMaxJ; j++) Sum += columnAbsorption(W, n, i, j, 1, 1, 1);
		if (jMinJ == W->jMIN) Sum += columnAbsorption(W, n, i, W->jMIN,-0.5,-1,-0.5);
		if (jMaxJ == W->jMAX) Sum += columnAbsorption(W, n, i, W->jMAX,-0.5, 0,-0.5);
	}
	/* each OpenMP-reduced loop of the reference sums from zero before
	 * joining the total */
	if (iMinJ == W->iMIN) {
		float part = 0;
		for (int j = jMinJ; j <= jMaxJ; j++) part += columnAbsorption(W, n, W->iMIN, j,-1,-0.5,-0.5);
		Sum += part;
		if (jMinJ == W->jMIN) Sum += columnAbsorption(W, n, W->iMIN, W->jMIN, 0.5, 0.5, 0.25);
		if (jMaxJ == W->jMAX) Sum += columnAbsorption(W, n, W->iMIN, W->jMAX, 0.5, 0.0, 0.25);
	}
	if (iMaxJ == W->iMAX) {
		float part = 0;
		for (int j = jMinJ; j <= jMaxJ; j++) part += columnAbsorption(W, n, W->iMAX, j, 0,-0.5,-0.5);
		Sum += part;
		if (jMinJ == W->jMIN) Sum += columnAbsorption(W, n, W->iMAX, W->jMIN, 0.0, 0.5, 0.25);
		if (jMaxJ == W->jMAX) Sum += columnAbsorption(W, n, W->iMAX, W->jMAX, 0.0, 0.0, 0.25);
	}
scale:
	if (W->Dom.x.Min==W->Dom.x.Max) Sum /= W->CH->dx[W->iMax]+W->CH->dx[W->iMax-1];
	if (W->Dom.y.Min==W->Dom.y.Max) Sum /= W->CH->dy[W->jMax]+W->CH->dy[W->jMax-1];
	if (W->Dom.z.Min==W->Dom.z.Max) Sum /= W->CH->dz[W->kMax]+W->CH->dz[W->kMax-1];
	if (W->xMinSur==SYM) Sum *= 2;
	if (W->yMinSur==SYM) Sum *= 2;
	if (W->zMinSur==SYM) Sum *= 2;
	return Sum / W->dt;
}

void exec(char *format, ...)
{
	char str[1024];
	va_list ap;
	va_start(ap, format);
	vsnprintf(str, sizeof str, format, ap);
	va_end(ap);
	if (system(str)) {}
}
