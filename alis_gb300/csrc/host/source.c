/*
 * source.c -- waveforms, point dipoles, TFSF plane waves and beams.
 *
 * Host half of the reference src/source.c.  Sources are descriptors
 * (region, amplitude map or scalar, waveform); the backend evaluates the
 * waveform once per half step on the host (glibc sinf/expf/cosf, so the
 * values equal the reference's) and adds amplitude * value on the device.
 * A TFSF plane wave owns an auxiliary world that is one Yee cell wide in
 * x and y; its field rows are aliased across the main grid exactly like
 * the reference (src/source.c:223-249) so that host observers see the
 * incident field at any (i, j).
 */
#include <string.h>
#include "engine.h"


/* --- waveforms (reference src/source.c:11-49) ---
 * Each initialises its parameters on the first call (S->N == 0) and sets
 * S->N, the number of steps during which the source is active.  The
 * parameters are computed in single precision (alis_f32), as the
 * reference computes them; the per-step values use the stored fields. */

/* CW sine with a raised-cosine turn-on over `supplement` periods */
float Sine(world W, source S, float t, float phase)
{
	if (!S->N) {
		alis_f32 lam = S->wavelength, sup = S->supplement, dt = W->dt;
		alis_f32 peak = dt * floorf(lam * sup / dt);
		S->frequency = (alis_f32)(2 * PI / lam);
		S->peaktime = peak;
		S->deviation = (alis_f32)(peak / PI);
		S->N = -1;
	}
	if (t < S->peaktime)
		return sinf(S->frequency * (t-S->peaktime) - phase) * (0.5 * (1 - cosf(t / S->deviation)));
	return sinf(S->frequency * (t-S->peaktime) - phase);
}

/* Gaussian-envelope carrier; supplement sets the bandwidth */
float Pulse(world W, source S, float t, float phase)
{
	if (!S->N) {
		alis_f32 lam = S->wavelength, sup = S->supplement, dt = W->dt;
		alis_f32 dev = 2 * sq(lam) / (PI * sup);
		alis_f32 steps = floorf((alis_f32)(PI * dev) / dt);
		S->frequency = (alis_f32)(2 * PI / lam);
		S->deviation = dev;
		S->peaktime = (alis_f32)(dt * steps);
		S->N = 2 * steps;
	}
	return sinf(S->frequency * (t-S->peaktime) - phase) * expf(-sq((t-S->peaktime) / S->deviation));
}

/* flat band between wavelength and supplement (difference of sincs) */
float Band(world W, source S, float t, float phase)
{
	(void)phase;
	if (!S->N) {
		alis_f32 lam = S->wavelength, sup = S->supplement, dt = W->dt;
		/* the `0.5` and `1.25` literals are double: those steps are
		 * double in the reference too, rounded to float where stored */
		alis_f32 res = sup > lam ? (alis_f32)ceilf((alis_f32)(1.25 * sup / lam + 0.5)) : 2;
		S->resolution = res;
		S->frequency = (alis_f32)(2 * PI / lam);
		S->deviation = (alis_f32)((alis_f32)(2 * PI / lam) / (res - 0.5));
		S->peaktime = (alis_f32)((alis_f32)floorf((alis_f32)(lam * (res - 0.5) / dt)) * dt);
		S->N = 2 * lam * (res - 0.5) / dt;
	}
	if (t == S->peaktime) return 0;
	return 2 * (cosf((t-S->peaktime) * S->deviation * S->resolution) - cosf((t-S->peaktime) * S->deviation)) / ((t-S->peaktime) * S->deviation);
}


/* --- field identity helpers --- */

static int isE(field F) { return F==Ex || F==Ey || F==Ez || F==iEx || F==iEy || F==iEz; }
static int isH(field F) { return F==Hx || F==Hy || F==Hz || F==iHx || F==iHy || F==iHz; }
/* does F point along / carry a half-cell offset in axis a (x=0, y=1, z=2)
 * on the Yee grid: E along a, or H transverse to a */
static int stagX(field F) { return F==Ex || F==Hy || F==Hz || F==iEx || F==iHy || F==iHz; }
static int stagY(field F) { return F==Ey || F==Hz || F==Hx || F==iEy || F==iHz || F==iHx; }
static int stagZ(field F) { return F==Ez || F==Hx || F==Hy || F==iEz || F==iHx || F==iHy; }

static float ***targetArray(world W, field F)
{
	field *names[12] = { Ex, Ey, Ez, Hx, Hy, Hz, iEx, iEy, iEz, iHx, iHy, iHz };
	for (int q = 0; q < 12; q++) {
		if (F != names[q]) continue;
		vfield *V = q % 6 < 3 ? &W->E[q/6] : &W->H[q/6];
		return q % 3 == 0 ? V->x : q % 3 == 1 ? V->y : V->z;
	}
	return 0;
}

/* new source appended to the E or H chain of W (reference src/source.c:52-75) */
static source newSource(world W, field F, waveform waveForm, float wavelength, float supplement, float resolution)
{
	source S;
	MALLOC(S, 0, 1);
	*S = (struct source) { waveForm, wavelength, supplement, resolution };
	waveForm(W, S, 0, 0);
	source *chain = isE(F) ? &W->SE : isH(F) ? &W->SH : 0;
	if (chain) {
		while (*chain) chain = &(*chain)->S;
		*chain = S;
		S->F = targetArray(W, F);
	}
	if (W->N < S->N && S->N != (unsigned long)-1) W->N = S->N;
	if (wavelength && W->T != wavelength/W->dt) W->f = 1/wavelength, W->T = wavelength/W->dt;
	if (!W->sourceType) W->sourceType = 1;
	return S;
}

/* amplitude map A = a * dtdx[i] dtdy[j] dtdz[k] * C[i][j][k]
 * (reference src/source.c:78-84) */
static void amplitudeMap(source S, float *dtdx, float *dtdy, float *dtdz, float ***C, float amplitude)
{
	for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
		S->Amplitude[i][j][k] = amplitude * dtdx[i] * dtdy[j] * dtdz[k] * (C ? C[i][j][k] : 1);
}

/* on a symmetry plane through the source the field parity follows from
 * the dipole orientation (reference src/source.c:91-96) */
static void dipoleParity(world W, field F, int i, int j, int k)
{
	if (W->xMinSur==SYM && !i) W->coskx = stagX(F) ? 1 : -1;
	if (W->yMinSur==SYM && !j) W->cosky = stagY(F) ? 1 : -1;
	if (W->zMinSur==SYM && !k) W->coskz = stagZ(F) ? 1 : -1;
	if (W->xMinSur==SYM && !W->coskx) W->coskx = stagX(F) ? -1 : 1;
	if (W->yMinSur==SYM && !W->cosky) W->cosky = stagY(F) ? -1 : 1;
	if (W->zMinSur==SYM && !W->coskz) W->coskz = stagZ(F) ? -1 : 1;
}

/* Two-cell soft dipole on the nearest Yee edge, normalised so that the
 * radiated power is independent of grid and time step
 * (reference src/source.c:87-124). */
void (pointDipole)(world W, field F, float x, float y, float z, waveform waveForm, float wavelength, float supplement, float amplitude, float phase, ...)
{
	int i = W->xtoi(W, x), j = W->ytoj(W, y), k = W->ztok(W, z);
	dipoleParity(W, F, i, j, k);
	if (waveForm) {
		if (!W->sourceType)
			W->sourceType = (W->Dom.x.Min==W->Dom.x.Max || W->Dom.y.Min==W->Dom.y.Max || W->Dom.z.Min==W->Dom.z.Max) ? 2 : 3;
		source S = newSource(W, F, waveForm, wavelength, supplement, amplitude);
		S->iMin = S->iMax = i, S->jMin = S->jMax = j, S->kMin = S->kMax = k;
		if (stagX(F)) S->iMax++;
		if (stagY(F)) S->jMax++;
		if (stagZ(F)) S->kMax++;
		if (!amplitude) amplitude = 1;
		if      (W->Dom.x.Min==W->Dom.x.Max) amplitude *= W->dx * sqrtf(2.5) * sqrtf(wavelength) / sq(W->dt);
		else if (W->Dom.y.Min==W->Dom.y.Max) amplitude *= W->dy * sqrtf(2.5) * sqrtf(wavelength) / sq(W->dt);
		else if (W->Dom.z.Min==W->Dom.z.Max) amplitude *= W->dz * sqrtf(2.5) * sqrtf(wavelength) / sq(W->dt);
		else amplitude *= sqrtf(1.5 / PI) * wavelength / sq(W->dt);
		S->phase = phase * PI / 180;
		S->Amplitude = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
		coeffs *E = W->CE, *H = W->CH;
		if (F==Ex || F==iEx) amplitudeMap(S, H->dtdx, E->dtdy, E->dtdz, E->x, amplitude*0.5);
		if (F==Ey || F==iEy) amplitudeMap(S, E->dtdx, H->dtdy, E->dtdz, E->y, amplitude*0.5);
		if (F==Ez || F==iEz) amplitudeMap(S, E->dtdx, E->dtdy, H->dtdz, E->z, amplitude*0.5);
		if (F==Hx || F==iHx) amplitudeMap(S, E->dtdx, H->dtdy, H->dtdz, H->x, amplitude*0.25);
		if (F==Hy || F==iHy) amplitudeMap(S, H->dtdx, E->dtdy, H->dtdz, H->y, amplitude*0.25);
		if (F==Hz || F==iHz) amplitudeMap(S, H->dtdx, H->dtdy, E->dtdz, H->z, amplitude*0.25);
	}
	if (wavelength && W->T != wavelength/W->dt) W->f = 1/wavelength, W->T = wavelength/W->dt;
	alis_be_sources_changed(W);
}

/* Guided-mode sources read their mode profile from HDF5, which this
 * build does not include (reference src/source.c:127-220). */
static void guidedUnavailable(void)
{
	fprintf(stderr, "alis: guidedWaveX/Y/Z need HDF5 mode files; unavailable in this build\n");
	exit(1);
}
void (guidedWaveX)(world W, char *file, field F, float x, waveform waveForm, float wavelength, float supplement, float amplitude, float phase, ...)
{ (void)W; (void)file; (void)F; (void)x; (void)waveForm; (void)wavelength; (void)supplement; (void)amplitude; (void)phase; guidedUnavailable(); }
void (guidedWaveY)(world W, char *file, field F, float x, waveform waveForm, float wavelength, float supplement, float amplitude, float phase, ...)
{ (void)W; (void)file; (void)F; (void)x; (void)waveForm; (void)wavelength; (void)supplement; (void)amplitude; (void)phase; guidedUnavailable(); }
void (guidedWaveZ)(world W, char *file, field F, float x, waveform waveForm, float wavelength, float supplement, float amplitude, float phase, ...)
{ (void)W; (void)file; (void)F; (void)x; (void)waveForm; (void)wavelength; (void)supplement; (void)amplitude; (void)phase; guidedUnavailable(); }


/* --- TFSF auxiliary worlds (reference src/source.c:223-334) --- */

/* Re-index a field of the auxiliary world SW so that f[i] is valid for
 * every i of the main world: rows beyond SW's last cell repeat its row
 * SW->iMAX+Alt. */
static float ***aliasRowsX(world W, world SW, float ***g, int Alt)
{
	float ***f;
	MALLOC(f, W->iMIN-1, W->iNUM+2);
	for (int i = SW->iMIN-1; i <= SW->iMAX; i++) f[i] = g[i];
	for (int i = SW->iMAX+1; i <= W->iMAX+1; i++) f[i] = g[SW->iMAX+Alt];
	free(&g[SW->iMIN-1]);
	return f;
}

static float ***aliasRowsY(world W, world SW, float ***g, int Alt)
{
	float ***f;
	MALLOC(f, SW->iMIN-1, SW->iNUM+2);
	MALLOC(f[SW->iMIN-1], W->jMIN-1, (SW->iNUM+2)*(W->jNUM+2));
	for (int i = SW->iMIN-1; i <= SW->iMAX+1; i++) {
		f[i] = f[SW->iMIN-1]+(W->jNUM+2)*(i-SW->iMIN+1);
		for (int j = SW->jMIN-1; j <= SW->jMAX; j++) f[i][j] = g[i][j];
		for (int j = SW->jMAX+1; j <= W->jMAX+1; j++) f[i][j] = g[i][SW->jMAX+Alt];
	}
	free(&g[SW->iMIN-1][SW->jMIN-1]);
	free(&g[SW->iMIN-1]);
	return f;
}

/* layered objects that reach outside the TFSF box also fill the
 * auxiliary world (reference src/source.c:251-266) */
static void auxiliaryObjects(world W, tfsf S, matter *M, object *O)
{
	int N = 0;
	while (O[N].S) N++;
	for (int i = W->iMIN; i <= W->iMAX; i++) for (int j = W->jMIN; j <= W->jMAX; j++) for (int k = W->kMIN; k <= W->kMAX; k++) {
		if (i < S->iMin || S->iMax < i || j < S->jMin || S->jMax < j || k < S->kMin || S->kMax < k) {
			int n = 0;
			float x = W->itox(W, i), y = W->jtoy(W, j), z = W->ktoz(W, k);
			while (O[n].S && !O[n].S(O[n], x, y, z)) n++;
			if (n < N) N = n;
		}
	}
	if (O[N].S || M[N].e.x != 1 || (M[N].e.y && M[N].e.y != 1) || (M[N].e.z && M[N].e.z != 1) || M[N].P->w || M[N].P->g)
		putObjectArray(S->W, M+N, O+N);
}

tfsf (createTFSF)(world W, dom DOM, sur SUR)
{
	tfsf S;
	MALLOC(S, 0, 1);
	tfsf *chain = &W->S;
	while (*chain) chain = &(*chain)->S;
	*chain = S;

	dom Dom = W->Dom;
	sur Sur = SUR;
	if (SUR.x.MinSur==NIL) {
		Dom.x.Min = (W->xMinSur==SYM) ? 0 : W->xMIN;
		Dom.x.Max = (W->xMinSur==SYM) ? 0 : W->itox(W, 1+W->xtoi(W, W->xMIN));
		Sur.x.MinSur = (W->xMinSur==SYM) ? SYM : (W->xMinSur==BBC) ? BBC : PBC;
	}
	if (SUR.y.MinSur==NIL) {
		Dom.y.Min = (W->yMinSur==SYM) ? 0 : W->yMIN;
		Dom.y.Max = (W->yMinSur==SYM) ? 0 : W->jtoy(W, 1+W->ytoj(W, W->yMIN));
		Sur.y.MinSur = (W->yMinSur==SYM) ? SYM : (W->yMinSur==BBC) ? BBC : PBC;
	}
	if (SUR.z.MinSur==NIL) {
		Dom.z.Min = W->ktoz(W, W->ztok(W, W->zMin)-1);
		Dom.z.Max = W->ktoz(W, W->ztok(W, W->zMax)+1);
		Sur.z.MinSur = Sur.z.MaxSur = PML;
	}
	S->W = createWorld(Dom, W->Res, Sur, "");
	strcpy(S->W->ID, W->ID);

	world A = S->W;
	if (SUR.y.MinSur==NIL) for (int n = 0; n <= A->complexField; n++) {
		A->E[n].x = aliasRowsY(W, A, A->E[n].x, 0);
		A->E[n].y = aliasRowsY(W, A, A->E[n].y, 1);
		A->E[n].z = aliasRowsY(W, A, A->E[n].z, 0);
		A->H[n].x = aliasRowsY(W, A, A->H[n].x, 1);
		A->H[n].y = aliasRowsY(W, A, A->H[n].y, 0);
		A->H[n].z = aliasRowsY(W, A, A->H[n].z, 1);
	}
	if (SUR.x.MinSur==NIL) for (int n = 0; n <= A->complexField; n++) {
		A->E[n].x = aliasRowsX(W, A, A->E[n].x, 1);
		A->E[n].y = aliasRowsX(W, A, A->E[n].y, 0);
		A->E[n].z = aliasRowsX(W, A, A->E[n].z, 0);
		A->H[n].x = aliasRowsX(W, A, A->H[n].x, 0);
		A->H[n].y = aliasRowsX(W, A, A->H[n].y, 1);
		A->H[n].z = aliasRowsX(W, A, A->H[n].z, 1);
	}

	/* TFSF box in main-grid indices; the staggered E planes start one
	 * cell in unless the box touches the grid edge */
	if ((!DOM.x.Max && DOM.x.Min>0) || SUR.x.MinSur==SYM) DOM.x.Min = -(DOM.x.Max = DOM.x.Max ? DOM.x.Max : DOM.x.Min);
	if ((!DOM.y.Max && DOM.y.Min>0) || SUR.y.MinSur==SYM) DOM.y.Min = -(DOM.y.Max = DOM.y.Max ? DOM.y.Max : DOM.y.Min);
	if ((!DOM.z.Max && DOM.z.Min>0) || SUR.z.MinSur==SYM) DOM.z.Min = -(DOM.z.Max = DOM.z.Max ? DOM.z.Max : DOM.z.Min);
	S->iMin = W->xMinSur==SYM ? 0 : DOM.x.Min == DOM.x.Max ? W->iMin : W->iMin > W->xtoi(W, DOM.x.Min) ? W->iMIN : W->xtoi(W, DOM.x.Min);
	S->jMin = W->yMinSur==SYM ? 0 : DOM.y.Min == DOM.y.Max ? W->jMin : W->jMin > W->ytoj(W, DOM.y.Min) ? W->jMIN : W->ytoj(W, DOM.y.Min);
	S->kMin = W->zMinSur==SYM ? 0 : DOM.z.Min == DOM.z.Max ? W->kMin : W->kMin > W->ztok(W, DOM.z.Min) ? W->kMIN : W->ztok(W, DOM.z.Min);
	S->iMax = DOM.x.Min == DOM.x.Max ? W->iMax : W->iMax < W->xtoi(W, DOM.x.Max) ? W->iMAX : W->xtoi(W, DOM.x.Max);
	S->jMax = DOM.y.Min == DOM.y.Max ? W->jMax : W->jMax < W->ytoj(W, DOM.y.Max) ? W->jMAX : W->ytoj(W, DOM.y.Max);
	S->kMax = DOM.z.Min == DOM.z.Max ? W->kMax : W->kMax < W->ztok(W, DOM.z.Max) ? W->kMAX : W->ztok(W, DOM.z.Max);
	S->iMIN = (S->iMin == W->iMIN) ? S->iMin : S->iMin + 1, S->iMAX = (S->iMax == W->iMAX) ? S->iMax + 1 : S->iMax;
	S->jMIN = (S->jMin == W->jMIN) ? S->jMin : S->jMin + 1, S->jMAX = (S->jMax == W->jMAX) ? S->jMax + 1 : S->jMax;
	S->kMIN = (S->kMin == W->kMIN) ? S->kMin : S->kMin + 1, S->kMAX = (S->kMax == W->kMAX) ? S->kMax + 1 : S->kMax;

	if (W->CE->M && W->CE->O) auxiliaryObjects(W, S, W->CE->M, W->CE->O);
	alis_be_sources_changed(W);
	return S;
}


/* --- plane-wave source planes (reference src/source.c:337-432) --- */

static void planeSource(world W, field F, int k, float kx, float ky, waveform waveForm, float wavelength, float supplement, float resolution, float amplitude, float phase)
{
	source S = newSource(W, F, waveForm, wavelength, supplement, resolution);
	S->amplitude = amplitude;
	S->phase = phase;
	S->iMin = W->iMIN, S->iMax = W->iMAX, S->jMin = W->jMIN, S->jMax = W->jMAX, S->kMin = k, S->kMax = k;
	if (W->complexField) {
		/* Bloch phase of each staggered sample across the plane */
		float di = (F==Ex||F==Hy||F==iEx||F==iHy) ? 0.5 : 0;
		float dj = (F==Ey||F==Hx||F==iEy||F==iHx) ? 0.5 : 0;
		S->Phase = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
		for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++)
			S->Phase[i][j][k] = phase + kx * W->itox(W, i-di) + ky * W->jtoy(W, j-dj);
	}
}

/* E and H sheets that launch a plane wave of polarisation pol at angles
 * (theta, phi) from the low (theta > 90) or high z edge; with waveForm 0
 * only the Bloch / symmetry phases of W are set */
static void planeSources(world W, tfield pol(phaser,float,float), float theta, float phi, waveform waveForm, float wavelength, float supplement, float resolution, float amplitude, float phase)
{
	int kE = (90<theta && theta<270) ? W->kMin : (theta<90 || 270<theta) ? W->kMax : 0;
	int kH = (90<theta && theta<270) ? W->kMin : (theta<90 || 270<theta) ? W->kMax+1 : 0;
	float sinth = sinf(theta*PI/180) * sqrtf(W->CE->z?1/W->CE->z[W->iMin][W->jMin][kH]:1);
	float costh = cosf(theta*PI/180) * sqrtf(W->CE->z?1/W->CE->z[W->iMin][W->jMin][kH]:1);
	float sinph = sinf(phi*PI/180);
	float cosph = cosf(phi*PI/180);
	float kx = -2 * PI * sinth * cosph / wavelength;
	float ky = -2 * PI * sinth * sinph / wavelength;

	if (W->xMinSur == BBC) W->coskx = cosf(kx*(W->xMax-W->xMin)), W->sinkx = sinf(kx*(W->xMax-W->xMin));
	if (W->yMinSur == BBC) W->cosky = cosf(ky*(W->yMax-W->yMin)), W->sinky = sinf(ky*(W->yMax-W->yMin));
	if ((W->xMinSur == SYM) && (phi==90 || phi==270)) W->coskx = pol==Ppol ? -1 : 1;
	if ((W->xMinSur == SYM) && (phi==0  || phi==180) && (theta==0 || theta==180)) W->coskx = pol==Ppol ? 1 : -1;
	if ((W->yMinSur == SYM) && (phi==0  || phi==180)) W->cosky = pol==Ppol ? -1 : 1;
	if ((W->yMinSur == SYM) && (phi==90 || phi==270) && (theta==0 || theta==180)) W->cosky = pol==Ppol ? 1 : -1;

	if (waveForm) {
		float n = (W->CE->z ? 1/sqrtf(W->CE->z[W->iMin][W->jMin][kH]) : 1);
		float kzdz = W->CE->dz[kE] * PI * fabsf(costh) / wavelength;
		float ampE = W->CE->dtdz[kE] * (amplitude ? amplitude : 1) * 2 / ((1+n) * sqrtf(n) * n);
		float ampH = W->CH->dtdz[kH] * (amplitude ? amplitude : 1) * 2 / ((1+n) * sqrtf(n));
		int notX = phi != 90 && phi != 270, notY = phi != 0 && phi != 180;
		float pE = (phase+90)*PI/180, pH = (phase+90)*PI/180+kzdz;
		float qE = phase*PI/180, qH = phase*PI/180+kzdz;
		if (pol == Ppol) {
			if (notX) planeSource(W, Ex, kE, kx, ky, waveForm, wavelength, supplement, resolution, ampE*cosph*costh, pE);
			if (notY) planeSource(W, Ey, kE, kx, ky, waveForm, wavelength, supplement, resolution, ampE*sinph*costh, pE);
			if (notY) planeSource(W, Hx, kH, kx, ky, waveForm, wavelength, supplement, resolution, ampH*sinph, pH);
			if (notX) planeSource(W, Hy, kH, kx, ky, waveForm, wavelength, supplement, resolution,-ampH*cosph, pH);
			if (W->complexField) {
				if (notX) planeSource(W, iEx, kE, kx, ky, waveForm, wavelength, supplement, resolution, ampE*cosph*costh, qE);
				if (notY) planeSource(W, iEy, kE, kx, ky, waveForm, wavelength, supplement, resolution, ampE*sinph*costh, qE);
				if (notY) planeSource(W, iHx, kH, kx, ky, waveForm, wavelength, supplement, resolution, ampH*sinph, qH);
				if (notX) planeSource(W, iHy, kH, kx, ky, waveForm, wavelength, supplement, resolution,-ampH*cosph, qH);
			}
		}
		if (pol == Spol) {
			if (notY) planeSource(W, Ex, kE, kx, ky, waveForm, wavelength, supplement, resolution,-ampE*sinph, pE);
			if (notX) planeSource(W, Ey, kE, kx, ky, waveForm, wavelength, supplement, resolution, ampE*cosph, pE);
			if (notX) planeSource(W, Hx, kH, kx, ky, waveForm, wavelength, supplement, resolution, ampH*cosph*costh, pH);
			if (notY) planeSource(W, Hy, kH, kx, ky, waveForm, wavelength, supplement, resolution, ampH*sinph*costh, pH);
			if (W->complexField) {
				if (notY) planeSource(W, iEx, kE, kx, ky, waveForm, wavelength, supplement, resolution,-ampE*sinph, qE);
				if (notX) planeSource(W, iEy, kE, kx, ky, waveForm, wavelength, supplement, resolution, ampE*cosph, qE);
				if (notX) planeSource(W, iHx, kH, kx, ky, waveForm, wavelength, supplement, resolution, ampH*cosph*costh, qH);
				if (notY) planeSource(W, iHy, kH, kx, ky, waveForm, wavelength, supplement, resolution, ampH*sinph*costh, qH);
			}
		}
	}
	if (wavelength && W->T != wavelength/W->dt) W->f = 1/wavelength, W->T = wavelength/W->dt;
}

void (planewave)(world W, dom Dom, tfield pol(phaser,float,float), float theta, float phi, waveform waveForm, float wavelength, float supplement, float amplitude, float phase, ...)
{
	while (theta < 0) theta += 360;
	while (theta >= 360) theta -= 360;
	while (phi < 0) phi += 360;
	while (phi >= 360) phi -= 360;
	sur Sur = {{NIL}, {NIL}, {NIL}};
	if ((theta != 0 && theta != 180) && (phi != 90 && phi != 270)) Sur.x.MinSur = BBC;
	if ((theta != 0 && theta != 180) && (phi !=  0 && phi != 180)) Sur.y.MinSur = BBC;
	float resolution = amplitude;
	if (!amplitude) amplitude = 1;
	tfsf S = createTFSF(W, Dom, Sur);
	planeSources(W, pol, theta, phi, 0, wavelength, supplement, resolution, 0, 0);
	planeSources(S->W, pol, theta, phi, waveForm, wavelength, supplement, resolution, amplitude, phase);
	W->N = S->W->N;
	alis_be_sources_changed(S->W);
	alis_be_sources_changed(W);
}


/* --- Gaussian beams (reference src/source.c:435-496) --- */

static void beam(world W, field F, float x, float y, float z, float theta, waveform waveForm, float wavelength, float supplement, float spotsize, float amplitude, float phase)
{
	while (theta < 0) theta += 360;
	while (theta >= 360) theta -= 360;
	if (W->xMinSur==SYM) W->coskx = (F==Ex || F==iEx) ? 1 : -1;
	if (W->yMinSur==SYM) W->cosky = (F==Ey || F==iEy) ? 1 : -1;
	if (waveForm) {
		int k = (90<theta && theta<270) ? W->kMin : (theta<90 || 270<theta) ? W->kMax : 0;
		float n = W->CE->z ? 1/sqrtf(W->CE->z[W->xtoi(W,MIN(x,W->xMax))][W->ytoj(W,MIN(y,W->yMax))][k]) : 1;
		source S = newSource(W, F, waveForm, wavelength, supplement, amplitude);
		S->iMin = W->iMIN, S->iMax = W->iMAX, S->jMin = W->jMIN, S->jMax = W->jMAX, S->kMin = k, S->kMax = k;
		if (!amplitude) amplitude = 1;
		amplitude /= sqrtf(n*n*n);
		if (spotsize) {
			float kz = 2 * PI * n / wavelength;
			float zz = fabsf(z - W->ktoz(W,k));
			float w0 = wavelength * (spotsize ? spotsize : 1) / (n * sqrtf(-2.0 * logf(0.5)));
			float z0 = PI * n * sq(w0) / wavelength;
			float wz = w0 * sqrtf(1 + sq(zz/z0));
			float Rz = zz * (1 + sq(z0/zz));
			float nz = atanf(zz/z0);
			S->Amplitude = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
			S->Phase = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
			for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) {
				float r2 = 0;
				if (x < INF) r2 += sq(x - W->itox(W,F==Ex?i-0.5:i));
				if (y < INF) r2 += sq(y - W->jtoy(W,F==Ey?j-0.5:j));
				S->Amplitude[i][j][k] = amplitude * w0/wz * expf(-r2/sq(wz));
				S->Phase[i][j][k] = phase * PI / 180 - kz * (0.5 * r2 / Rz) + nz;
			}
		} else {
			S->amplitude = amplitude;
			S->phase = phase * PI / 180;
		}
	}
	if (wavelength && W->T != wavelength/W->dt) W->f = 1/wavelength, W->T = wavelength/W->dt;
}

void (focusedBeam)(world W, dom Dom, field F, float x, float y, float z, float theta, waveform waveForm, float wavelength, float supplement, float spotsize, float amplitude, float phase, ...)
{
	if (Dom.x.Min==W->Dom.x.Min && Dom.x.Max==W->Dom.x.Max &&
	    Dom.y.Min==W->Dom.y.Min && Dom.y.Max==W->Dom.y.Max &&
	    Dom.z.Min==W->Dom.z.Min && Dom.z.Max==W->Dom.z.Max) {
		beam(W, F, x, y, z, theta, waveForm, wavelength, supplement, spotsize, amplitude, phase);
	} else {
		sur Sur = {{NIL}, {NIL}, {NIL}};
		if (x < INF) Sur.x.MinSur = W->Sur.x.MinSur, Sur.x.MaxSur = W->Sur.x.MaxSur;
		if (y < INF) Sur.y.MinSur = W->Sur.y.MinSur, Sur.y.MaxSur = W->Sur.y.MaxSur;
		tfsf S = createTFSF(W, Dom, Sur);
		beam(W, F, x, y, z, theta, 0, wavelength, supplement, 0, 0, 0);
		beam(S->W, F, x, y, z, theta, waveForm, wavelength, supplement, spotsize, amplitude, phase);
		W->N = S->W->N;
		alis_be_sources_changed(S->W);
	}
	alis_be_sources_changed(W);
}


/* --- removal (reference src/source.c:499-524) --- */

static void freeSource(source S)
{
	if (S->S) freeSource(S->S);
	if (S->Amplitude) removeField(S->Amplitude, S->iMin, S->jMin, S->kMin);
	if (S->Phase) removeField(S->Phase, S->iMin, S->jMin, S->kMin);
	free(S);
}

static void freeTFSF(tfsf S)
{
	if (S->S) freeTFSF(S->S);
	deleteWorld(S->W);
	free(S);
}

void removeSources(world W)
{
	if (W->SE) freeSource(W->SE), W->SE = 0;
	if (W->SH) freeSource(W->SH), W->SH = 0;
	if (W->S) freeTFSF(W->S), W->S = 0;
	W->f = 0;
	W->T = 0;
	W->N = 0;
	alis_be_sources_changed(W);
}

/* 1 when source S adds to its field in the current half step
 * (reference src/update.c:163) */
int alis_source_active(world W, source S)
{
	return W->n < S->N;
}
