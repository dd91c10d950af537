/*
 * gpu_backend.c -- the GPU stepping backend behind the ALiS API.
 *
 * Implements updateE / updateH / updatePhaser and the engine hooks of
 * engine.h by translating the host data model (struct world, sources,
 * TFSF boxes, phasers) into calls of the device C-ABI (alisgpu.h).
 * Live state is in HBM; host arrays are mirrors refreshed on demand.
 *
 * Per half step (reference src/update.c:275-341) the host evaluates the
 * source waveforms with the same C library calls as the reference, lists
 * the boundary ghost copies with the world's current Bloch/symmetry
 * factors, and issues one alisgpu_half_step_run per world (the main
 * world, then each TFSF auxiliary world).  Time bookkeeping (n, t, E->t,
 * H->t) is done here exactly as in the reference.
 */
#include <stdint.h>
#include <string.h>
#include "engine.h"
#include "alisgpu.h"

int alis_needs_currents(matter M);
void alisgpu__forget_tfsf(const alisgpu_tfsf *s);

#define MAX_TFSF 4
#define MAX_GHOST 24

typedef struct devWorld {
	world W;
	alisgpu_world *dw;
	int ownStreams;           /* W (and its auxiliary worlds) on streams of their own */
	int objectsDirty;         /* eps maps / dispersive objects need upload */
	int hostStale;            /* device ahead of the host mirrors */
	int ntf;
	alisgpu_tfsf tf[MAX_TFSF];
	int isAux;                /* the auxiliary world of a TFSF box */
	int stepped;              /* has taken a half step */
	struct devWorld *next;
} devWorld;

typedef struct devPhaser {
	phaser P;                 /* first element of the set */
	int nfreq, nface;
	int faceSlot[6];          /* cfield index (0..5: xMin,xMax,yMin,yMax,zMin,zMax) of each device face */
	alisgpu_phaser *dp;
	int hostStale;
	int fluxStale;            /* face fluxes behind the accumulators */
	float *flux;              /* [nfreq][6] face fluxes by cfield slot */
	float *phE, *phH;
	struct devPhaser *next;
} devPhaser;

/* Host threads may step different worlds at once (creation and deletion
 * stay on one thread): the lookup cache and the per-call staging are per
 * thread. */
static devWorld *worlds;
static _Thread_local devWorld *lastWorld;
/* deletions so far: a thread's cached lookup is stale after one */
static unsigned long worldsDeleted;
static _Thread_local unsigned long lastWorldEpoch;
static devPhaser *phasers;

/* a sliceFreqDom accumulator on the device; h is 0 once its world is gone */
typedef struct devSliceDft {
	devWorld *d;
	alisgpu_slice_dft *h;
	struct devSliceDft *next;
} devSliceDft;
static devSliceDft *sliceDfts;

static void die(const char *what, int rc)
{
	fprintf(stderr, "alis: %s failed (%d): %s\n", what, rc, alisgpu_last_error());
	exit(1);
}
#define CHECK(what, call) do { int rc_ = (call); if (rc_) die(what, rc_); } while (0)

static devWorld *findWorld(world W)
{
	if (lastWorld && lastWorldEpoch == worldsDeleted && lastWorld->W == W) return lastWorld;
	for (devWorld *d = worlds; d; d = d->next)
		if (d->W == W) {
			lastWorldEpoch = worldsDeleted;
			return lastWorld = d;
		}
	return 0;
}

static devPhaser *findPhaser(phaser P)
{
	for (devPhaser *d = phasers; d; d = d->next) if (P >= d->P && P < d->P + d->nfreq) return d;
	return 0;
}

/* ---- world lifecycle ---- */

static void uploadLineTables(devWorld *d)
{
	world W = d->W;
	for (int grid = 0; grid < 2; grid++) {
		coeffs *C = grid ? W->CH : W->CE;
		const float *dtd[3] = { &C->dtdx[W->iMIN], &C->dtdy[W->jMIN], &C->dtdz[W->kMIN] };
		const float *cp[9] = {
			C->xP ? &C->xP[W->iMIN] : 0, C->xPy ? &C->xPy[W->iMIN] : 0, C->xPz ? &C->xPz[W->iMIN] : 0,
			C->yP ? &C->yP[W->jMIN] : 0, C->yPz ? &C->yPz[W->jMIN] : 0, C->yPx ? &C->yPx[W->jMIN] : 0,
			C->zP ? &C->zP[W->kMIN] : 0, C->zPx ? &C->zPx[W->kMIN] : 0, C->zPy ? &C->zPy[W->kMIN] : 0 };
		CHECK("set_line_tables", alisgpu_set_line_tables(d->dw, grid, dtd, cp));
	}
	const float *dE[3] = { &W->CE->dx[W->iMIN], &W->CE->dy[W->jMIN], &W->CE->dz[W->kMIN] };
	const float *dH[3] = { &W->CH->dx[W->iMIN], &W->CH->dy[W->jMIN], &W->CH->dz[W->kMIN] };
	CHECK("set_spacing", alisgpu_set_spacing(d->dw, dE, dH));
}

void alis_be_world_created(world W)
{
	CHECK("init", alisgpu_init());
	devWorld *d = calloc(1, sizeof *d);
	d->W = W;
	alisgpu_geometry g = {
		W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMIN, W->kMAX,
		W->iMin, W->iMax, W->jMin, W->jMax, W->kMin, W->kMax,
		W->complexField,
		{ W->xMinSur==PML, W->yMinSur==PML, W->zMinSur==PML, W->xMaxSur==PML, W->yMaxSur==PML, W->zMaxSur==PML } };
	CHECK("world_create", alisgpu_world_create(&g, &d->dw));
	uploadLineTables(d);
	d->next = worlds;
	worlds = d;
}

void alis_be_world_deleted(world W)
{
	devWorld **pp = &worlds;
	while (*pp && (*pp)->W != W) pp = &(*pp)->next;
	if (!*pp) return;
	devWorld *d = *pp;
	*pp = d->next;
	if (lastWorld == d) lastWorld = 0;
	worldsDeleted++;
	for (devSliceDft *s = sliceDfts; s; s = s->next)
		if (s->d == d) alisgpu_slice_dft_destroy(s->h), s->h = 0, s->d = 0;
	for (int q = 0; q < d->ntf; q++) alisgpu__forget_tfsf(&d->tf[q]);
	alisgpu_world_destroy(d->dw);
	free(d);
}

void alis_be_objects_changed(world W)
{
	devWorld *d = findWorld(W);
	if (d) d->objectsDirty = 1;
}

static void buildTfsf(devWorld *d);

void alis_be_sources_changed(world W)
{
	devWorld *d = findWorld(W);
	if (d) buildTfsf(d);
}

void alis_be_world_reset(world W)
{
	devWorld *d = findWorld(W);
	if (!d) return;
	CHECK("world_reset", alisgpu_world_reset(d->dw));
	d->hostStale = 0;
}

/* eps^-1 maps and dispersive objects (reference src/object.c:339-405) */
static void uploadObjects(devWorld *d)
{
	world W = d->W;
	coeffs *C = W->CE;
	if (C->x) CHECK("set_eps", alisgpu_set_eps(d->dw, &C->x[W->iMIN][W->jMIN][W->kMIN], &C->y[W->iMIN][W->jMIN][W->kMIN], &C->z[W->iMIN][W->jMIN][W->kMIN]));
	else CHECK("set_eps", alisgpu_set_eps(d->dw, 0, 0, 0));
	alisgpu_dispersive *o = calloc(C->N ? C->N : 1, sizeof *o);
	for (int n = 0; n < C->N; n++) {
		o[n].iMin = C->iMin[n], o[n].iMax = C->iMax[n], o[n].jMin = C->jMin[n], o[n].jMax = C->jMax[n];
		o[n].kMin = C->kMin[n], o[n].kMax = C->kMax[n];
		o[n].NJ = C->NJ[n], o[n].NK = C->NK[n];
		float ****fill[3] = { C->Jx, C->Jy, C->Jz };
		float *a[3] = { C->ax, C->ay, C->az };
		float **JJ[3] = { C->JJx, C->JJy, C->JJz }, **JK[3] = { C->JKx, C->JKy, C->JKz }, **JE[3] = { C->JEx, C->JEy, C->JEz };
		float **KJ[3] = { C->KJx, C->KJy, C->KJz }, **KK[3] = { C->KKx, C->KKy, C->KKz }, **KE[3] = { C->KEx, C->KEy, C->KEz };
		for (int q = 0; q < 3; q++) {
			o[n].fill[q] = &fill[q][n][C->iMin[n]][C->jMin[n]][C->kMin[n]];
			o[n].a[q] = a[q][n];
			o[n].JJ[q] = JJ[q][n], o[n].JK[q] = JK[q][n], o[n].JE[q] = JE[q][n];
			o[n].KJ[q] = KJ[q][n], o[n].KK[q] = KK[q][n], o[n].KE[q] = KE[q][n];
		}
	}
	CHECK("set_dispersive", alisgpu_set_dispersive(d->dw, C->N, o));
	free(o);
	d->objectsDirty = 0;
}

/* TFSF boxes of W with their auxiliary worlds (reference src/source.c:269-334) */
static void buildTfsf(devWorld *d)
{
	world W = d->W;
	for (int q = 0; q < d->ntf; q++) alisgpu__forget_tfsf(&d->tf[q]);
	d->ntf = 0;
	for (tfsf S = W->S; S; S = S->S) {
		if (d->ntf == MAX_TFSF) { fprintf(stderr, "alis: more than %d TFSF sources\n", MAX_TFSF); exit(1); }
		devWorld *a = findWorld(S->W);
		if (!a) continue;
		alisgpu_tfsf *t = &d->tf[d->ntf++];
		memset(t, 0, sizeof *t);
		t->aux = a->dw;
		a->isAux = 1;
		t->iMin = S->iMin, t->iMax = S->iMax, t->jMin = S->jMin, t->jMax = S->jMax, t->kMin = S->kMin, t->kMax = S->kMax;
		t->iMIN = S->iMIN, t->iMAX = S->iMAX, t->jMIN = S->jMIN, t->jMAX = S->jMAX, t->kMIN = S->kMIN, t->kMAX = S->kMAX;
		t->auxIMAX = S->W->iMAX, t->auxJMAX = S->W->jMAX;
		/* rows were aliased when the auxiliary world is narrower than W */
		t->aliasX = S->W->iMAX < W->iMAX + 1 && S->W->iNUM < W->iNUM;
		t->aliasY = S->W->jMAX < W->jMAX + 1 && S->W->jNUM < W->jNUM;
	}
}

/* ---- host mirrors ---- */

static void downloadCurrents(devWorld *d, int n);

static void downloadWorld(devWorld *d)
{
	world W = d->W;
	CHECK("synchronize", alisgpu_synchronize());
	for (int m = 0; m <= W->complexField; m++) {
		float ***E[3] = { W->E[m].x, W->E[m].y, W->E[m].z }, ***H[3] = { W->H[m].x, W->H[m].y, W->H[m].z };
		for (int c = 0; c < 3; c++) {
			CHECK("field_download", alisgpu_field_download(d->dw, 0, m, c, &E[c][W->iMIN-1][W->jMIN-1][W->kMIN-1]));
			CHECK("field_download", alisgpu_field_download(d->dw, 1, m, c, &H[c][W->iMIN-1][W->jMIN-1][W->kMIN-1]));
		}
	}
	for (int n = 0; n < W->CE->N; n++) downloadCurrents(d, n);
	d->hostStale = 0;
}

static _Thread_local world heldWorld;

void alis_be_hold_sync(world W) { heldWorld = W; }

void alis_be_sync_world(world W)
{
	if (W == heldWorld) return;
	devWorld *d = findWorld(W);
	if (d && d->hostStale) downloadWorld(d);
}

/* index range of the cells field functions evaluated over [lo, hi] read:
 * +-2, and across a symmetry plane the mirrored cells as well */
static void nearRange(int lo, int hi, int sym, int lo0, int hi0, int *a, int *b)
{
	lo -= 2, hi += 2;
	if (sym && lo < 0) hi = MAX(hi, 3 - lo);
	*a = MAX(lo, lo0), *b = MIN(hi, hi0);
}

/* currents of dispersive object n into the host mirrors (one transfer) */
static void downloadCurrents(devWorld *d, int n)
{
	world W = d->W;
	coeffs *C = W->CE;
	size_t cells = (size_t)(1 + C->iMax[n] - C->iMin[n]) * (1 + C->jMax[n] - C->jMin[n]) * (1 + C->kMax[n] - C->kMin[n]);
	size_t arrays = (size_t)(1 + W->complexField) * 3 * (2 * C->NK[n] - C->NJ[n]);
	if (!cells || !arrays) return;
	float *buf = malloc(cells * arrays * sizeof(float)), *src = buf;
	CHECK("object_currents_download", alisgpu_object_currents_download(d->dw, n, buf));
	for (int m = 0; m <= W->complexField; m++) {
		float *****J[3] = { W->E[m].Jx, W->E[m].Jy, W->E[m].Jz }, *****K[3] = { W->E[m].Kx, W->E[m].Ky, W->E[m].Kz };
		for (int p = 0; p < C->NK[n]; p++) for (int c = 0; c < 3; c++) {
			memcpy(&J[c][n][p][C->iMin[n]][C->jMin[n]][C->kMin[n]], src, cells * sizeof(float)), src += cells;
			if (p >= C->NJ[n]) memcpy(&K[c][n][p][C->iMin[n]][C->jMin[n]][C->kMin[n]], src, cells * sizeof(float)), src += cells;
		}
	}
	free(buf);
}

int alis_be_sync_box(world W, int bi0, int bi1, int bj0, int bj1, int bk0, int bk1)
{
	devWorld *d = findWorld(W);
	if (!d) return 0;
	if (!d->hostStale) return 1;
	int i0, i1, j0, j1, k0, k1;
	nearRange(MIN(bi0, bi1), MAX(bi0, bi1), W->xMinSur==SYM, W->iMIN-1, W->iMAX+1, &i0, &i1);
	nearRange(MIN(bj0, bj1), MAX(bj0, bj1), W->yMinSur==SYM, W->jMIN-1, W->jMAX+1, &j0, &j1);
	nearRange(MIN(bk0, bk1), MAX(bk0, bk1), W->zMinSur==SYM, W->kMIN-1, W->kMAX+1, &k0, &k1);
	if (i1 < i0 || j1 < j0 || k1 < k0) return 0;
	int ni = 1 + i1 - i0, nj = 1 + j1 - j0, nk = 1 + k1 - k0, nm = 1 + W->complexField;
	size_t cells = (size_t)ni * nj * nk;
	/* most of the world: one whole download is cheaper */
	if (cells * 2 > (size_t)(W->iNUM + 2) * (W->jNUM + 2) * (W->kNUM + 2)) return 0;
	float *buf = malloc(cells * 6 * nm * sizeof(float));
	CHECK("field_box_download", alisgpu_field_box_download(d->dw, i0, i1, j0, j1, k0, k1, buf));
	for (int f = 0; f < 2; f++) for (int m = 0; m < nm; m++) {
		vfield *V = f ? &W->H[m] : &W->E[m];
		float ***A[3] = { V->x, V->y, V->z };
		for (int c = 0; c < 3; c++) {
			const float *src = buf + ((size_t)(f * nm + m) * 3 + c) * cells;
			for (int a = 0; a < ni; a++) for (int b = 0; b < nj; b++)
				memcpy(&A[c][i0+a][j0+b][k0], src + ((size_t)a * nj + b) * nk, nk * sizeof(float));
		}
	}
	free(buf);
	coeffs *C = W->CE;
	for (int n = 0; n < C->N; n++)
		if (C->iMin[n] <= i1 && i0 <= C->iMax[n] && C->jMin[n] <= j1 && j0 <= C->jMax[n] && C->kMin[n] <= k1 && k0 <= C->kMax[n])
			downloadCurrents(d, n);
	return 1;
}

int alis_be_sync_near(world W, int i, int j, int k)
{
	return alis_be_sync_box(W, i, i, j, j, k, k);
}

/* ---- half steps ---- */

typedef struct {
	alisgpu_source_patch p[64];
	int n;
	float *v;
	int nv, cap;
} patchList;

static _Thread_local patchList srcList;

/* E or H field set and component a source writes to */
static int sourceTarget(world W, source S, int field, int *m, int *comp)
{
	for (int q = 0; q <= W->complexField; q++) {
		vfield *V = field ? &W->H[q] : &W->E[q];
		float ***c[3] = { V->x, V->y, V->z };
		for (int a = 0; a < 3; a++) if (S->F == c[a]) { *m = q, *comp = a; return 1; }
	}
	return 0;
}

/* per-cell increments of the active sources of a chain, in chain order
 * (reference src/update.c:161-179) */
static void collectSources(world W, source S, int field, float t)
{
	srcList.n = 0, srcList.nv = 0;
	for (; S; S = S->S) {
		if (!(W->n < S->N)) continue;
		int m, comp;
		if (!sourceTarget(W, S, field, &m, &comp)) continue;
		int cells = (1+S->iMax-S->iMin)*(1+S->jMax-S->jMin)*(1+S->kMax-S->kMin);
		if (srcList.nv + cells > srcList.cap) {
			srcList.cap = 2*(srcList.nv + cells);
			srcList.v = realloc(srcList.v, srcList.cap * sizeof(float));
		}
		if (srcList.n == 64) { fprintf(stderr, "alis: more than 64 active sources on one field\n"); exit(1); }
		alisgpu_source_patch *p = &srcList.p[srcList.n++];
		*p = (alisgpu_source_patch){ m, comp, S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax, srcList.nv };
		float *v = srcList.v + srcList.nv;
		int q = 0;
		if (S->Phase) {
			for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
				v[q++] = (S->Amplitude ? S->Amplitude[i][j][k] : S->amplitude) * S->waveForm(W, S, t, S->Phase[i][j][k]);
		} else {
			float f = S->waveForm(W, S, t, S->phase);
			for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
				v[q++] = S->Amplitude ? S->Amplitude[i][j][k] * f : S->amplitude * f;
		}
		srcList.nv += cells;
	}
}

static int ghostList(world W, int field, alisgpu_ghost_copy *g)
{
	int n = 0;
	int iAlt = (W->xMinSur==PBC || W->xMinSur==BBC ? W->iNUM-1 : 1);
	int jAlt = (W->yMinSur==PBC || W->yMinSur==BBC ? W->jNUM-1 : 1);
	int kAlt = (W->zMinSur==PBC || W->zMinSur==BBC ? W->kNUM-1 : 1);
#define G(c, co, si, i0, i1, j0, j1, k0, k1, di, dj, dk) g[n++] = (alisgpu_ghost_copy){ c, i0, i1, j0, j1, k0, k1, di, dj, dk, co, si }
	if (field == 0) {
		/* reference src/update.c:284-297 */
		G(0, W->coskx, -W->sinkx, W->iMAX+1, W->iMAX+1, W->jMIN, W->jMAX, W->kMIN, W->kMAX, -iAlt, 0, 0);
		G(2, W->coskz, -W->sinkz, W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMAX+1, W->kMAX+1, 0, 0, -kAlt);
		if (W->yMinSur==HBC) {
			G(1, W->coskym, -W->sinkym, W->iMIN, 0, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMAX, 1-W->jNUM, 0);
			G(1, W->coskyp, -W->sinkyp, 1, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMIN, 1-W->jNUM, 0);
		} else {
			G(1, W->cosky, -W->sinky, W->iMIN, W->iMAX, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, 0, -jAlt, 0);
		}
	} else {
		/* reference src/update.c:311-339 */
		G(1, W->xMaxSur==PEC?1:W->coskx, -W->sinkx, W->iMAX+1, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, -iAlt, 0, 0);
		G(2, W->xMaxSur==PEC?1:W->coskx, -W->sinkx, W->iMAX+1, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, -iAlt, 0, 0);
		G(0, W->zMaxSur==PEC?1:W->coskz, -W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMAX+1, W->kMAX+1, 0, 0, -kAlt);
		G(1, W->zMaxSur==PEC?1:W->coskz, -W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMAX+1, W->kMAX+1, 0, 0, -kAlt);
		G(1, W->coskx, W->sinkx, W->iMIN, W->iMIN, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, iAlt, 0, 0);
		G(2, W->coskx, W->sinkx, W->iMIN, W->iMIN, W->jMIN, W->jMAX+1, W->kMIN, W->kMAX+1, iAlt, 0, 0);
		G(0, W->coskz, W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMIN, 0, 0, kAlt);
		G(1, W->coskz, W->sinkz, W->iMIN, W->iMAX+1, W->jMIN, W->jMAX+1, W->kMIN, W->kMIN, 0, 0, kAlt);
		if (W->yMinSur==HBC) {
			G(0, W->coskyp, W->sinkyp, W->iMIN, 0, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMAX, W->jNUM-1, 0);
			G(2, W->coskyp, W->sinkyp, W->iMIN, 0, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMAX, W->jNUM-1, 0);
			G(0, W->coskym, -W->sinkym, W->iMIN, 0, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMAX, 1-W->jNUM, 0);
			G(2, W->coskym, -W->sinkym, W->iMIN, 0, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMAX, 1-W->jNUM, 0);
			G(0, W->coskym, W->sinkym, 1, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMIN, W->jNUM-1, 0);
			G(2, W->coskym, W->sinkym, 1, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX, W->iMIN, W->jNUM-1, 0);
			G(0, W->coskyp, -W->sinkyp, 1, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMIN, 1-W->jNUM, 0);
			G(2, W->coskyp, -W->sinkyp, 1, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX, W->iMIN, 1-W->jNUM, 0);
		} else {
			G(2, W->yMaxSur==PEC?1:W->cosky, -W->sinky, W->iMIN, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX+1, 0, -jAlt, 0);
			G(0, W->yMaxSur==PEC?1:W->cosky, -W->sinky, W->iMIN, W->iMAX+1, W->jMAX+1, W->jMAX+1, W->kMIN, W->kMAX+1, 0, -jAlt, 0);
			G(2, W->cosky, W->sinky, W->iMIN, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX+1, 0, jAlt, 0);
			G(0, W->cosky, W->sinky, W->iMIN, W->iMAX+1, W->jMIN, W->jMIN, W->kMIN, W->kMAX+1, 0, jAlt, 0);
		}
	}
#undef G
	return n;
}

/* the auxiliary worlds of a world with streams of its own share them */
static void shareStreams(devWorld *d)
{
	for (tfsf S = d->W->S; S; S = S->S) {
		devWorld *a = findWorld(S->W);
		if (a) CHECK("world_share_streams", alisgpu_world_share_streams(a->dw, d->dw));
	}
}

void alis_be_world_streams(world W)
{
	devWorld *d = findWorld(W);
	if (!d) return;
	CHECK("world_own_streams", alisgpu_world_own_streams(d->dw));
	d->ownStreams = 1;
	shareStreams(d);
}

/* FP16 field storage of the worlds the user steps (ALIS_FIELD_STORAGE=half;
 * their TFSF auxiliary worlds, and worlds with complex fields, stay
 * float): set before a world's first half step, see
 * alisgpu_world_set_storage */
static int halfStorage(void)
{
	static int on = -1;
	if (on < 0) {
		const char *e = getenv("ALIS_FIELD_STORAGE");
		on = e && !strcmp(e, "half");
	}
	return on;
}

static void halfStepAs(world W, int field, int attach)
{
	devWorld *d = findWorld(W);
	if (!d) { fprintf(stderr, "alis: world unknown to the GPU backend\n"); exit(1); }
	if (!d->stepped && !d->isAux && !W->complexField && halfStorage())
		CHECK("world_set_storage", alisgpu_world_set_storage(d->dw, ALISGPU_STORAGE_HALF));
	d->stepped = 1;
	if (d->ownStreams) shareStreams(d);
	if (d->objectsDirty) uploadObjects(d);
	alisgpu_ghost_copy g[MAX_GHOST];
	alisgpu_half_step s;
	memset(&s, 0, sizeof s);
	s.field = field;
	s.ntfsf = d->ntf;
	s.tfsf = d->tf;
	collectSources(W, field ? W->SH : W->SE, field, field ? W->E->t : W->H->t);
	s.nsrc = srcList.n;
	s.src = srcList.p;
	s.values = srcList.v;
	s.nvalues = srcList.nv;
	s.nghost = ghostList(W, field, g);
	s.ghost = g;
	s.concurrent = d->isAux;
	s.attach = attach;
	CHECK("half_step", alisgpu_half_step_run(d->dw, &s));
	d->hostStale = 1;
}

static void halfStep(world W, int field) { halfStepAs(W, field, 0); }

/* A world with one TFSF box whose auxiliary world has no box of its own:
 * the auxiliary half step is handed over first and runs inside the
 * world's own launch of the same field (the device falls back to a launch
 * of its own when it cannot).  That saves a launch and four event
 * operations per half step, which pays where launches are the limit --
 * worlds on streams of their own, stepped in turn with others -- and on
 * large worlds; a small world stepped alone loses more to the larger
 * launch (measured on 32 periodic unit cells: 11.6 against 9.4 Gcell/s
 * one after another, 25.4 against 21.3 served).  ALISGPU_AUX_ATTACH=0
 * turns it off, =2 turns it on for every world. */
static __thread int batchOn;

static int attachAux(world W)
{
	static int enabled = -1;
	if (enabled < 0) {
		const char *e = getenv("ALISGPU_AUX_ATTACH");
		enabled = e ? atoi(e) : 1;
	}
	if (!enabled || !W->S || W->S->S || !W->S->W || W->S->W->S || !findWorld(W->S->W)) return 0;
	devWorld *d = findWorld(W);
	return d && (enabled == 2 || batchOn || d->ownStreams || (long)W->iNUM * W->jNUM * W->kNUM >= (1L << 22));
}

/* batched launches over the worlds this thread steps (alisBatchBegin):
 * their TFSF auxiliary columns always ride in the parent's entry */
void alis_be_batch(int begin)
{
	if (begin) {
		CHECK("batch_begin", alisgpu_batch_begin());
		batchOn = 1;
	} else {
		batchOn = 0;
		CHECK("batch_end", alisgpu_batch_end());
	}
}

/* reference src/update.c:275-299 */
void updateE(world W)
{
	if (attachAux(W)) {
		world A = W->S->W;
		halfStepAs(A, 0, 1);
		halfStep(W, 0);
		A->t = A->E->t = ++A->n * A->dt;
	} else {
		halfStep(W, 0);
		for (tfsf S = W->S; S; S = S->S) updateE(S->W);
	}
	W->t = W->E->t = ++W->n * W->dt;
}

/* reference src/update.c:302-341 */
void updateH(world W)
{
	if (attachAux(W)) {
		world A = W->S->W;
		halfStepAs(A, 1, 1);
		halfStep(W, 1);
		A->t = A->H->t = A->E->t + 0.5 * A->dt;
	} else {
		halfStep(W, 1);
		for (tfsf S = W->S; S; S = S->S) updateH(S->W);
	}
	W->t = W->H->t = W->E->t + 0.5 * W->dt;
}


/* ---- phasers ---- */

static int phaserRing(void)
{
	const char *e = getenv("ALISGPU_PHASER_RING");
	int r = e ? atoi(e) : 64;
	return r > 0 ? r : 64;
}

void alis_be_phaser_created(phaser P)
{
	devPhaser *d = calloc(1, sizeof *d);
	d->P = P;
	while (P[d->nfreq].f) d->nfreq++;
	world W = P->W;
	devWorld *dw = findWorld(W);
	if (!dw) { fprintf(stderr, "alis: phaser on a world unknown to the GPU backend\n"); exit(1); }
	alisgpu_face faces[6];
	cfield *cf[6] = { &P->xMin, &P->xMax, &P->yMin, &P->yMax, &P->zMin, &P->zMax };
	int boxes[6][6] = {
		{ P->iMin, P->iMin, P->jMin, P->jMax, P->kMin, P->kMax }, { P->iMax, P->iMax, P->jMin, P->jMax, P->kMin, P->kMax },
		{ P->iMin, P->iMax, P->jMin, P->jMin, P->kMin, P->kMax }, { P->iMin, P->iMax, P->jMax, P->jMax, P->kMin, P->kMax },
		{ P->iMin, P->iMax, P->jMin, P->jMax, P->kMin, P->kMin }, { P->iMin, P->iMax, P->jMin, P->jMax, P->kMax, P->kMax } };
	for (int s = 0; s < 6; s++) {
		int axis = s / 2;
		int present = axis == 0 ? cf[s]->Ey != 0 : axis == 1 ? cf[s]->Ez != 0 : cf[s]->Ex != 0;
		if (!present) continue;
		faces[d->nface] = (alisgpu_face){ axis, boxes[s][0], boxes[s][1], boxes[s][2], boxes[s][3], boxes[s][4], boxes[s][5] };
		d->faceSlot[d->nface++] = s;
	}
	const char *k = getenv("ALISGPU_PHASER_KAHAN");
	CHECK("phaser_create", alisgpu_phaser_create(dw->dw, d->nfreq, d->nface, faces, phaserRing(), k && k[0] == '1', &d->dp));
	d->phE = calloc(2 * d->nfreq, sizeof(float));
	d->phH = calloc(2 * d->nfreq, sizeof(float));
	d->flux = calloc((size_t)6 * d->nfreq, sizeof(float));
	d->fluxStale = 1;
	d->next = phasers;
	phasers = d;
}

void alis_be_phaser_deleted(phaser P)
{
	devPhaser **pp = &phasers;
	while (*pp && (*pp)->P != P) pp = &(*pp)->next;
	if (!*pp) return;
	devPhaser *d = *pp;
	*pp = d->next;
	alisgpu_phaser_destroy(d->dp);
	free(d->phE);
	free(d->phH);
	free(d->flux);
	free(d);
}

/* phase factors of every frequency of the set, as the reference computes
 * them per call (src/phaser.c:97-98); frequencies before P are skipped */
/* the phase factors last computed by this thread, with what they were
 * computed from: worlds of a sweep share their frequencies and times */
#define PHASE_MEMO 512
static _Thread_local struct {
	int nfreq, first;
	float tE, tH;
	float f[PHASE_MEMO];
	float phE[2 * PHASE_MEMO], phH[2 * PHASE_MEMO];
} phaseMemo;

void updatePhaser(world W, phaser P)
{
	devPhaser *d = findPhaser(P);
	if (!d) { fprintf(stderr, "alis: updatePhaser on an unknown phaser\n"); exit(1); }
	int first = (int)(P - d->P);
	int same = d->nfreq <= PHASE_MEMO && phaseMemo.nfreq == d->nfreq && phaseMemo.first == first &&
	           !memcmp(&phaseMemo.tE, &W->E->t, sizeof(float)) && !memcmp(&phaseMemo.tH, &W->H->t, sizeof(float));
	for (int n = 0; same && n < d->nfreq; n++) same = !memcmp(&phaseMemo.f[n], &d->P[n].f, sizeof(float));
	if (same) {
		memcpy(d->phE, phaseMemo.phE, 2 * d->nfreq * sizeof(float));
		memcpy(d->phH, phaseMemo.phH, 2 * d->nfreq * sizeof(float));
	} else {
		for (int n = 0; n < d->nfreq; n++) {
			float complex pE = 0, pH = 0;
			if (n >= first) {
				pE = cexpf(2 * PI * I * d->P[n].f * W->E->t);
				pH = cexpf(2 * PI * I * d->P[n].f * W->H->t);
			}
			d->phE[2*n] = crealf(pE), d->phE[2*n+1] = cimagf(pE);
			d->phH[2*n] = crealf(pH), d->phH[2*n+1] = cimagf(pH);
		}
		if (d->nfreq <= PHASE_MEMO) {
			phaseMemo.nfreq = d->nfreq, phaseMemo.first = first;
			phaseMemo.tE = W->E->t, phaseMemo.tH = W->H->t;
			for (int n = 0; n < d->nfreq; n++) phaseMemo.f[n] = d->P[n].f;
			memcpy(phaseMemo.phE, d->phE, 2 * d->nfreq * sizeof(float));
			memcpy(phaseMemo.phH, d->phH, 2 * d->nfreq * sizeof(float));
		}
	}
	CHECK("phaser_record", alisgpu_phaser_record(d->dp, d->phE, d->phH));
	d->hostStale = 1;
	d->fluxStale = 1;
}

/* face fluxes of every frequency of the set, reduced on the device from
 * the accumulators, with the spacing tables of the phaser box */
int alis_be_phaser_flux(phaser P, float face[6])
{
	devPhaser *d = findPhaser(P);
	if (!d) return 0;
	if (d->fluxStale) {
		phaser p = d->P;
		world W = p->W;
		int lo[3] = { p->iMin, p->jMin, p->kMin }, hi[3] = { p->iMax, p->jMax, p->kMax };
		const float *wE[3] = { &W->CE->dx[p->iMin], &W->CE->dy[p->jMin], &W->CE->dz[p->kMin] };
		const float *wH[3] = { &W->CH->dx[p->iMin], &W->CH->dy[p->jMin], &W->CH->dz[p->kMin] };
		float *out = malloc((size_t)d->nfreq * (d->nface ? d->nface : 1) * sizeof(float));
		CHECK("phaser_face_flux", alisgpu_phaser_face_flux(d->dp, wE, wH, lo, hi, out));
		memset(d->flux, 0, (size_t)6 * d->nfreq * sizeof(float));
		for (int n = 0; n < d->nfreq; n++)
			for (int f = 0; f < d->nface; f++) d->flux[n * 6 + d->faceSlot[f]] = out[n * d->nface + f];
		free(out);
		d->fluxStale = 0;
	}
	memcpy(face, d->flux + (P - d->P) * 6, 6 * sizeof(float));
	return 1;
}

static void downloadPhaser(devPhaser *d)
{
	CHECK("phaser_flush", alisgpu_phaser_flush(d->dp));
	for (int n = 0; n < d->nfreq; n++) {
		phaser p = d->P + n;
		cfield *cf[6] = { &p->xMin, &p->xMax, &p->yMin, &p->yMax, &p->zMin, &p->zMax };
		int lo[6][3] = {
			{ p->iMin, p->jMin, p->kMin }, { p->iMax, p->jMin, p->kMin }, { p->iMin, p->jMin, p->kMin },
			{ p->iMin, p->jMax, p->kMin }, { p->iMin, p->jMin, p->kMin }, { p->iMin, p->jMin, p->kMax } };
		for (int f = 0; f < d->nface; f++) {
			int s = d->faceSlot[f], axis = s / 2;
			cfield *c = cf[s];
			float complex ***q[4];
			if (axis == 0) q[0] = c->Ey, q[1] = c->Ez, q[2] = c->Hy, q[3] = c->Hz;
			else if (axis == 1) q[0] = c->Ez, q[1] = c->Ex, q[2] = c->Hz, q[3] = c->Hx;
			else q[0] = c->Ex, q[1] = c->Ey, q[2] = c->Hx, q[3] = c->Hy;
			for (int r = 0; r < 4; r++)
				CHECK("phaser_download", alisgpu_phaser_download(d->dp, n, f, r, (float *)&q[r][lo[s][0]][lo[s][1]][lo[s][2]]));
		}
	}
	d->hostStale = 0;
}

void alis_be_sync_phaser(phaser P)
{
	devPhaser *d = findPhaser(P);
	if (d && d->hostStale) downloadPhaser(d);
}

int alis_be_plane_flux(world W, int axis, int pos, int uLo, int uHi, int vLo, int vHi, float *out)
{
	devWorld *d = findWorld(W);
	if (!d) return 0;
	if (d->objectsDirty) uploadObjects(d);
	int lo[2] = { uLo, vLo }, hi[2] = { uHi, vHi };
	CHECK("plane_flux", alisgpu_plane_flux(d->dw, axis, pos, lo, hi, out));
	return 1;
}

int alis_be_object_absorption(world W, int n, float *out)
{
	devWorld *d = findWorld(W);
	if (!d) return 0;
	if (d->objectsDirty) uploadObjects(d);
	CHECK("object_absorption", alisgpu_object_absorption(d->dw, n, out));
	return 1;
}

void alis_be_nonlinear(world WS, world WP1, world WP2, float Alt)
{
	devWorld *s = findWorld(WS), *p1 = findWorld(WP1), *p2 = findWorld(WP2);
	if (!s || !p1 || !p2) { fprintf(stderr, "alis: nonlinear coupling of worlds unknown to the GPU backend\n"); exit(1); }
	if (s->objectsDirty) uploadObjects(s);
	/* the reference takes the tensor of C->M[n] for dispersive object n */
	for (int n = 0; n < WS->CE->N; n++)
		for (int m = 0; m <= WS->complexField; m++)
			CHECK("nonlinear_twm", alisgpu_nonlinear_twm(s->dw, p1->dw, p2->dw, n, m, (const float (*)[6])WS->CE->M[n].d, Alt));
	s->hostStale = 1;
}

void alis_be_sync_phasers_of(world W)
{
	for (devPhaser *d = phasers; d; d = d->next) if (d->P->W == W && d->hostStale) downloadPhaser(d);
}

void alis_be_sync_all(void)
{
	CHECK("synchronize", alisgpu_synchronize());
	for (devPhaser *d = phasers; d; d = d->next) if (d->hostStale) downloadPhaser(d);
	for (devWorld *d = worlds; d; d = d->next) if (d->hostStale) downloadWorld(d);
}


/* ---- far field (reference src/farfld.c:248-459) ----
 * FP64 face sums on the GPU over the phaser's device accumulators. */
int alis_gpu_farfield(phaser P, int nA, const tfield *T, const float *kx, const float *ky, double complex *out);
alisgpu_phaser *alis_gpu_phaser_handle(phaser P, int *index, int *faceSlot, int *nface);

void alis_be_farfield_sums(phaser P, int nA, const tfield *T, const float *kx, const float *ky, double complex *out)
{
	devPhaser *d = findPhaser(P);
	if (!d) { fprintf(stderr, "alis: far field of an unknown phaser\n"); exit(1); }
	CHECK("phaser_flush", alisgpu_phaser_flush(d->dp));
	if (alis_gpu_farfield(P, nA, T, kx, ky, out)) die("farfield_sums", ALISGPU_ECUDA);
}

/* device handle of a phaser set and the index of P in it */
alisgpu_phaser *alis_gpu_phaser_handle(phaser P, int *index, int *faceSlot, int *nface)
{
	devPhaser *d = findPhaser(P);
	if (!d) return 0;
	*index = (int)(P - d->P);
	*nface = d->nface;
	memcpy(faceSlot, d->faceSlot, sizeof d->faceSlot);
	return d->dp;
}

/* FP64 face sums of a batch of directions: host tables in double, the
 * test fields widened to double, per-face partials from the device
 * combined with the reference's face signs (-min, +max). */
int alis_gpu_farfield(phaser P, int nA, const tfield *T, const float *kx, const float *ky, double complex *out)
{
	int index, slots[6], nface;
	alisgpu_phaser *dp = alis_gpu_phaser_handle(P, &index, slots, &nface);
	if (!dp) return -1;
	world W = P->W;
	alisgpu_farfield_geom g;
	memset(&g, 0, sizeof g);
	g.iMin = P->iMin, g.iMax = P->iMax, g.jMin = P->jMin, g.jMax = P->jMax, g.kMin = P->kMin, g.kMax = P->kMax, g.kMIN = P->kMIN;
	g.sym[0] = W->xMinSur==SYM, g.sym[1] = W->yMinSur==SYM, g.sym[2] = W->zMinSur==SYM;
	g.cosk[0] = W->coskx, g.cosk[1] = W->cosky, g.cosk[2] = W->coskz;
	g.xLen = 1 + P->iMax - P->iMin, g.yLen = 1 + P->jMax - P->jMin, g.zLen = 2 + P->kMax - P->kMIN;
	double *tab = calloc(4*g.xLen + 4*g.yLen + 2*g.zLen, sizeof(double));
	double *xE = tab, *xH = xE + g.xLen, *dxE = xH + g.xLen, *dxH = dxE + g.xLen;
	double *yE = dxH + g.xLen, *yH = yE + g.yLen, *dyE = yH + g.yLen, *dyH = dyE + g.yLen;
	double *dzE = dyH + g.yLen, *dzH = dzE + g.zLen;
	for (int i = P->iMin; i <= P->iMax; i++) {
		int q = i - P->iMin;
		xE[q] = W->itox(W, i), xH[q] = W->itox(W, i-0.5), dxE[q] = W->CE->dx[i], dxH[q] = W->CH->dx[i];
	}
	for (int j = P->jMin; j <= P->jMax; j++) {
		int q = j - P->jMin;
		yE[q] = W->jtoy(W, j), yH[q] = W->jtoy(W, j-0.5), dyE[q] = W->CE->dy[j], dyH[q] = W->CH->dy[j];
	}
	for (int k = P->kMIN; k <= P->kMax+1; k++) {
		int q = k - P->kMIN;
		dzE[q] = W->CE->dz[k], dzH[q] = W->CH->dz[k];
	}
	g.xE = xE, g.xH = xH, g.dxE = dxE, g.dxH = dxH, g.yE = yE, g.yH = yH, g.dyE = dyE, g.dyH = dyH, g.dzE = dzE, g.dzH = dzH;
	int nk = g.zLen;
	double *Td = calloc((size_t)nA * 6 * nk * 2, sizeof(double));
	unsigned char *pr = calloc((size_t)nA * 6, 1);
	double *kxd = calloc(nA, sizeof(double)), *kyd = calloc(nA, sizeof(double));
	for (int a = 0; a < nA; a++) {
		float complex *c[6] = { T[a].Ex, T[a].Ey, T[a].Ez, T[a].Hx, T[a].Hy, T[a].Hz };
		for (int q = 0; q < 6; q++) {
			if (!c[q]) continue;
			pr[a*6+q] = 1;
			for (int k = P->kMIN; k <= P->kMax+1; k++) {
				size_t o = (((size_t)a*6 + q)*nk + (k - P->kMIN))*2;
				Td[o] = crealf(c[q][k]), Td[o+1] = cimagf(c[q][k]);
			}
		}
		kxd[a] = kx[a], kyd[a] = ky[a];
	}
	double *part = calloc((size_t)nA * 12, sizeof(double));
	int rc = alisgpu_farfield_sums(dp, index, &g, nA, Td, nk, pr, kxd, kyd, part);
	if (!rc) for (int a = 0; a < nA; a++) {
		double complex s = 0;
		for (int f = 0; f < nface; f++) {
			double complex v = part[(a*6+f)*2] + I * part[(a*6+f)*2+1];
			if (slots[f] % 2 == 0) s -= v; else s += v;
		}
		out[a] = s;
	}
	free(tab); free(Td); free(pr); free(kxd); free(kyd); free(part);
	return rc;
}


/* ---- voxelization (reference src/object.c:70-121, 229-279) ----
 * The object list becomes a node array for the device shape predicates:
 * list objects first, members of compound shapes after their owner.  The
 * shape is told by its function; a list holding a shape the device does
 * not evaluate (ImportContour, user functions) stays with the host loops.
 * The host supplies every sample coordinate through the world's own
 * itox/jtoy/ktoz and the glibc trigonometric values of rotations. */

#define VOX_MAX_DEPTH 12   /* nesting the device recursion allows */

typedef struct {
	alisgpu_vox_node *node;
	int n, cap;
	float *pool;
	int npool, pcap;
} voxList;

static int shapeTypeOf(shape *S)
{
	static shape *const known[ALISGPU_SHAPE_COUNT] = {
		[ALISGPU_SHAPE_BOX] = Box, [ALISGPU_SHAPE_BALL] = Ball, [ALISGPU_SHAPE_DIAMOND] = Diamond,
		[ALISGPU_SHAPE_BICONEX] = BiconeX, [ALISGPU_SHAPE_BICONEY] = BiconeY, [ALISGPU_SHAPE_BICONEZ] = BiconeZ,
		[ALISGPU_SHAPE_RODX] = RodX, [ALISGPU_SHAPE_RODY] = RodY, [ALISGPU_SHAPE_RODZ] = RodZ,
		[ALISGPU_SHAPE_DRODX] = DRodX, [ALISGPU_SHAPE_DRODY] = DRodY, [ALISGPU_SHAPE_DRODZ] = DRodZ,
		[ALISGPU_SHAPE_HRODXY] = HRodXY, [ALISGPU_SHAPE_HRODYZ] = HRodYZ, [ALISGPU_SHAPE_HRODZX] = HRodZX,
		[ALISGPU_SHAPE_HRODXZ] = HRodXZ, [ALISGPU_SHAPE_HRODYX] = HRodYX, [ALISGPU_SHAPE_HRODZY] = HRodZY,
		[ALISGPU_SHAPE_TRANSLATION] = Translation, [ALISGPU_SHAPE_ROTATION] = Rotation,
		[ALISGPU_SHAPE_COMBINATION] = Combination, [ALISGPU_SHAPE_INTERSECTION] = Intersection,
		[ALISGPU_SHAPE_DIFFERENCE] = Difference, [ALISGPU_SHAPE_LATTICE] = Lattice, [ALISGPU_SHAPE_DLATTICE] = DLattice,
		[ALISGPU_SHAPE_CLATTICEX] = CLatticeX, [ALISGPU_SHAPE_CLATTICEY] = CLatticeY, [ALISGPU_SHAPE_CLATTICEZ] = CLatticeZ,
	};
	for (int t = 0; t < ALISGPU_SHAPE_COUNT; t++) if (S && S == known[t]) return t;
	return -1;
}

/* count new zeroed nodes; index of the first */
static int voxNodes(voxList *L, int count)
{
	if (L->n + count > L->cap) {
		L->cap = 2 * (L->n + count) + 16;
		L->node = realloc(L->node, L->cap * sizeof *L->node);
	}
	memset(L->node + L->n, 0, count * sizeof *L->node);
	L->n += count;
	return L->n - count;
}

static int voxPool(voxList *L, int count)
{
	if (L->npool + count > L->pcap) {
		L->pcap = 2 * (L->npool + count) + 16;
		L->pool = realloc(L->pool, L->pcap * sizeof *L->pool);
	}
	L->npool += count;
	return L->npool - count;
}

/* node id from object O and its members; 0 if the device cannot evaluate it */
static int voxObject(voxList *L, int id, object O, int depth)
{
	int t = shapeTypeOf(O.S);
	if (t < 0 || depth > VOX_MAX_DEPTH) return 0;
	alisgpu_vox_node *x = &L->node[id];
	x->type = t;
	memcpy(x->f, O.f, sizeof x->f);
	int members = 0;
	switch (t) {
	case ALISGPU_SHAPE_ROTATION:
		/* the values Rotation computes (reference src/shapes.c:133-140) */
		x->rot[0] = cosf(O.f[0][0]*PI/180.), x->rot[1] = sinf(O.f[0][0]*PI/180.);
		x->rot[2] = cosf(O.f[0][1]*PI/180.), x->rot[3] = sinf(O.f[0][1]*PI/180.);
		x->rot[4] = cosf(O.f[0][2]*PI/180.), x->rot[5] = sinf(O.f[0][2]*PI/180.);
		members = 1;
		break;
	case ALISGPU_SHAPE_CLATTICEX: case ALISGPU_SHAPE_CLATTICEY: case ALISGPU_SHAPE_CLATTICEZ: {
		/* the angles CLatticeX/Y/Z step through (reference src/shapes.c:193-221) */
		int N = O.f[0][0];
		int at = voxPool(L, N > 0 ? 2 * N : 0);
		for (int n = 0; n < N; n++) {
			float t = 2 * PI * n / N;
			L->pool[at + n] = cosf(t), L->pool[at + N + n] = sinf(t);
		}
		L->node[id].trig = at;
		members = 1;
		break;
	}
	case ALISGPU_SHAPE_TRANSLATION: case ALISGPU_SHAPE_LATTICE: case ALISGPU_SHAPE_DLATTICE:
		members = 1;
		break;
	case ALISGPU_SHAPE_COMBINATION: case ALISGPU_SHAPE_INTERSECTION: case ALISGPU_SHAPE_DIFFERENCE:
		members = O.f[0][0];
		if (members < 0) members = 0;
		if (t == ALISGPU_SHAPE_DIFFERENCE && members < 1) return 0;
		break;
	}
	if (!members) return 1;
	if (!O.p) return 0;
	int c = voxNodes(L, members);
	L->node[id].child = c, L->node[id].nchild = members;
	object *m = O.p;
	for (int n = 0; n < members; n++) if (!voxObject(L, c + n, m[n], depth + 1)) return 0;
	return 1;
}

/* sample coordinates of one axis over indices lo..hi: kinds n - 1/2, n,
 * n + 1/2, each moved by the offsets fillFactor applies (reference
 * src/object.c:84-121) in the slot order the device expects */
static float *voxTable(world W, float (*itox)(world, float), int lo, int hi, int nslot)
{
	int subN = W->subN;
	float h = (subN-1.0) / (subN*2.0);
	float *tab = malloc((size_t)(1 + hi - lo) * 3 * nslot * sizeof *tab);
	for (int n = lo; n <= hi; n++) for (int kind = 0; kind < 3; kind++) {
		float b = kind == 0 ? n-0.5 : kind == 1 ? n : n+0.5;
		float *s = tab + ((size_t)(n - lo) * 3 + kind) * nslot;
		s[0] = itox(W, b);
		s[1] = itox(W, b-0.5);
		s[2] = itox(W, b+0.5);
		if (nslot > 3) {
			s[3] = itox(W, b+(-1)*h);
			s[4] = itox(W, b+1*h);
			for (int q = 0, di = 1-subN; di < subN; q++, di += 2) s[5+q] = itox(W, b+0.5*di/subN);
		}
	}
	return tab;
}

void *alis_be_vox_begin(world W, object *O, int N)
{
	/* the supersampling counts hits exactly up to 2^24 samples */
	if (N <= 0 || W->subN > 256) return NULL;
	voxList L = { 0 };
	voxNodes(&L, N);
	int ok = 1;
	for (int o = 0; o < N && ok; o++) ok = voxObject(&L, o, O[o], 0);
	alisgpu_voxelizer *v = NULL;
	if (ok) {
		int nslot = W->subN >= 2 ? 5 + W->subN : 3;
		int MIN[3] = { W->iMIN, W->jMIN, W->kMIN }, MAX[3] = { W->iMAX, W->jMAX, W->kMAX };
		int lo[3], hi[3];
		float (*itox[3])(world, float) = { W->itox, W->jtoy, W->ktoz };
		float *tab[3];
		for (int a = 0; a < 3; a++) lo[a] = MIN[a] - 1, hi[a] = MAX[a] + 2, tab[a] = voxTable(W, itox[a], lo[a], hi[a], nslot);
		CHECK("voxelizer_create", alisgpu_voxelizer_create(L.node, L.n, L.pool, L.npool, (const float *const *)tab, lo, hi,
		                                                   nslot, W->subN, MIN, MAX, &v));
		for (int a = 0; a < 3; a++) free(tab[a]);
	}
	free(L.node);
	free(L.pool);
	return v;
}

int alis_be_vox_bounds(void *v, int N, int *box)
{
	CHECK("voxelizer_bounds", alisgpu_voxelizer_bounds(v, N, box));
	return 1;
}

int alis_be_vox_fill(void *v, int o, const int *b, float *fx, float *fy, float *fz)
{
	CHECK("voxelizer_fill", alisgpu_voxelizer_fill(v, o, b[0], b[1], b[2], b[3], b[4], b[5], fx, fy, fz));
	return 1;
}

int alis_be_vox_fill_edge(void *v, int o, int axis, int n, int u0, int u1, int v0, int v1, float *out)
{
	CHECK("voxelizer_fill_edge", alisgpu_voxelizer_fill_edge(v, o, axis, n, u0, u1, v0, v1, out));
	return 1;
}

void alis_be_vox_end(void *v)
{
	if (v) alisgpu_voxelizer_destroy(v);
}


/* ---- sliceFreqDom's running DFT (reference src/slices.c:326-356) ----
 * Field functions that sample E or H (src/fields.c:130-291) run on the
 * device; the others (currents, incident and scattered fields) stay with
 * the host loop over the synced box. */

static int sampleOf(field *F, int *fld, int *m, int *comp, int *avg, int sgn[3])
{
	static const struct { field *F; int fld, m, comp, avg, s[3]; } tab[] = {
		{ rawEx, 0, 0, 0, 0, { 1, -1, -1 } }, { rawEy, 0, 0, 1, 0, { -1, 1, -1 } }, { rawEz, 0, 0, 2, 0, { -1, -1, 1 } },
		{ rawHx, 1, 0, 0, 0, { -1, 1, 1 } }, { rawHy, 1, 0, 1, 0, { 1, -1, 1 } }, { rawHz, 1, 0, 2, 0, { 1, 1, -1 } },
		{ Ex, 0, 0, 0, 1, { 1, -1, -1 } }, { Ey, 0, 0, 1, 1, { -1, 1, -1 } }, { Ez, 0, 0, 2, 1, { -1, -1, 1 } },
		{ iEx, 0, 1, 0, 1, { 1, -1, -1 } }, { iEy, 0, 1, 1, 1, { -1, 1, -1 } }, { iEz, 0, 1, 2, 1, { -1, -1, 1 } },
		{ Hx, 1, 0, 0, 1, { -1, 1, 1 } }, { Hy, 1, 0, 1, 1, { 1, -1, 1 } }, { Hz, 1, 0, 2, 1, { 1, 1, -1 } },
		{ iHx, 1, 1, 0, 1, { -1, 1, 1 } }, { iHy, 1, 1, 1, 1, { 1, -1, 1 } }, { iHz, 1, 1, 2, 1, { 1, 1, -1 } },
	};
	for (int n = 0; n < (int)(sizeof tab / sizeof *tab); n++) if (tab[n].F == F) {
		*fld = tab[n].fld, *m = tab[n].m, *comp = tab[n].comp, *avg = tab[n].avg;
		for (int a = 0; a < 3; a++) sgn[a] = tab[n].s[a];
		return 1;
	}
	return 0;
}

void *alis_be_slice_dft_begin(world W, const int box[6])
{
	devWorld *d = findWorld(W);
	if (!d) return NULL;
	alisgpu_slice_dft *h = NULL;
	CHECK("slice_dft_create", alisgpu_slice_dft_create(d->dw, box, &h));
	devSliceDft *s = calloc(1, sizeof *s);
	s->d = d, s->h = h, s->next = sliceDfts, sliceDfts = s;
	return s;
}

int alis_be_slice_dft_add(void *v, world W, field *F, float re, float im)
{
	devSliceDft *s = v;
	int fld, m, comp, avg, sgn[3];
	if (!s || !s->h || s->d->W != W || !sampleOf(F, &fld, &m, &comp, &avg, sgn)) return 0;
	/* the mirror parities the field functions apply: sign times the Bloch cosine */
	int sym[3] = { W->xMinSur == SYM, W->yMinSur == SYM, W->zMinSur == SYM };
	float par[3] = { sgn[0] * W->coskx, sgn[1] * W->cosky, sgn[2] * W->coskz };
	CHECK("slice_dft_add", alisgpu_slice_dft_add(s->h, fld, m, comp, avg, sym, par, re, im));
	return 1;
}

int alis_be_slice_dft_read(void *v, float *F, float *G)
{
	devSliceDft *s = v;
	if (!s || !s->h) return 0;
	CHECK("slice_dft_download", alisgpu_slice_dft_download(s->h, F, G));
	return 1;
}

void alis_be_slice_dft_end(void *v)
{
	devSliceDft *s = v;
	if (!s) return;
	devSliceDft **pp = &sliceDfts;
	while (*pp && *pp != s) pp = &(*pp)->next;
	if (*pp) *pp = s->next;
	if (s->h) alisgpu_slice_dft_destroy(s->h);
	free(s);
}
