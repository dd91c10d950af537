// world.cu -- device worlds and the fused Yee half-step kernel.
//
// One launch per field set m updates every cell of a world in the order
// of the reference's updateF / updateJ (src/update.c:87-158):
//   conductivity factors of every dispersive object
//   -> subtraction of every ADE current
//   -> curl with dt/ds tables and eps^-1
//   -> CPML psi recursions (faces xMin, yMin, zMin, xMax, yMax, zMax)
//   -> TFSF incident-field corrections (src/update.c:194-272)
//   -> (H half step) ADE current update driven by E.
// The file is compiled with -fmad=false so that every add and multiply
// rounds exactly as the reference's scalar code does; the arithmetic is
// HBM-bound, so the lost FMAs cost nothing measurable.
// Sources and ghost-cell copies follow as small launches, in the
// reference order.
#include <cstdio>
#include <cstdarg>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <algorithm>
#include <atomic>
#include <unordered_map>
#include <mutex>
#include <cooperative_groups.h>
#include "common.cuh"
#include "batch.cuh"
namespace cg = cooperative_groups;

// ---------------------------------------------------------------------
// process-wide state: device, stream groups, error text, launch counter
// ---------------------------------------------------------------------
// Several host threads may step different worlds at once: what a call
// uses besides its world is per thread (the current stream group, the
// launch-parameter staging, the error text) or atomic (the counters).
static int gInit;
static thread_local char gErr[512];
static std::atomic<unsigned long long> gLaunches;
static unsigned int *gErrWord;

extern "C" int alisgpu__fail(int code, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(gErr, sizeof gErr, fmt, ap);
	va_end(ap);
	return code;
}

extern "C" int alisgpu__check(cudaError_t e, const char *what)
{
	int code = e == cudaErrorMemoryAllocation ? ALISGPU_ENOMEM : ALISGPU_ECUDA;
	return alisgpu__fail(code, "%s: %s", what, cudaGetErrorString(e));
}

// The streams of a group of worlds -- a world and its TFSF auxiliary
// worlds.  Every world belongs to the default group unless it asks for a
// group of its own; the steps of worlds in different groups overlap on
// the device.  In a group:
// * the main stream orders the worlds' half steps, phasers and results;
// * the side stream runs the half steps of the auxiliary worlds
//   concurrently with their parent's.  An auxiliary step of field F waits
//   for the parent's last step of the other field (which read the
//   auxiliary F it is about to overwrite); a parent step of field F waits
//   for the last auxiliary step of the other field (whose result it
//   reads).  Any other call that touches world data joins the two streams
//   first, and the next auxiliary step then waits for everything issued
//   before it;
// * the gather stream runs phaser gathers beside the H ghost copies.
struct StreamGroup {
	cudaStream_t main, side, gather;
	cudaEvent_t evMainDone[2], evAuxDone[2], evJoin, evGatherDone;
	int mainRec[2], auxRec[2], sideUsed, sideWaitsAll;
	int users;                                // worlds in an own group
};
static StreamGroup gDefaultGroup;
static std::vector<StreamGroup *> gOwnGroups;
static std::mutex gGroupsLock;
// the group of the world the current call works on (set by bindWorld)
static thread_local StreamGroup *gGroup = &gDefaultGroup;
#define gStream (gGroup->main)
#define gSide (gGroup->side)
#define gGather (gGroup->gather)
#define gEvMainDone (gGroup->evMainDone)
#define gEvAuxDone (gGroup->evAuxDone)
#define gEvJoin (gGroup->evJoin)
#define gEvGatherDone (gGroup->evGatherDone)
#define gMainRec (gGroup->mainRec)
#define gAuxRec (gGroup->auxRec)
#define gSideUsed (gGroup->sideUsed)
#define gSideWaitsAll (gGroup->sideWaitsAll)
// operations that change world data, enqueued so far (launches and uploads)
static std::atomic<unsigned long long> gOps;

static int groupCreate(StreamGroup *g)
{
	ALIS_CUDA(cudaStreamCreateWithFlags(&g->main, cudaStreamNonBlocking));
	// the side stream's small blocks take the first free slots
	int prLeast = 0, prGreatest = 0;
	ALIS_CUDA(cudaDeviceGetStreamPriorityRange(&prLeast, &prGreatest));
	ALIS_CUDA(cudaStreamCreateWithPriority(&g->side, cudaStreamNonBlocking, prGreatest));
	ALIS_CUDA(cudaStreamCreateWithFlags(&g->gather, cudaStreamNonBlocking));
	for (int f = 0; f < 2; f++) {
		ALIS_CUDA(cudaEventCreateWithFlags(&g->evMainDone[f], cudaEventDisableTiming));
		ALIS_CUDA(cudaEventCreateWithFlags(&g->evAuxDone[f], cudaEventDisableTiming));
	}
	ALIS_CUDA(cudaEventCreateWithFlags(&g->evJoin, cudaEventDisableTiming));
	ALIS_CUDA(cudaEventCreateWithFlags(&g->evGatherDone, cudaEventDisableTiming));
	g->sideWaitsAll = 1;
	return ALISGPU_OK;
}

static void groupDestroy(StreamGroup *g)
{
	cudaStreamSynchronize(g->side), cudaStreamSynchronize(g->gather), cudaStreamSynchronize(g->main);
	cudaStreamDestroy(g->main), cudaStreamDestroy(g->side), cudaStreamDestroy(g->gather);
	for (int f = 0; f < 2; f++) cudaEventDestroy(g->evMainDone[f]), cudaEventDestroy(g->evAuxDone[f]);
	cudaEventDestroy(g->evJoin), cudaEventDestroy(g->evGatherDone);
}

static void fullJoin(void)
{
	if (gSideUsed) {
		cudaEventRecord(gEvJoin, gSide);
		cudaStreamWaitEvent(gStream, gEvJoin, 0);
	}
	gSideWaitsAll = 1;
}

extern "C" const char *alisgpu_last_error(void) { return gErr; }
extern "C" void alisgpu__count_launch(void) { gLaunches++, gOps++; }
extern "C" unsigned long long alisgpu_launch_count(void) { return gLaunches; }
static std::atomic<int> gDenyAllocs;
extern "C" int alisgpu_inject_alloc_failures(int n) { return gDenyAllocs.exchange(n > 0 ? n : 0); }
extern "C" int alisgpu__alloc_denied(void)
{
	int n = gDenyAllocs.load();
	while (n > 0 && !gDenyAllocs.compare_exchange_weak(n, n - 1)) {}
	return n > 0;
}
extern "C" cudaStream_t alisgpu__stream(void) { return gStream; }
extern "C" void *alisgpu_stream(void) { return (void *)gDefaultGroup.main; }

extern "C" int alisgpu_init(void)
{
	if (gInit) return ALISGPU_OK;
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
		return alisgpu__fail(ALISGPU_ENODEV, "no CUDA device available");
	const char *env = getenv("ALISGPU_DEVICE");
	int dev = env ? atoi(env) : 0;
	ALIS_CUDA(cudaSetDevice(dev));
	int rc = groupCreate(&gDefaultGroup);
	if (rc) return rc;
	// freed device memory stays in the pool for the next world
	cudaMemPool_t pool;
	ALIS_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
	unsigned long long keep = ~0ull;
	ALIS_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
	ALIS_CUDA(cudaMalloc(&gErrWord, sizeof(unsigned int)));
	ALIS_CUDA(cudaMemset(gErrWord, 0, sizeof(unsigned int)));
	gInit = 1;
	return ALISGPU_OK;
}

// ---- optional per-kernel event timing ----
struct ProfSlot { cudaEvent_t a, b; int kind; };
static std::vector<ProfSlot> gProf;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> gProfFree;
static int gProfOn;
static double gProfMs[ALISGPU_K_KINDS];
static unsigned long long gProfN[ALISGPU_K_KINDS];

extern "C" int alisgpu_profile(int enable)
{
	// auxiliary steps change streams with the mode: order them across it
	if (gInit) fullJoin();
	gProfOn = enable;
	return ALISGPU_OK;
}

extern "C" int alisgpu__prof_start(void)
{
	if (!gProfOn) return -1;
	ProfSlot s;
	if (!gProfFree.empty()) { s.a = gProfFree.back().first; s.b = gProfFree.back().second; gProfFree.pop_back(); }
	else { cudaEventCreate(&s.a); cudaEventCreate(&s.b); }
	s.kind = -1;
	cudaEventRecord(s.a, gStream);
	gProf.push_back(s);
	return (int)gProf.size() - 1;
}

extern "C" void alisgpu__prof_stop(int slot, int kind)
{
	if (slot < 0) return;
	gProf[slot].kind = kind;
	cudaEventRecord(gProf[slot].b, gStream);
}

static void profDrain(void)
{
	if (gProf.empty()) return;
	cudaStreamSynchronize(gStream);
	for (ProfSlot &s : gProf) {
		float ms = 0;
		if (s.kind >= 0 && cudaEventElapsedTime(&ms, s.a, s.b) == cudaSuccess) gProfMs[s.kind] += ms, gProfN[s.kind]++;
		gProfFree.push_back(std::make_pair(s.a, s.b));
	}
	gProf.clear();
}

extern "C" int alisgpu_profile_read(int kind, double *ms, unsigned long long *launches)
{
	if (kind < 0 || kind >= ALISGPU_K_KINDS) return alisgpu__fail(ALISGPU_EINVAL, "profile_read: bad kind");
	profDrain();
	if (ms) *ms = gProfMs[kind];
	if (launches) *launches = gProfN[kind];
	gProfMs[kind] = 0, gProfN[kind] = 0;
	return ALISGPU_OK;
}

extern "C" int alisgpu_synchronize(void)
{
	ALIS_BATCH_GUARD();
	if (!gInit) return ALISGPU_OK;
	std::lock_guard<std::mutex> lock(gGroupsLock);
	for (size_t q = 0; q <= gOwnGroups.size(); q++) {
		gGroup = q < gOwnGroups.size() ? gOwnGroups[q] : &gDefaultGroup;
		fullJoin();
		ALIS_CUDA(cudaStreamSynchronize(gStream));
	}
	unsigned int e = 0;
	ALIS_CUDA(cudaMemcpy(&e, gErrWord, sizeof e, cudaMemcpyDeviceToHost));
	if (e) return alisgpu__fail(ALISGPU_ERANGE, "device error word %#x", e);
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// world storage
// ---------------------------------------------------------------------
struct alisgpu_world {
	StreamGroup *group;                    // own stream group, or null: the default group
	alisgpu_geometry g;
	float *vbuf;                           // source values of large patches
	int vcap;
	float *vpin[2];                        // their pinned host staging, two in turn
	cudaEvent_t vpinFree[2];
	int vpinCap, vpinNext;
	Layout L;
	float *E[2][3], *H[2][3];
	float *C[3];
	float *dtd[2][3];
	float *cp[2][9];
	BoxArr psi[2][2][6][2];           // [grid E/H][m][face][which]
	std::vector<DevObj> objs;
	DevObj *dObjs;
	std::vector<void *> objMem;
	size_t bytes;
	unsigned short *cls[2][3];             // per-axis cell classes of the E / H step
	std::vector<unsigned short> clsHost[2][3];
	// ghost copies of the last E half step, not yet applied: they only
	// write E's upper halo, which no half step reads, so they run once
	// before the host reads E (same bytes: each copy is a function of the
	// current interior E)
	std::vector<alisgpu_ghost_copy> pendingE;
	// per field: the last ghost list seen and whether its chains qualify
	// for the one-launch form (k_ghost_chain)
	std::vector<alisgpu_ghost_copy> ghostSeen[2];
	bool ghostChain[2];
	// the block shape of each field's half step: timed over the first
	// ALIS_TUNE_STEPS launches, then fixed
	struct TyTuner {
		int choice = -1, seen = 0;
		cudaEvent_t a[9], b[9];
		int variant[9];
	} tune[2];
	// an auxiliary world's half step waiting to run inside its parent's
	// launch of the same field
	struct SmallStepParams *staged[2];
	bool stagedValid[2];
	// the last H half step: its ghost copies, an event after its cell
	// updates, and the operation count after its ghost launch (a phaser
	// gather that follows directly may run beside the ghost copies)
	std::vector<alisgpu_ghost_copy> hGhosts;
	cudaEvent_t evHCells;
	unsigned long long hOps;
	bool hRecorded;
	float *planeTab;                       // scratch of the observer kernels
	size_t planeTabFloats;
	float *sp[2][3];                       // cell spacings (CE, CH) per axis, indexed from MIN
	void *matIdx;                          // eps^-1 triple index per cell (few distinct triples)
	float4 *matTab;
	int matWide;                           // the index has 16 bits (else 8)
	// batched stepping: device copies of the half-step parameters per field
	// and m, of a one-block step, of the source patches and of the ghost
	// copies; the values of an auxiliary step staged for the parent's
	// batched launch; the batch group the world last joined
	ParamSlot bS[2], bSrc[2], bG[2];
	long long ghostCells[2];                // cells of the ghost copies in bG
	std::vector<float> stagedVals[2];
	unsigned long long batchStamp;
	// the device form of its TFSF boxes (tfsfFor)
	struct TfsfCache { const alisgpu_tfsf *key; int field; DevTfsf T; };
	std::vector<TfsfCache> tfCache;
	unsigned long long tfEpoch;
	// what the cell-class tables of each field were made from: the CPML
	// slabs, the TFSF boxes and the object boxes
	std::vector<int> clsKey[2];
	// per-tile object lists of a world with more than 8 objects, and the
	// object boxes they were made from
	int *tileStart, *tileObj;
	std::vector<int> tileKey;
	// FP16 storage (alisgpu_world_set_storage), per field: by the parity
	// of the step, the exponents as read and as computed and the scales as
	// read; the next step's inverse scales; the plane maxima of two steps
	// in turn; the half steps taken.  written: a step or upload wrote the
	// fields
	int half;
	signed char *ex[2][2], *exK[2][2];
	float *sc[2][2], *inv[2], *tab[2];
	unsigned *mx[2][2];
	long long nHalf[2];
	bool tabFresh[2];                      // tab[f] holds the scales of f's next step
	bool written;
};

// the exponents of a half world's field as its readers use them now, and
// their scales
static inline const signed char *halfRead(const alisgpu_world *w, int field)
{
	return w->ex[field][(w->nHalf[field] + 1) & 1];
}
static inline const float *halfScales(const alisgpu_world *w, int field)
{
	return w->sc[field][(w->nHalf[field] + 1) & 1];
}

static inline void bindWorld(const alisgpu_world *w)
{
	gGroup = w && w->group ? w->group : &gDefaultGroup;
}

extern "C" void alisgpu__bind(alisgpu_world *w) { bindWorld(w); }

// A blocking copy ordered on the current group's main stream: device
// memory from the stream-ordered pool is valid in that stream's order.
static cudaError_t orderedCopy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind)
{
	cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, gStream);
	return e == cudaSuccess ? cudaStreamSynchronize(gStream) : e;
}

static int applyPendingGhosts(alisgpu_world *w);
static void freeStaged(alisgpu_world *w);

static Layout makeLayout(const alisgpu_geometry *g)
{
	Layout L;
	L.i0 = g->iMIN - 1, L.j0 = g->jMIN - 1, L.k0 = g->kMIN - 1;
	L.ni = g->iMAX - g->iMIN + 3, L.nj = g->jMAX - g->jMIN + 3, L.nk = g->kMAX - g->kMIN + 3;
	// row pitch: padding keeps the last float4 of a row and its k+1
	// neighbour inside the row
	L.sj = ((ALIS_KOFF + L.nk + 4 + 31) / 32) * 32;
	L.si = L.sj * L.nj;
	return L;
}

static int devAlloc(alisgpu_world *w, float **p, size_t n)
{
	ALIS_CUDA(alisgpu__mallocAsync(p, n * sizeof(float)));
	ALIS_CUDA(cudaMemsetAsync(*p, 0, n * sizeof(float), gStream));
	w->bytes += n * sizeof(float);
	return ALISGPU_OK;
}

// psi slab boxes of face f for the E (Offset 0) or H (Offset 1) lattice,
// same ranges as the host layer (reference src/world.c:174-186)
static BoxArr slabBox(const alisgpu_geometry *g, int face, int Offset)
{
	int r[6] = { g->iMIN, g->iMAX, g->jMIN, g->jMAX, g->kMIN, g->kMAX };
	int mins[3] = { g->iMin, g->jMin, g->kMin }, maxs[3] = { g->iMax, g->jMax, g->kMax };
	int MINs[3] = { g->iMIN, g->jMIN, g->kMIN }, MAXs[3] = { g->iMAX, g->jMAX, g->kMAX };
	int d = face % 3;
	if (face < 3) r[2*d] = MINs[d] + Offset, r[2*d+1] = mins[d] + Offset - 2;
	else r[2*d] = maxs[d] + 2, r[2*d+1] = MAXs[d];
	BoxArr b;
	b.p = 0;
	b.i0 = r[0], b.i1 = r[1], b.j0 = r[2], b.j1 = r[3], b.k0 = r[4], b.k1 = r[5];
	b.sj = 1 + b.k1 - b.k0;
	b.si = b.sj * (1 + b.j1 - b.j0);
	return b;
}

extern "C" int alisgpu_world_create(const alisgpu_geometry *g, alisgpu_world **out)
{
	int rc = alisgpu_init();
	if (rc) return rc;
	if (!g || !out) return alisgpu__fail(ALISGPU_EINVAL, "world_create: null argument");
	if (g->iMAX < g->iMIN || g->jMAX < g->jMIN || g->kMAX < g->kMIN)
		return alisgpu__fail(ALISGPU_EINVAL, "world_create: empty grid");
	alisgpu_world *w = new alisgpu_world();
	bindWorld(w);
	w->g = *g;
	w->L = makeLayout(g);
	size_t n = w->L.elems();
	for (int m = 0; m <= g->complexField; m++) for (int c = 0; c < 3; c++) {
		if ((rc = devAlloc(w, &w->E[m][c], n)) || (rc = devAlloc(w, &w->H[m][c], n))) { alisgpu_world_destroy(w); return rc; }
	}
	for (int grid = 0; grid < 2; grid++) for (int m = 0; m <= g->complexField; m++) for (int f = 0; f < 6; f++) {
		if (!g->pml[f]) continue;
		for (int q = 0; q < 2; q++) {
			BoxArr b = slabBox(g, f, grid);
			if (b.i1 < b.i0 || b.j1 < b.j0 || b.k1 < b.k0) continue;
			if ((rc = devAlloc(w, &b.p, b.elems()))) { alisgpu_world_destroy(w); return rc; }
			w->psi[grid][m][f][q] = b;
		}
	}
	*out = w;
	return ALISGPU_OK;
}

static void freeObjects(alisgpu_world *w)
{
	for (void *p : w->objMem) alisgpu__freeAsync(p);
	w->objMem.clear();
	w->objs.clear();
	if (w->dObjs) alisgpu__freeAsync(w->dObjs), w->dObjs = 0;
}

extern "C" int alisgpu_world_destroy(alisgpu_world *w)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w) return ALISGPU_OK;
	cudaStreamSynchronize(gStream);
	for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
		if (w->E[m][c]) alisgpu__freeAsync(w->E[m][c]);
		if (w->H[m][c]) alisgpu__freeAsync(w->H[m][c]);
	}
	for (int c = 0; c < 3; c++) if (w->C[c]) alisgpu__freeAsync(w->C[c]);
	for (int f = 0; f < 2; f++) {
		for (int p = 0; p < 2; p++) {
			alisgpu__freeAsync(w->ex[f][p]), alisgpu__freeAsync(w->exK[f][p]);
			alisgpu__freeAsync(w->sc[f][p]), alisgpu__freeAsync(w->mx[f][p]);
		}
		alisgpu__freeAsync(w->inv[f]), alisgpu__freeAsync(w->tab[f]);
	}
	if (w->planeTab) alisgpu__freeAsync(w->planeTab);
	alisgpu__freeAsync(w->tileStart), alisgpu__freeAsync(w->tileObj);
	if (w->matIdx) alisgpu__freeAsync(w->matIdx);
	if (w->matTab) alisgpu__freeAsync(w->matTab);
	for (int grid = 0; grid < 2; grid++) for (int a = 0; a < 3; a++) if (w->sp[grid][a]) alisgpu__freeAsync(w->sp[grid][a]);
	for (int grid = 0; grid < 2; grid++) {
		for (int c = 0; c < 3; c++) if (w->dtd[grid][c]) alisgpu__freeAsync(w->dtd[grid][c]);
		for (int c = 0; c < 9; c++) if (w->cp[grid][c]) alisgpu__freeAsync(w->cp[grid][c]);
		for (int m = 0; m < 2; m++) for (int f = 0; f < 6; f++) for (int q = 0; q < 2; q++)
			if (w->psi[grid][m][f][q].p) alisgpu__freeAsync(w->psi[grid][m][f][q].p);
	}
	freeObjects(w);
	for (int f = 0; f < 2; f++) alisgpu__slot_free(&w->bS[f]), alisgpu__slot_free(&w->bSrc[f]), alisgpu__slot_free(&w->bG[f]);
	for (int f = 0; f < 2; f++) for (int a = 0; a < 3; a++) if (w->cls[f][a]) alisgpu__freeAsync(w->cls[f][a]);
	if (w->evHCells) cudaEventDestroy(w->evHCells);
	if (w->vbuf) alisgpu__freeAsync(w->vbuf);
	freeStaged(w);
	for (int f = 0; f < 2; f++)
		if (w->tune[f].choice < 0)
			for (int q = 0; q < w->tune[f].seen; q++) cudaEventDestroy(w->tune[f].a[q]), cudaEventDestroy(w->tune[f].b[q]);
	for (int b = 0; b < 2; b++)
		if (w->vpin[b]) cudaEventSynchronize(w->vpinFree[b]), cudaFreeHost(w->vpin[b]), cudaEventDestroy(w->vpinFree[b]);
	StreamGroup *grp = w->group;
	delete w;
	if (grp && --grp->users == 0) {
		groupDestroy(grp);
		std::lock_guard<std::mutex> lock(gGroupsLock);
		gOwnGroups.erase(std::find(gOwnGroups.begin(), gOwnGroups.end(), grp));
		delete grp;
	}
	gGroup = &gDefaultGroup;
	return ALISGPU_OK;
}

extern "C" size_t alisgpu_world_bytes(const alisgpu_world *w) { return w ? w->bytes : 0; }

// Move world w to a stream group of its own (after the work it has
// queued), so that its steps overlap on the device with those of worlds in
// other groups.
extern "C" int alisgpu_world_own_streams(alisgpu_world *w)
{
	if (!w) return alisgpu__fail(ALISGPU_EINVAL, "world_own_streams: null world");
	if (w->group && w->group->users == 1) return ALISGPU_OK;
	bindWorld(w);
	fullJoin();
	cudaEvent_t done = gEvJoin;
	ALIS_CUDA(cudaEventRecord(done, gStream));
	StreamGroup *grp = new StreamGroup();
	int rc = groupCreate(grp);
	if (rc) { delete grp; return rc; }
	ALIS_CUDA(cudaStreamWaitEvent(grp->main, done, 0));
	if (w->group) w->group->users--;
	grp->users = 1;
	{
		std::lock_guard<std::mutex> lock(gGroupsLock);
		gOwnGroups.push_back(grp);
	}
	w->group = grp;
	bindWorld(w);
	return ALISGPU_OK;
}

// Put world w into the stream group of world parent (a TFSF auxiliary
// world and the world whose box it feeds).
extern "C" int alisgpu_world_share_streams(alisgpu_world *w, alisgpu_world *parent)
{
	if (!w || !parent) return alisgpu__fail(ALISGPU_EINVAL, "world_share_streams: null world");
	if (w->group == parent->group) return ALISGPU_OK;
	bindWorld(w);
	fullJoin();
	cudaEvent_t done = gEvJoin;
	ALIS_CUDA(cudaEventRecord(done, gStream));
	bindWorld(parent);
	ALIS_CUDA(cudaStreamWaitEvent(gStream, done, 0));
	if (w->group && --w->group->users == 0) {
		StreamGroup *old = w->group;
		groupDestroy(old);
		std::lock_guard<std::mutex> lock(gGroupsLock);
		gOwnGroups.erase(std::find(gOwnGroups.begin(), gOwnGroups.end(), old));
		delete old;
	}
	w->group = parent->group;
	if (w->group) w->group->users++;
	return ALISGPU_OK;
}

extern "C" void *alisgpu_world_stream(const alisgpu_world *w)
{
	return (void *)(w && w->group ? w->group->main : gDefaultGroup.main);
}

__global__ void k_fill(float *p, float v, int n)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t < n) p[t] = v;
}

static int halfTable(alisgpu_world *w, int field);

// exponents and scales back to their start value (the first step finds
// no maxima), maxima and step counts to zero
static int halfStateReset(alisgpu_world *w)
{
	const int n = 3 * w->L.ni;
	for (int f = 0; f < 2; f++) {
		for (int p = 0; p < 2; p++) {
			ALIS_CUDA(cudaMemsetAsync(w->ex[f][p], (unsigned char)(signed char)HALF_E0, n, gStream));
			ALIS_CUDA(cudaMemsetAsync(w->exK[f][p], (unsigned char)(signed char)HALF_E0, n, gStream));
			k_fill<<<(n + 255) / 256, 256, 0, gStream>>>(w->sc[f][p], ldexpf(1.0f, HALF_E0), n);
			ALIS_CUDA(cudaMemsetAsync(w->mx[f][p], 0, (size_t)n * HALF_SLOTS * sizeof(unsigned), gStream));
		}
		k_fill<<<(n + 255) / 256, 256, 0, gStream>>>(w->inv[f], ldexpf(1.0f, -HALF_E0), n);
		alisgpu__count_launch(), alisgpu__count_launch(), alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
		w->nHalf[f] = 0;
	}
	for (int f = 0; f < 2; f++) {
		int rc = halfTable(w, f);
		if (rc) return rc;
	}
	return ALISGPU_OK;
}

// device bytes of a half world's exponent, scale and maxima arrays
static size_t halfPlaneBytes(const alisgpu_world *w)
{
	const size_t n = 3 * (size_t)w->L.ni;
	return 2 * (2 * (2 * n + n * sizeof(float) + n * HALF_SLOTS * sizeof(unsigned)) + n * sizeof(float) +
	            (size_t)w->L.ni * HALF_TAB * sizeof(float));
}

extern "C" int alisgpu_world_set_storage(alisgpu_world *w, int storage)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	if (!w || (storage != ALISGPU_STORAGE_FLOAT && storage != ALISGPU_STORAGE_HALF))
		return alisgpu__fail(ALISGPU_EINVAL, "world_set_storage: bad argument");
	if (storage == w->half) return ALISGPU_OK;
	if (w->written || w->nHalf[0] || w->nHalf[1])
		return alisgpu__fail(ALISGPU_EINVAL, "world_set_storage: the world has been stepped or written");
	if (storage == ALISGPU_STORAGE_HALF && w->g.complexField)
		return alisgpu__fail(ALISGPU_ENOTSUP, "world_set_storage: half storage needs real fields");
	fullJoin();
	const size_t n = w->L.elems(), esz = storage == ALISGPU_STORAGE_HALF ? 2 : sizeof(float), np = 3 * (size_t)w->L.ni;
	// the new arrays first: on failure the world keeps its form
	float *E[3] = {}, *H[3] = {}, *sc[2][2] = {}, *inv[2] = {}, *tab[2] = {};
	signed char *ex[2][2] = {}, *exK[2][2] = {};
	unsigned *mx[2][2] = {};
	auto release = [](float *const (&e)[3], float *const (&h)[3], signed char *const (&x)[2][2], signed char *const (&k)[2][2],
	                  float *const (&c)[2][2], float *const (&iv)[2], float *const (&tb)[2], unsigned *const (&m)[2][2]) {
		for (int q = 0; q < 3; q++) alisgpu__freeAsync(e[q]), alisgpu__freeAsync(h[q]);
		for (int f = 0; f < 2; f++) {
			for (int p = 0; p < 2; p++)
				alisgpu__freeAsync(x[f][p]), alisgpu__freeAsync(k[f][p]), alisgpu__freeAsync(c[f][p]), alisgpu__freeAsync(m[f][p]);
			alisgpu__freeAsync(iv[f]), alisgpu__freeAsync(tb[f]);
		}
	};
	cudaError_t e = cudaSuccess;
	for (int c = 0; c < 3 && e == cudaSuccess; c++) {
		if ((e = alisgpu__mallocAsync(&E[c], n * esz)) == cudaSuccess) e = alisgpu__mallocAsync(&H[c], n * esz);
		if (e == cudaSuccess) e = cudaMemsetAsync(E[c], 0, n * esz, gStream);
		if (e == cudaSuccess) e = cudaMemsetAsync(H[c], 0, n * esz, gStream);
	}
	if (storage == ALISGPU_STORAGE_HALF)
		for (int f = 0; f < 2 && e == cudaSuccess; f++) {
			for (int p = 0; p < 2 && e == cudaSuccess; p++) {
				if ((e = alisgpu__mallocAsync(&ex[f][p], np)) == cudaSuccess) e = alisgpu__mallocAsync(&exK[f][p], np);
				if (e == cudaSuccess) e = alisgpu__mallocAsync(&sc[f][p], np * sizeof(float));
				if (e == cudaSuccess) e = alisgpu__mallocAsync(&mx[f][p], np * HALF_SLOTS * sizeof(unsigned));
			}
			if (e == cudaSuccess) e = alisgpu__mallocAsync(&inv[f], np * sizeof(float));
			if (e == cudaSuccess) e = alisgpu__mallocAsync(&tab[f], (size_t)w->L.ni * HALF_TAB * sizeof(float));
		}
	if (e != cudaSuccess) {
		release(E, H, ex, exK, sc, inv, tab, mx);
		return alisgpu__check(e, "world_set_storage");
	}
	// the old arrays go, the new ones take their place
	float *oE[3], *oH[3];
	for (int c = 0; c < 3; c++) oE[c] = w->E[0][c], oH[c] = w->H[0][c], w->E[0][c] = E[c], w->H[0][c] = H[c];
	release(oE, oH, w->ex, w->exK, w->sc, w->inv, w->tab, w->mx);
	memcpy(w->ex, ex, sizeof ex), memcpy(w->exK, exK, sizeof exK), memcpy(w->sc, sc, sizeof sc);
	memcpy(w->inv, inv, sizeof inv), memcpy(w->tab, tab, sizeof tab), memcpy(w->mx, mx, sizeof mx);
	const size_t before = w->half ? 2 : sizeof(float);
	w->bytes = w->bytes - 6 * n * before + 6 * n * esz;
	w->bytes = storage == ALISGPU_STORAGE_HALF ? w->bytes + halfPlaneBytes(w) : w->bytes - halfPlaneBytes(w);
	w->half = storage;
	return w->half ? halfStateReset(w) : ALISGPU_OK;
}

extern "C" int alisgpu_world_reset(alisgpu_world *w)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	gOps++;
	fullJoin();
	if (w) w->pendingE.clear();
	if (!w) return alisgpu__fail(ALISGPU_EINVAL, "world_reset: null world");
	size_t n = w->L.elems() * (w->half ? 2 : sizeof(float));
	if (w->half) {
		int rc = halfStateReset(w);
		if (rc) return rc;
	}
	w->written = false;
	for (int m = 0; m <= w->g.complexField; m++) for (int c = 0; c < 3; c++) {
		ALIS_CUDA(cudaMemsetAsync(w->E[m][c], 0, n, gStream));
		ALIS_CUDA(cudaMemsetAsync(w->H[m][c], 0, n, gStream));
	}
	for (int grid = 0; grid < 2; grid++) for (int m = 0; m < 2; m++) for (int f = 0; f < 6; f++) for (int q = 0; q < 2; q++) {
		BoxArr &b = w->psi[grid][m][f][q];
		if (b.p) ALIS_CUDA(cudaMemsetAsync(b.p, 0, b.elems() * sizeof(float), gStream));
	}
	for (DevObj &o : w->objs) {
		size_t cells = (size_t)(1 + o.i1 - o.i0) * o.si;
		for (int m = 0; m < 2; m++) for (int p = 0; p < ALIS_MAXPOLES; p++) for (int a = 0; a < 3; a++) {
			if (o.J[m][p][a]) ALIS_CUDA(cudaMemsetAsync(o.J[m][p][a], 0, cells * sizeof(float), gStream));
			if (o.K[m][p][a]) ALIS_CUDA(cudaMemsetAsync(o.K[m][p][a], 0, cells * sizeof(float), gStream));
		}
	}
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// uploads and downloads
// ---------------------------------------------------------------------
static int upload1D(alisgpu_world *w, float **dst, const float *src, int n)
{
	if (*dst) { alisgpu__freeAsync(*dst); *dst = 0; }
	if (!src) return ALISGPU_OK;
	ALIS_CUDA(alisgpu__mallocAsync(dst, n * sizeof(float)));
	ALIS_CUDA(orderedCopy(*dst, src, n * sizeof(float), cudaMemcpyHostToDevice));
	(void)w;
	return ALISGPU_OK;
}

extern "C" int alisgpu_set_line_tables(alisgpu_world *w, int grid, const float *const dtd[3], const float *const cpml[9])
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w || grid < 0 || grid > 1 || !dtd) return alisgpu__fail(ALISGPU_EINVAL, "set_line_tables: bad argument");
	int len[3] = { w->g.iMAX - w->g.iMIN + 1, w->g.jMAX - w->g.jMIN + 1, w->g.kMAX - w->g.kMIN + 1 };
	int rc;
	for (int a = 0; a < 3; a++) if ((rc = upload1D(w, &w->dtd[grid][a], dtd[a], len[a]))) return rc;
	for (int q = 0; q < 9; q++) if ((rc = upload1D(w, &w->cp[grid][q], cpml ? cpml[q] : 0, len[q / 3]))) return rc;
	return ALISGPU_OK;
}

extern "C" int alisgpu_set_spacing(alisgpu_world *w, const float *const dE[3], const float *const dH[3])
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w || !dE || !dH) return alisgpu__fail(ALISGPU_EINVAL, "set_spacing: bad argument");
	const alisgpu_geometry &g = w->g;
	int len[3] = { g.iMAX - g.iMIN + 1, g.jMAX - g.jMIN + 1, g.kMAX - g.kMIN + 1 }, rc;
	for (int a = 0; a < 3; a++) {
		if ((rc = upload1D(w, &w->sp[0][a], dE[a], len[a]))) return rc;
		if ((rc = upload1D(w, &w->sp[1][a], dH[a], len[a]))) return rc;
	}
	return ALISGPU_OK;
}

// host box [i0,i1]x[j0,j1]x[k0,k1] -> device halo'd layout
static int uploadBoxToLayout(alisgpu_world *w, float *dev, const float *host, int i0, int i1, int j0, int j1, int k0, int k1)
{
	int nj = 1 + j1 - j0, nk = 1 + k1 - k0;
	for (int i = i0; i <= i1; i++) {
		const float *src = host + (size_t)(i - i0) * nj * nk;
		float *dst = dev + w->L.at(i, j0, k0);
		ALIS_CUDA(cudaMemcpy2DAsync(dst, w->L.sj * sizeof(float), src, nk * sizeof(float), nk * sizeof(float), nj,
		                            cudaMemcpyHostToDevice, gStream));
	}
	return ALISGPU_OK;
}

extern "C" int alisgpu_set_eps(alisgpu_world *w, const float *cx, const float *cy, const float *cz)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w) return alisgpu__fail(ALISGPU_EINVAL, "set_eps: null world");
	const alisgpu_geometry &g = w->g;
	const float *src[3] = { cx, cy, cz };
	int rc;
	for (int a = 0; a < 3; a++) {
		if (!src[a]) {
			if (w->C[a]) { cudaStreamSynchronize(gStream); alisgpu__freeAsync(w->C[a]); w->bytes -= w->L.elems() * sizeof(float); w->C[a] = 0; }
			continue;
		}
		if (!w->C[a] && (rc = devAlloc(w, &w->C[a], w->L.elems()))) return rc;
		int i1 = g.iMAX + (a == 0), j1 = g.jMAX + (a == 1), k1 = g.kMAX + (a == 2);
		if ((rc = uploadBoxToLayout(w, w->C[a], src[a], g.iMIN, i1, g.jMIN, j1, g.kMIN, k1))) return rc;
	}
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	// the E half step reads (C[0], C[1], C[2]) at the cells of [MIN, MAX]^3:
	// with at most 256 distinct triples it reads a byte per cell instead,
	// with at most 65536 two bytes (supersampled object edges)
	if (w->matIdx) { alisgpu__freeAsync(w->matIdx); w->matIdx = 0; }
	if (w->matTab) { alisgpu__freeAsync(w->matTab); w->matTab = 0; }
	w->matWide = 0;
	if (cx && cy && cz) {
		const int ni = g.iMAX - g.iMIN + 1, nj = g.jMAX - g.jMIN + 1, nk = g.kMAX - g.kMIN + 1;
		std::vector<unsigned short> idx(w->L.elems(), 0);
		std::vector<float4> tab;
		// distinct triples by their bits, numbered in first-seen order
		struct Key { unsigned b[3]; bool operator==(const Key &o) const { return !memcmp(b, o.b, sizeof b); } };
		struct KeyHash {
			size_t operator()(const Key &k) const {
				unsigned long long h = 0x9e3779b97f4a7c15ull;
				for (int a = 0; a < 3; a++) h = (h ^ k.b[a]) * 0x100000001b3ull;
				return (size_t)(h ^ (h >> 29));
			}
		};
		std::unordered_map<Key, int, KeyHash> seen;
		Key last = { { 0, 0, 0 } };
		int lastQ = -1;
		bool ok = true;
		for (int i = 0; i < ni && ok; i++) for (int j = 0; j < nj && ok; j++) for (int k = 0; k < nk; k++) {
			const float v[3] = { cx[((size_t)i * nj + j) * nk + k], cy[((size_t)i * (nj + 1) + j) * nk + k],
			                     cz[((size_t)i * nj + j) * (nk + 1) + k] };
			Key key;
			memcpy(key.b, v, sizeof key.b);
			int q = lastQ;
			if (q < 0 || !(key == last)) {
				auto it = seen.find(key);
				if (it != seen.end()) q = it->second;
				else {
					if (tab.size() == 65536) { ok = false; break; }
					q = (int)tab.size();
					seen.emplace(key, q);
					tab.push_back(make_float4(v[0], v[1], v[2], 0.0f));
				}
				last = key, lastQ = q;
			}
			idx[w->L.at(g.iMIN + i, g.jMIN + j, g.kMIN + k)] = (unsigned short)q;
		}
		if (ok) {
			w->matWide = tab.size() > 256;
			if (w->matWide) {
				ALIS_CUDA(alisgpu__mallocAsync((unsigned short **)&w->matIdx, idx.size() * sizeof(unsigned short)));
				ALIS_CUDA(orderedCopy(w->matIdx, idx.data(), idx.size() * sizeof(unsigned short), cudaMemcpyHostToDevice));
			} else {
				std::vector<unsigned char> narrow(idx.begin(), idx.end());
				ALIS_CUDA(alisgpu__mallocAsync((unsigned char **)&w->matIdx, narrow.size()));
				ALIS_CUDA(orderedCopy(w->matIdx, narrow.data(), narrow.size(), cudaMemcpyHostToDevice));
			}
			ALIS_CUDA(alisgpu__mallocAsync(&w->matTab, tab.size() * sizeof(float4)));
			ALIS_CUDA(orderedCopy(w->matTab, tab.data(), tab.size() * sizeof(float4), cudaMemcpyHostToDevice));
		}
	}
	return ALISGPU_OK;
}

// ALISGPU_PRECISE_CONDUCTION=1: a conducting object's E loses E b per step,
// b = 2 a u / (1 + a u), instead of being multiplied by the reference's
// q = (1 - a u) / (1 + a u) = 1 - b.  q is rounded to float the same way
// at every step, so the reference's field drifts by the step count times
// that rounding (2.85e-4 of the benchmark world's flux after 4000 steps);
// the rounding of b moves the applied factor b times as little.  An
// opt-in precision mode: results then differ from the reference's.
static bool preciseConduction()
{
	static const bool on = [] {
		const char *e = getenv("ALISGPU_PRECISE_CONDUCTION");
		return e && e[0] == '1';
	}();
	return on;
}

extern "C" int alisgpu_set_dispersive(alisgpu_world *w, int n, const alisgpu_dispersive *objs)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w || n < 0 || (n && !objs)) return alisgpu__fail(ALISGPU_EINVAL, "set_dispersive: bad argument");
	cudaStreamSynchronize(gStream);
	freeObjects(w);
	for (int q = 0; q < n; q++) {
		const alisgpu_dispersive &s = objs[q];
		if (s.NK > ALIS_MAXPOLES || s.NJ > s.NK || s.NJ < 0)
			return alisgpu__fail(ALISGPU_ERANGE, "set_dispersive: object %d has %d poles (max %d)", q, s.NK, ALIS_MAXPOLES);
		DevObj o;
		memset(&o, 0, sizeof o);
		o.i0 = s.iMin, o.i1 = s.iMax, o.j0 = s.jMin, o.j1 = s.jMax, o.k0 = s.kMin, o.k1 = s.kMax;
		o.NJ = s.NJ, o.NK = s.NK;
		o.sj = 1 + o.k1 - o.k0;
		o.si = o.sj * (1 + o.j1 - o.j0);
		size_t cells = (size_t)(1 + o.i1 - o.i0) * o.si;
		for (int a = 0; a < 3; a++) {
			o.a[a] = s.a[a];
			for (int p = 0; p < s.NK; p++) {
				o.JJ[p][a] = s.JJ[a][p], o.JK[p][a] = s.JK[a] ? s.JK[a][p] : 0, o.JE[p][a] = s.JE[a][p];
				if (p >= s.NJ) o.KJ[p][a] = s.KJ[a][p], o.KK[p][a] = s.KK[a][p], o.KE[p][a] = s.KE[a][p];
			}
			float *d;
			int rc = devAlloc(w, &d, cells);
			if (rc) return rc;
			w->objMem.push_back(d);
			ALIS_CUDA(orderedCopy(d, s.fill[a], cells * sizeof(float), cudaMemcpyHostToDevice));
			o.fill[a] = d;
		}
		o.cond = s.a[0] != 0 || s.a[1] != 0 || s.a[2] != 0 ? (preciseConduction() ? 2 : 1) : 0;
		for (int m = 0; m <= w->g.complexField; m++) for (int p = 0; p < s.NK; p++) for (int a = 0; a < 3; a++) {
			float *d;
			int rc = devAlloc(w, &d, cells);
			if (rc) return rc;
			w->objMem.push_back(d);
			o.J[m][p][a] = d;
			if (p >= s.NJ) {
				if ((rc = devAlloc(w, &d, cells))) return rc;
				w->objMem.push_back(d);
				o.K[m][p][a] = d;
			}
		}
		w->objs.push_back(o);
	}
	if (n) {
		ALIS_CUDA(alisgpu__mallocAsync(&w->dObjs, n * sizeof(DevObj)));
		ALIS_CUDA(orderedCopy(w->dObjs, w->objs.data(), n * sizeof(DevObj), cudaMemcpyHostToDevice));
	}
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

static float *fieldPtr(alisgpu_world *w, int field, int m, int comp)
{
	if (field < 0 || field > 1 || m < 0 || m > w->g.complexField || comp < 0 || comp > 2) return 0;
	return field ? w->H[m][comp] : w->E[m][comp];
}

// one component of a half world as floats, rows of nk in the host's order
__global__ void k_field_decode(const float *src, const signed char *ex, const Layout L, float *out)
{
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long long)L.ni * L.nj * L.nk) return;
	const long long row = t / L.nk;
	const int kk = (int)(t - row * L.nk);
	out[t] = halfAt(src, row * L.sj + ALIS_KOFF + kk, pow2f(ex[row / L.nj]));
}

// the world's observer scratch, grown to n floats
static int scratchFloats(alisgpu_world *w, size_t n)
{
	if (n <= w->planeTabFloats) return ALISGPU_OK;
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	if (w->planeTab) alisgpu__freeAsync(w->planeTab);
	w->planeTab = 0, w->planeTabFloats = 0;
	ALIS_CUDA(alisgpu__mallocAsync(&w->planeTab, n * sizeof(float)));
	w->planeTabFloats = n;
	return ALISGPU_OK;
}

extern "C" int alisgpu_field_download(alisgpu_world *w, int field, int m, int comp, float *host)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (w) {
		int rc = applyPendingGhosts(w);
		if (rc) return rc;
	}
	float *d = w && host ? fieldPtr(w, field, m, comp) : 0;
	if (!d) return alisgpu__fail(ALISGPU_EINVAL, "field_download: bad argument");
	const Layout &L = w->L;
	if (w->half) {
		const size_t n = (size_t)L.ni * L.nj * L.nk;
		int rc = scratchFloats(w, n);
		if (rc) return rc;
		k_field_decode<<<(unsigned)((n + 255) / 256), 256, 0, gStream>>>(d, halfRead(w, field) + comp * L.ni, L, w->planeTab);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
		ALIS_CUDA(cudaMemcpyAsync(host, w->planeTab, n * sizeof(float), cudaMemcpyDeviceToHost, gStream));
		ALIS_CUDA(cudaStreamSynchronize(gStream));
		return ALISGPU_OK;
	}
	ALIS_CUDA(cudaMemcpy2DAsync(host, L.nk * sizeof(float), d + ALIS_KOFF, L.sj * sizeof(float), L.nk * sizeof(float),
	                            (size_t)L.ni * L.nj, cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

extern "C" int alisgpu_field_upload(alisgpu_world *w, int field, int m, int comp, const float *host)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	gOps++;
	fullJoin();
	if (w && field == 0) w->pendingE.clear();        // the host's halo wins
	float *d = w && host ? fieldPtr(w, field, m, comp) : 0;
	if (!d) return alisgpu__fail(ALISGPU_EINVAL, "field_upload: bad argument");
	if (w->half) return alisgpu__fail(ALISGPU_ENOTSUP, "field_upload: the world stores half values");
	w->written = true;
	const Layout &L = w->L;
	ALIS_CUDA(cudaMemcpy2DAsync(d + ALIS_KOFF, L.sj * sizeof(float), host, L.nk * sizeof(float), L.nk * sizeof(float),
	                            (size_t)L.ni * L.nj, cudaMemcpyHostToDevice, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

// every current array of one object in one gather launch and one copy
#define CUR_MAX (2 * ALIS_MAXPOLES * 3 * 2)
struct CurGather { const float *src[CUR_MAX]; int count; long long cells; float *out; };

__global__ void k_current_gather(const CurGather P)
{
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= P.cells * P.count) return;
	P.out[t] = P.src[t / P.cells][t % P.cells];
}

extern "C" int alisgpu_object_currents_download(alisgpu_world *w, int n, float *host)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w || !host || n < 0 || n >= (int)w->objs.size()) return alisgpu__fail(ALISGPU_EINVAL, "object_currents_download: bad argument");
	const DevObj &o = w->objs[n];
	CurGather P;
	memset(&P, 0, sizeof P);
	P.cells = (long long)(1 + o.i1 - o.i0) * o.si;
	for (int m = 0; m <= w->g.complexField; m++)
		for (int p = 0; p < o.NK; p++) for (int c = 0; c < 3; c++) {
			P.src[P.count++] = o.J[m][p][c];
			if (p >= o.NJ) P.src[P.count++] = o.K[m][p][c];
		}
	if (!P.count || !P.cells) return ALISGPU_OK;
	const size_t n4 = (size_t)P.cells * P.count;
	if (n4 > w->planeTabFloats) {
		ALIS_CUDA(cudaStreamSynchronize(gStream));
		if (w->planeTab) alisgpu__freeAsync(w->planeTab);
		w->planeTab = 0, w->planeTabFloats = 0;
		ALIS_CUDA(alisgpu__mallocAsync(&w->planeTab, n4 * sizeof(float)));
		w->planeTabFloats = n4;
	}
	P.out = w->planeTab;
	k_current_gather<<<(unsigned)((n4 + 255) / 256), 256, 0, gStream>>>(P);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	ALIS_CUDA(cudaMemcpyAsync(host, P.out, n4 * sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

extern "C" int alisgpu_current_download(alisgpu_world *w, int n, int m, int p, int comp, int isK, float *host)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	fullJoin();
	if (!w || !host || n < 0 || n >= (int)w->objs.size() || m < 0 || m > w->g.complexField || comp < 0 || comp > 2)
		return alisgpu__fail(ALISGPU_EINVAL, "current_download: bad argument");
	DevObj &o = w->objs[n];
	if (p < 0 || p >= o.NK || (isK && p < o.NJ)) return alisgpu__fail(ALISGPU_EINVAL, "current_download: bad pole");
	float *d = isK ? o.K[m][p][comp] : o.J[m][p][comp];
	size_t cells = (size_t)(1 + o.i1 - o.i0) * o.si;
	ALIS_CUDA(cudaMemcpyAsync(host, d, cells * sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// the fused half-step kernel
// ---------------------------------------------------------------------

// aux-world index of a main-world cell, with the row aliasing of the
// reference's expandFieldX/Y (src/source.c:223-249)
__device__ __forceinline__ long long auxAt(const DevTfsf &t, int i, int j, int k, int altX, int altY)
{
	if (t.aliasX && i > t.auxIMAX) i = t.auxIMAX + altX;
	if (t.aliasY && j > t.auxJMAX) j = t.auxJMAX + altY;
	// outside the auxiliary grid the reference reads undefined memory;
	// here the sample is skipped and the error word records it
	if (i < t.L.i0 || i >= t.L.i0 + t.L.ni || j < t.L.j0 || j >= t.L.j0 + t.L.nj || k < t.L.k0 || k >= t.L.k0 + t.L.nk)
		return -1;
	return t.L.at(i, j, k);
}

// aux sample, 0 (and error bit 1) when outside the auxiliary grid
__device__ __forceinline__ float auxGet(const float *A, long long q, unsigned int *err)
{
	if (q < 0) { atomicOr(err, 1u); return 0.0f; }
	return A[q];
}

// Pieces of the per-cell half step, in the reference order.  ALT = +1: E
// half step (neighbours at +1); ALT = -1: H half step (neighbours at -1).
// g*0 are the other field at the cell, gyk/gxk its k neighbours, gzj/gxj
// its j neighbours, gzi/gyi its i neighbours.

// objects whose box holds the cell, in list order: the tile's list when the
// world has more than 8 objects, else every object whose class bit is set
#define FOR_CELL_OBJECTS(...)                                                               \
	for (int q_ = 0; q_ < nIter; q_++) {                                                    \
		const int n_ = list ? list[q_] : q_;                                                \
		if (!list && n_ < 8 && !((objm >> n_) & 1u)) continue;                              \
		const DevObj &o = P.obj[n_];                                                        \
		if (i < o.i0 || i > min(o.i1, P.iMAX) || j < o.j0 || j > min(o.j1, P.jMAX) ||       \
		    k < o.k0 || k > min(o.k1, P.kMAX)) continue;                                    \
		const int b = (i - o.i0) * (int)o.si + (j - o.j0) * (int)o.sj + (k - o.k0);         \
		__VA_ARGS__                                                                         \
	}

// conductivity factors, then polarisation currents (reference
// src/update.c:89-108); E half step only -- H is updated with CH, whose
// object list is always empty
__device__ __forceinline__ void objectsBeforeCurl(const HalfStepParams &P, int i, int j, int k,
	float &fx, float &fy, float &fz, unsigned objm, const int *list, int nIter)
{
	FOR_CELL_OBJECTS(
		if (o.cond == 1) {
			float ux = o.fill[0][b], uy = o.fill[1][b], uz = o.fill[2][b];
			fx *= (1 - o.a[0] * ux) / (1 + o.a[0] * ux);
			fy *= (1 - o.a[1] * uy) / (1 + o.a[1] * uy);
			fz *= (1 - o.a[2] * uz) / (1 + o.a[2] * uz);
		} else if (o.cond) {
			// the compensated form (ALISGPU_PRECISE_CONDUCTION=1)
			float px = o.a[0] * o.fill[0][b], py = o.a[1] * o.fill[1][b], pz = o.a[2] * o.fill[2][b];
			fx -= fx * (2 * px / (1 + px));
			fy -= fy * (2 * py / (1 + py));
			fz -= fz * (2 * pz / (1 + pz));
		})
	FOR_CELL_OBJECTS(
		for (int p = 0; p < o.NK; p++) {
			fx -= o.J[P.m][p][0][b];
			fy -= o.J[P.m][p][1][b];
			fz -= o.J[P.m][p][2][b];
		})
}

// ADE currents driven by E, run inside updateH (reference src/update.c:128-158)
__device__ __forceinline__ void objectsAfterCurl(const HalfStepParams &P, int i, int j, int k,
	float gx0, float gy0, float gz0, unsigned objm, const int *list, int nIter)
{
	// poles outer, the three axes inner: the axes' updates of a pole are
	// independent, and each current sees the same operations as in the
	// reference's loop order
	FOR_CELL_OBJECTS(
		const float e[3] = { gx0, gy0, gz0 };
		const float fe[3] = { o.fill[0][b], o.fill[1][b], o.fill[2][b] };
		for (int p = 0; p < o.NJ; p++) {
#pragma unroll
			for (int a = 0; a < 3; a++) {
				float *J = o.J[P.m][p][a];
				J[b] = o.JJ[p][a] * J[b] + o.JE[p][a] * fe[a] * e[a];
			}
		}
		for (int p = o.NJ; p < o.NK; p++) {
#pragma unroll
			for (int a = 0; a < 3; a++) {
				float *J = o.J[P.m][p][a], *K = o.K[P.m][p][a];
				float jn = o.JJ[p][a] * J[b] + o.JK[p][a] * K[b] + o.JE[p][a] * fe[a] * e[a];
				J[b] = jn;
				K[b] = o.KJ[p][a] * jn + o.KK[p][a] * K[b] + o.KE[p][a] * fe[a] * e[a];
			}
		})
}

// CPML of face F (xMin,yMin,zMin,xMax,yMax,zMax), reference src/update.c:48-84, 119-124
template <int F>
__device__ __forceinline__ void pmlFace(const HalfStepParams &P, int i, int j, int k,
	float &fx, float &fy, float &fz, float gx0, float gy0, float gz0,
	float gyk, float gxk, float gzj, float gxj, float gzi, float gyi,
	bool hasC, float cx, float cy, float cz)
{
	const BoxArr &A = P.psi[F][0], &B = P.psi[F][1];
	const int a = (i - A.i0) * (int)A.si + (j - A.j0) * (int)A.sj + (k - A.k0);
	if (F % 3 == 0) {
		const int q = i - P.iMIN;
		float py = P.cp[0][q] * A.p[a] + P.cp[1][q] * (gz0 - gzi);
		float pz = P.cp[0][q] * B.p[a] + P.cp[2][q] * (gy0 - gyi);
		A.p[a] = py, B.p[a] = pz;
		if (hasC) fy += py * cy, fz += pz * cz; else fy += py, fz += pz;
	} else if (F % 3 == 1) {
		const int q = j - P.jMIN;
		float pz = P.cp[3][q] * A.p[a] + P.cp[4][q] * (gx0 - gxj);
		float px = P.cp[3][q] * B.p[a] + P.cp[5][q] * (gz0 - gzj);
		A.p[a] = pz, B.p[a] = px;
		if (hasC) fz += pz * cz, fx += px * cx; else fz += pz, fx += px;
	} else {
		const int q = k - P.kMIN;
		float px = P.cp[6][q] * A.p[a] + P.cp[7][q] * (gy0 - gyk);
		float py = P.cp[6][q] * B.p[a] + P.cp[8][q] * (gx0 - gxk);
		A.p[a] = px, B.p[a] = py;
		if (hasC) fx += px * cx, fy += py * cy; else fx += px, fy += py;
	}
}

// TFSF incident-field corrections (reference src/update.c:205-272).
// E step: aux H; H step: aux E.  Face-by-face in the reference order;
// (dtds * G) * C rounds like the reference's `dtds * G[..] * C[..]`.
// KONLY: the cell lies on no i or j face plane, only the k faces apply.
template <int ALT, bool KONLY = false>
__device__ __forceinline__ void tfsfCell(const HalfStepParams &P, int i, int j, int k,
	float &fx, float &fy, float &fz, bool hasC, float cx, float cy, float cz)
{
	for (int s = 0; s < P.ntfsf; s++) {
		const DevTfsf &T = P.tf[s];
		const float *A0 = T.G[P.m][0], *A1 = T.G[P.m][1], *A2 = T.G[P.m][2];
		if (ALT == 1) {
			// alias Alt of the aux H components: x rows (0,1,1), y rows (1,0,1)
			if (!KONLY && T.iMin > P.iMIN && i == T.iMin) {
				if (j >= T.jMin && j <= T.jMax && k >= T.kMIN && k <= T.kMAX) { float v = -T.dtdMin[0] * auxGet(A1, auxAt(T, i, j, k, 1, 0), P.err); fz += hasC ? v * cz : v; }
				if (j >= T.jMIN && j <= T.jMAX && k >= T.kMin && k <= T.kMax) { float v = T.dtdMin[0] * auxGet(A2, auxAt(T, i, j, k, 1, 1), P.err); fy += hasC ? v * cy : v; }
			}
			if (!KONLY && T.jMin > P.jMIN && j == T.jMin) {
				if (i >= T.iMIN && i <= T.iMAX && k >= T.kMin && k <= T.kMax) { float v = -T.dtdMin[1] * auxGet(A2, auxAt(T, i, j, k, 1, 1), P.err); fx += hasC ? v * cx : v; }
				if (i >= T.iMin && i <= T.iMax && k >= T.kMIN && k <= T.kMAX) { float v = T.dtdMin[1] * auxGet(A0, auxAt(T, i, j, k, 0, 1), P.err); fz += hasC ? v * cz : v; }
			}
			if (T.kMin > P.kMIN && k == T.kMin) {
				if (i >= T.iMin && i <= T.iMax && j >= T.jMIN && j <= T.jMAX) { float v = -T.dtdMin[2] * auxGet(A0, auxAt(T, i, j, k, 0, 1), P.err); fy += hasC ? v * cy : v; }
				if (i >= T.iMIN && i <= T.iMAX && j >= T.jMin && j <= T.jMax) { float v = T.dtdMin[2] * auxGet(A1, auxAt(T, i, j, k, 1, 0), P.err); fx += hasC ? v * cx : v; }
			}
			if (!KONLY && T.iMax < P.iMAX && i == T.iMax) {
				if (j >= T.jMin && j <= T.jMax && k >= T.kMIN && k <= T.kMAX) { float v = T.dtdMax[0] * auxGet(A1, auxAt(T, i + 1, j, k, 1, 0), P.err); fz += hasC ? v * cz : v; }
				if (j >= T.jMIN && j <= T.jMAX && k >= T.kMin && k <= T.kMax) { float v = -T.dtdMax[0] * auxGet(A2, auxAt(T, i + 1, j, k, 1, 1), P.err); fy += hasC ? v * cy : v; }
			}
			if (!KONLY && T.jMax < P.jMAX && j == T.jMax) {
				if (i >= T.iMIN && i <= T.iMAX && k >= T.kMin && k <= T.kMax) { float v = T.dtdMax[1] * auxGet(A2, auxAt(T, i, j + 1, k, 1, 1), P.err); fx += hasC ? v * cx : v; }
				if (i >= T.iMin && i <= T.iMax && k >= T.kMIN && k <= T.kMAX) { float v = -T.dtdMax[1] * auxGet(A0, auxAt(T, i, j + 1, k, 0, 1), P.err); fz += hasC ? v * cz : v; }
			}
			if (T.kMax < P.kMAX && k == T.kMax) {
				if (i >= T.iMin && i <= T.iMax && j >= T.jMIN && j <= T.jMAX) { float v = T.dtdMax[2] * auxGet(A0, auxAt(T, i, j, k + 1, 0, 1), P.err); fy += hasC ? v * cy : v; }
				if (i >= T.iMIN && i <= T.iMAX && j >= T.jMin && j <= T.jMax) { float v = -T.dtdMax[2] * auxGet(A1, auxAt(T, i, j, k + 1, 1, 0), P.err); fx += hasC ? v * cx : v; }
			}
		} else {
			// alias Alt of the aux E components: x rows (1,0,0), y rows (0,1,0)
			if (!KONLY && T.iMin > P.iMIN && i == T.iMin) {
				if (j >= T.jMIN && j <= T.jMAX && k >= T.kMin && k <= T.kMax) fz += T.dtdMin[0] * auxGet(A1, auxAt(T, i, j, k, 0, 1), P.err);
				if (j >= T.jMin && j <= T.jMax && k >= T.kMIN && k <= T.kMAX) fy += -T.dtdMin[0] * auxGet(A2, auxAt(T, i, j, k, 0, 0), P.err);
			}
			if (!KONLY && T.jMin > P.jMIN && j == T.jMin) {
				if (i >= T.iMin && i <= T.iMax && k >= T.kMIN && k <= T.kMAX) fx += T.dtdMin[1] * auxGet(A2, auxAt(T, i, j, k, 0, 0), P.err);
				if (i >= T.iMIN && i <= T.iMAX && k >= T.kMin && k <= T.kMax) fz += -T.dtdMin[1] * auxGet(A0, auxAt(T, i, j, k, 1, 0), P.err);
			}
			if (T.kMin > P.kMIN && k == T.kMin) {
				if (i >= T.iMIN && i <= T.iMAX && j >= T.jMin && j <= T.jMax) fy += T.dtdMin[2] * auxGet(A0, auxAt(T, i, j, k, 1, 0), P.err);
				if (i >= T.iMin && i <= T.iMax && j >= T.jMIN && j <= T.jMAX) fx += -T.dtdMin[2] * auxGet(A1, auxAt(T, i, j, k, 0, 1), P.err);
			}
			if (!KONLY && T.iMax < P.iMAX && i == T.iMax + 1) {
				if (j >= T.jMIN && j <= T.jMAX && k >= T.kMin && k <= T.kMax) fz += -T.dtdMax[0] * auxGet(A1, auxAt(T, i - 1, j, k, 0, 1), P.err);
				if (j >= T.jMin && j <= T.jMax && k >= T.kMIN && k <= T.kMAX) fy += T.dtdMax[0] * auxGet(A2, auxAt(T, i - 1, j, k, 0, 0), P.err);
			}
			if (!KONLY && T.jMax < P.jMAX && j == T.jMax + 1) {
				if (i >= T.iMin && i <= T.iMax && k >= T.kMIN && k <= T.kMAX) fx += -T.dtdMax[1] * auxGet(A2, auxAt(T, i, j - 1, k, 0, 0), P.err);
				if (i >= T.iMIN && i <= T.iMAX && k >= T.kMin && k <= T.kMax) fz += T.dtdMax[1] * auxGet(A0, auxAt(T, i, j - 1, k, 1, 0), P.err);
			}
			if (T.kMax < P.kMAX && k == T.kMax + 1) {
				if (i >= T.iMIN && i <= T.iMAX && j >= T.jMin && j <= T.jMax) fy += -T.dtdMax[2] * auxGet(A0, auxAt(T, i, j, k - 1, 1, 0), P.err);
				if (i >= T.iMin && i <= T.iMax && j >= T.jMIN && j <= T.jMAX) fx += T.dtdMax[2] * auxGet(A1, auxAt(T, i, j, k - 1, 0, 1), P.err);
			}
		}
	}
}

// Field loads and stores of a half step.  Float storage, or (HALF) IEEE
// half values times the plane's power of two.  The scales are the same
// for a warp (one plane): uniform loads from the plane's entry of the
// step's table, the other field's at plane i (HS_G) and i + ALT (HS_GI),
// the stepped field's as stored (HS_F) and the inverse scales the step
// stores with (HS_INV).
#define HS_T(i) (P.h.tab + (size_t)((i) - P.L.i0) * HALF_TAB)
#define HS_G(q) (HALF ? __ldg(HS_T(i) + (q)) : 1.0f)
#define HS_GI(q) (HALF ? __ldg(HS_T(i) + 3 + (q)) : 1.0f)
#define HS_F(q) (HALF ? __ldg(HS_T(i) + 6 + (q)) : 1.0f)
#define HS_INV(q) __ldg(HS_T(i) + 9 + (q))
template <bool HALF>
__device__ __forceinline__ float ldG(const float *p, int c, float s)
{
	if (HALF) return __half2float(__ushort_as_half(__ldg((const unsigned short *)p + c))) * s;
	return __ldg(p + c);
}
template <bool HALF>
__device__ __forceinline__ float ldF(const float *p, int c, float s)
{
	if (HALF) return halfAt(p, c, s);
	return p[c];
}
template <bool HALF>
__device__ __forceinline__ void stF(float *p, int c, float v, float inv)
{
	if (HALF) ((unsigned short *)p)[c] = halfOf(v, inv);
	else p[c] = v;
}
// the step's largest magnitudes per component of plane i (float bits of
// |v|, NaN above infinity): a maximum over the lanes here, one atomic per
// component into one of the plane's HALF_SLOTS words, chosen by the
// warp's position, so that the plane's warps spread over them
__device__ __forceinline__ void halfMax(const HalfStepParams &P, int i, float fx, float fy, float fz)
{
	const unsigned mask = __activemask();
	const unsigned ax = __reduce_max_sync(mask, __float_as_uint(fabsf(fx)));
	const unsigned ay = __reduce_max_sync(mask, __float_as_uint(fabsf(fy)));
	const unsigned az = __reduce_max_sync(mask, __float_as_uint(fabsf(fz)));
	if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) {
		const int slot = (int)((blockIdx.x * blockDim.y + blockIdx.y + threadIdx.y) % HALF_SLOTS);
		unsigned *m = P.h.mCur + (size_t)(i - P.L.i0) * HALF_SLOTS + slot;
		const size_t comp = (size_t)P.L.ni * HALF_SLOTS;
		atomicMax(m, ax);
		atomicMax(m + comp, ay);
		atomicMax(m + 2 * comp, az);
	}
}
template <bool HALF>
__device__ __forceinline__ void storeCell(const HalfStepParams &P, int i, int c, float fx, float fy, float fz)
{
	if (HALF) {
		stF<true>(P.F[0], c, fx, HS_INV(0));
		stF<true>(P.F[1], c, fy, HS_INV(1));
		stF<true>(P.F[2], c, fz, HS_INV(2));
		halfMax(P, i, fx, fy, fz);
	} else {
		P.F[0][c] = fx, P.F[1][c] = fy, P.F[2][c] = fz;
	}
}

// One cell of a half step, in the reference order: conductivity and -J
// (E), curl, CPML faces, TFSF corrections, ADE update (H).  Three per-axis
// bit tables classify the cell by its i, j and k (CPML slab side, TFSF face
// plane, dispersive object range); a cell with none of these bits takes
// only the curl.  list/nIter: the objects to visit (a tile's list, or all
// objects filtered by the class bits when list is null).
template <int ALT, bool HALF = false>
__device__ __forceinline__ void stepCell(const HalfStepParams &P, int i, int j, int k, const int *list, int nIter)
{
	const int sj = (int)P.L.sj, si = (int)P.L.si;
	const int c = (i - P.L.i0) * si + (j - P.L.j0) * sj + (k - P.L.k0) + ALIS_KOFF;
	const unsigned bi = __ldg(P.cls[0] + (i - P.iMIN)), bj = __ldg(P.cls[1] + (j - P.jMIN)), bk = __ldg(P.cls[2] + (k - P.kMIN));
	const unsigned any = bi | bj | bk;
	const unsigned objm = bi & bj & bk & 0x1FFu;
	const float *Gx = P.G[0], *Gy = P.G[1], *Gz = P.G[2];
	const float sx = HS_G(0), sy = HS_G(1), sz = HS_G(2);
	const float gx0 = ldG<HALF>(Gx, c, sx), gy0 = ldG<HALF>(Gy, c, sy), gz0 = ldG<HALF>(Gz, c, sz);
	const float gyk = ldG<HALF>(Gy, c + ALT, sy), gxk = ldG<HALF>(Gx, c + ALT, sx);
	const float gzj = ldG<HALF>(Gz, c + ALT * sj, sz), gxj = ldG<HALF>(Gx, c + ALT * sj, sx);
	const float gzi = ldG<HALF>(Gz, c + ALT * si, HS_GI(2)), gyi = ldG<HALF>(Gy, c + ALT * si, HS_GI(1));
	float fx = ldF<HALF>(P.F[0], c, HS_F(0)), fy = ldF<HALF>(P.F[1], c, HS_F(1)), fz = ldF<HALF>(P.F[2], c, HS_F(2));
	const bool hasC = P.C[0] != 0;
	float cx = 1, cy = 1, cz = 1;
	if (hasC) cx = __ldg(P.C[0] + c), cy = __ldg(P.C[1] + c), cz = __ldg(P.C[2] + c);

	if (ALT == 1 && objm) objectsBeforeCurl(P, i, j, k, fx, fy, fz, objm, list, nIter);

	// curl (reference src/update.c:109-118)
	const float dx = __ldg(P.dtd[0] + (i - P.iMIN)), dy = __ldg(P.dtd[1] + (j - P.jMIN)), dz = __ldg(P.dtd[2] + (k - P.kMIN));
	if (hasC) {
		fx += (dz * (gy0 - gyk) + dy * (gzj - gz0)) * cx;
		fy += (dx * (gz0 - gzi) + dz * (gxk - gx0)) * cy;
		fz += (dy * (gx0 - gxj) + dx * (gyi - gy0)) * cz;
	} else {
		fx += (dz * (gy0 - gyk) + dy * (gzj - gz0));
		fy += (dx * (gz0 - gzi) + dz * (gxk - gx0));
		fz += (dy * (gx0 - gxj) + dx * (gyi - gy0));
	}
	// CPML faces in the reference order xMin, yMin, zMin, xMax, yMax, zMax
	if (any & (CLS_PML_LO | CLS_PML_HI)) {
#define PML_ARGS P, i, j, k, fx, fy, fz, gx0, gy0, gz0, gyk, gxk, gzj, gxj, gzi, gyi, hasC, cx, cy, cz
		if (bi & CLS_PML_LO) pmlFace<0>(PML_ARGS);
		if (bj & CLS_PML_LO) pmlFace<1>(PML_ARGS);
		if (bk & CLS_PML_LO) pmlFace<2>(PML_ARGS);
		if (bi & CLS_PML_HI) pmlFace<3>(PML_ARGS);
		if (bj & CLS_PML_HI) pmlFace<4>(PML_ARGS);
		if (bk & CLS_PML_HI) pmlFace<5>(PML_ARGS);
#undef PML_ARGS
	}
	if (tfsfBits(bi, bj, bk)) tfsfCell<ALT>(P, i, j, k, fx, fy, fz, hasC, cx, cy, cz);
	if (ALT == -1 && objm) objectsAfterCurl(P, i, j, k, gx0, gy0, gz0, objm, list, nIter);
	storeCell<HALF>(P, i, c, fx, fy, fz);
}

// Cells on a TFSF face plane or inside a dispersive object box run the
// full sequence out of line (their neighbours' lean code stays small);
// P is the kernel's __grid_constant__ parameter, passed by reference.
template <int ALT, bool HALF = false>
__device__ __noinline__ void hardCell(const HalfStepParams &P, int i, int j, int k, const int *list, int nIter)
{
	stepCell<ALT, HALF>(P, i, j, k, list, nIter);
}

#define TX 32
// Block shapes: TX x TY threads over one i plane, TY rows of 32 cells,
// 32 registers at full occupancy (2048 threads per SM) for every TY.  The
// tuner picks TY per world and field from these by timing its first half
// steps (32 x 4 measured best on the 256^3 dispersive world).
#define ALIS_TY_CHOICES 3
static const int kTyChoice[ALIS_TY_CHOICES] = { 2, 4, 8 };
#define STEP_MINB(TY) (2048 / (TX * (TY)))
// The lean tiers for NC cells k, k + TX, ... of one row, all in range and
// none of them hard: the loads of every cell first, then the updates, so
// the cells' memory round trips overlap and share their index arithmetic.
template <int ALT, int NC, bool HALF = false>
__device__ __forceinline__ void leanCells(const HalfStepParams &P, int i, int j, int k, unsigned bi, unsigned bj, const unsigned *bk)
{
	const int sj = (int)P.L.sj, si = (int)P.L.si;
	const int c0 = (i - P.L.i0) * si + (j - P.L.j0) * sj + (k - P.L.k0) + ALIS_KOFF;
	const float *Gx = P.G[0], *Gy = P.G[1], *Gz = P.G[2];
	float gx0[NC], gy0[NC], gz0[NC], gyk[NC], gxk[NC], gzj[NC], gxj[NC], gzi[NC], gyi[NC];
	float fx[NC], fy[NC], fz[NC], cx[NC], cy[NC], cz[NC], dz[NC];
	const bool hasC = P.C[0] != 0;
#pragma unroll
	for (int q = 0; q < NC; q++) {
		const int c = c0 + q * TX;
		const float sx = HS_G(0), sy = HS_G(1), sz = HS_G(2);
		gx0[q] = ldG<HALF>(Gx, c, sx), gy0[q] = ldG<HALF>(Gy, c, sy), gz0[q] = ldG<HALF>(Gz, c, sz);
		gyk[q] = ldG<HALF>(Gy, c + ALT, sy), gxk[q] = ldG<HALF>(Gx, c + ALT, sx);
		gzj[q] = ldG<HALF>(Gz, c + ALT * sj, sz), gxj[q] = ldG<HALF>(Gx, c + ALT * sj, sx);
		gzi[q] = ldG<HALF>(Gz, c + ALT * si, HS_GI(2)), gyi[q] = ldG<HALF>(Gy, c + ALT * si, HS_GI(1));
		fx[q] = ldF<HALF>(P.F[0], c, HS_F(0)), fy[q] = ldF<HALF>(P.F[1], c, HS_F(1));
		fz[q] = ldF<HALF>(P.F[2], c, HS_F(2));
		dz[q] = __ldg(P.dtd[2] + (k + q * TX - P.kMIN));
		cx[q] = 1, cy[q] = 1, cz[q] = 1;
		if (hasC) {
			if (P.matIdx) {
				// the same floats from the table of distinct triples
				const float4 t = matTriple(P, c);
				cx[q] = t.x, cy[q] = t.y, cz[q] = t.z;
			} else {
				cx[q] = __ldg(P.C[0] + c), cy[q] = __ldg(P.C[1] + c), cz[q] = __ldg(P.C[2] + c);
			}
		}
	}
	const float dx = __ldg(P.dtd[0] + (i - P.iMIN)), dy = __ldg(P.dtd[1] + (j - P.jMIN));
#pragma unroll
	for (int q = 0; q < NC; q++) {
		const int kq = k + q * TX, c = c0 + q * TX;
		// curl (reference src/update.c:109-118)
		if (hasC) {
			fx[q] += (dz[q] * (gy0[q] - gyk[q]) + dy * (gzj[q] - gz0[q])) * cx[q];
			fy[q] += (dx * (gz0[q] - gzi[q]) + dz[q] * (gxk[q] - gx0[q])) * cy[q];
			fz[q] += (dy * (gx0[q] - gxj[q]) + dx * (gyi[q] - gy0[q])) * cz[q];
		} else {
			fx[q] += (dz[q] * (gy0[q] - gyk[q]) + dy * (gzj[q] - gz0[q]));
			fy[q] += (dx * (gz0[q] - gzi[q]) + dz[q] * (gxk[q] - gx0[q]));
			fz[q] += (dy * (gx0[q] - gxj[q]) + dx * (gyi[q] - gy0[q]));
		}
		// CPML faces in the reference order xMin, yMin, zMin, xMax, yMax, zMax
		if ((bi | bj | bk[q]) & (CLS_PML_LO | CLS_PML_HI)) {
#define PML_ARGS P, i, j, kq, fx[q], fy[q], fz[q], gx0[q], gy0[q], gz0[q], gyk[q], gxk[q], gzj[q], gxj[q], gzi[q], gyi[q], hasC, cx[q], cy[q], cz[q]
			if (bi & CLS_PML_LO) pmlFace<0>(PML_ARGS);
			if (bj & CLS_PML_LO) pmlFace<1>(PML_ARGS);
			if (bk[q] & CLS_PML_LO) pmlFace<2>(PML_ARGS);
			if (bi & CLS_PML_HI) pmlFace<3>(PML_ARGS);
			if (bj & CLS_PML_HI) pmlFace<4>(PML_ARGS);
			if (bk[q] & CLS_PML_HI) pmlFace<5>(PML_ARGS);
#undef PML_ARGS
		}
		// TFSF k face planes (cells on an i or j face plane are hard)
		if (tfsfBits(bi, bj, bk[q])) tfsfCell<ALT, true>(P, i, j, kq, fx[q], fy[q], fz[q], hasC, cx[q], cy[q], cz[q]);
		storeCell<HALF>(P, i, c, fx[q], fy[q], fz[q]);
	}
}

// A cell with no class bits: the curl alone (reference
// src/update.c:109-118), with the loads and arithmetic of leanCells.
template <int ALT, bool HALF = false>
__device__ __forceinline__ void plainCell(const HalfStepParams &P, int i, int j, int k)
{
	const int sj = (int)P.L.sj, si = (int)P.L.si;
	const int c = (i - P.L.i0) * si + (j - P.L.j0) * sj + (k - P.L.k0) + ALIS_KOFF;
	const float *Gx = P.G[0], *Gy = P.G[1], *Gz = P.G[2];
	const float sx = HS_G(0), sy = HS_G(1), sz = HS_G(2);
	const float gx0 = ldG<HALF>(Gx, c, sx), gy0 = ldG<HALF>(Gy, c, sy), gz0 = ldG<HALF>(Gz, c, sz);
	const float gyk = ldG<HALF>(Gy, c + ALT, sy), gxk = ldG<HALF>(Gx, c + ALT, sx);
	const float gzj = ldG<HALF>(Gz, c + ALT * sj, sz), gxj = ldG<HALF>(Gx, c + ALT * sj, sx);
	const float gzi = ldG<HALF>(Gz, c + ALT * si, HS_GI(2)), gyi = ldG<HALF>(Gy, c + ALT * si, HS_GI(1));
	float fx = ldF<HALF>(P.F[0], c, HS_F(0)), fy = ldF<HALF>(P.F[1], c, HS_F(1)), fz = ldF<HALF>(P.F[2], c, HS_F(2));
	const float dx = __ldg(P.dtd[0] + (i - P.iMIN)), dy = __ldg(P.dtd[1] + (j - P.jMIN)), dz = __ldg(P.dtd[2] + (k - P.kMIN));
	if (P.C[0]) {
		float cx, cy, cz;
		if (P.matIdx) {
			const float4 t = matTriple(P, c);
			cx = t.x, cy = t.y, cz = t.z;
		} else {
			cx = __ldg(P.C[0] + c), cy = __ldg(P.C[1] + c), cz = __ldg(P.C[2] + c);
		}
		fx += (dz * (gy0 - gyk) + dy * (gzj - gz0)) * cx;
		fy += (dx * (gz0 - gzi) + dz * (gxk - gx0)) * cy;
		fz += (dy * (gx0 - gxj) + dx * (gyi - gy0)) * cz;
	} else {
		fx += (dz * (gy0 - gyk) + dy * (gzj - gz0));
		fy += (dx * (gz0 - gzi) + dz * (gxk - gx0));
		fz += (dy * (gx0 - gxj) + dx * (gyi - gy0));
	}
	storeCell<HALF>(P, i, c, fx, fy, fz);
}

// Fused half step of a large world over one tile: one thread per cell,
// TX cells of a row along k per warp, TY_ rows, one i plane.  Tiers by
// the cell's class bits: a warp whose cells have none takes the curl
// alone on a path without further tests; otherwise plain cells take the
// curl, CPML cells and cells on TFSF k face planes add their face updates,
// all inline, and cells on TFSF i or j face planes (whole blocks or
// warps) and dispersive cells go to hardCell.  Index arithmetic is 32-bit
// (at most 2^31 elements per array, checked on the host).  Worlds with
// more than 8 objects read the list of the objects that meet the block's
// tile (made on the host when the objects change, objectTiles).
template <int ALT, int TY_, bool HALF = false>
__device__ __forceinline__ void halfStepBlock(const HalfStepParams &P, int bx, int by, int plane)
{
	const int k = P.kMIN + bx * TX + threadIdx.x;
	const int j = P.jMIN + by * TY_ + threadIdx.y;
	// E sweeps i downwards, H upwards: each starts on the planes the other
	// touched last, which are still in L2
	const int i = ALT == 1 ? P.iMAX - plane : P.iMIN + plane;
	// worlds with more than 8 objects: the objects of the block's tile (a
	// block lies in one tile: TX = ALIS_TILE_K, TY_ divides ALIS_TILE_J);
	// a tile that meets none has no object cells
	const int *list = 0;
	int nIter = P.nobj;
	bool objTile = true;
	if (P.tileStart) {
		const int t = ((i - P.iMIN) * P.tjn + (by * TY_) / ALIS_TILE_J) * P.tkn + bx;
		const int s0 = __ldg(P.tileStart + t);
		list = P.tileObj + s0, nIter = __ldg(P.tileStart + t + 1) - s0, objTile = nIter > 0;
	}
	const bool inRange = k <= P.kMAX && j <= P.jMAX;
	unsigned bi = 0, bj = 0, bk = 0;
	if (inRange) bi = __ldg(P.cls[0] + (i - P.iMIN)), bj = __ldg(P.cls[1] + (j - P.jMIN)), bk = __ldg(P.cls[2] + (k - P.kMIN));
	const unsigned objm = objTile ? bi & bj & bk & 0x1FFu : 0u;
	const unsigned tf = tfsfBits(bi, bj, bk);
	const bool plain = inRange && !((bi | bj | bk) & (CLS_PML_LO | CLS_PML_HI)) && !tf && !objm;
	if (__all_sync(0xffffffffu, plain)) {
		plainCell<ALT, HALF>(P, i, j, k);
		return;
	}
	if (!inRange) return;
	if (!(tf && ((bi | bj) & CLS_TFSF)) && !objm) {
		leanCells<ALT, 1, HALF>(P, i, j, k, bi, bj, &bk);
		return;
	}
	// hard cells run the full sequence out of line (object loops: the
	// tile's list, or all objects filtered by class bits)
	hardCell<ALT, HALF>(P, i, j, k, list, nIter);
}

// planes a block of the one-world launches steps, one after the other in
// the sweep direction: each plane's i neighbours of the other field are
// the previous plane's own cells, still in L1.  Four for half storage
// (0.415 ms per pair on the 256^3 dispersive world against 0.433 with
// two, 0.444 with one and 0.433 with eight), one for float (two: 0.332
// against 0.305, from register pressure)
#define BLOCK_PLANES(HALF) ((HALF) ? 4 : 1)
template <int ALT, int TY, bool HALF = false>
__global__ void __launch_bounds__(TX * TY, STEP_MINB(TY)) k_half_step(const __grid_constant__ HalfStepParams P)
{
	if constexpr (BLOCK_PLANES(HALF) == 1) {
		halfStepBlock<ALT, TY, HALF>(P, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z);
	} else {
		const int np = P.iMAX - P.iMIN + 1;
#pragma unroll 1
		for (int q = 0; q < BLOCK_PLANES(HALF); q++) {
			const int plane = (int)blockIdx.z * BLOCK_PLANES(HALF) + q;
			if (plane < np) halfStepBlock<ALT, TY, HALF>(P, (int)blockIdx.x, (int)blockIdx.y, plane);
		}
	}
}

// sources, in list order; one block so later patches see earlier ones
// (reference src/update.c:161-179)
#define ALIS_MAXSRC 32
// source values travel in the launch parameters up to this count, beyond
// it through the world's device buffer (large launch parameters cost every
// launch host and device time)
#define ALIS_MAXSRCV 256
struct SourceParams {
	int n;
	Layout L;
	float *F[2][3];
	alisgpu_source_patch p[ALIS_MAXSRC];
	const float *vdev;                       // values beyond the inline buffer
	unsigned int *err;
	const signed char *ex;                   // half storage: the step's exponents (else null)
	float v[ALIS_MAXSRCV];
};

// the patches of one world by one block; vals: the values (null: those of P)
__device__ __forceinline__ void sourcesBlock(const SourceParams &P, const float *vals)
{
	for (int q = 0; q < P.n; q++) {
		const alisgpu_source_patch &s = P.p[q];
		int nk = 1 + s.k1 - s.k0, nj = 1 + s.j1 - s.j0, ni = 1 + s.i1 - s.i0;
		int cells = ni * nj * nk;
		float *F = P.F[s.m][s.comp];
		for (int t = threadIdx.x; t < cells; t += blockDim.x) {
			int kk = t % nk, jj = (t / nk) % nj, ii = t / (nk * nj);
			float v = vals ? vals[s.voff + t] : P.vdev ? P.vdev[s.voff + t] : P.v[s.voff + t];
			int i = s.i0 + ii, j = s.j0 + jj, k = s.k0 + kk;
			if (i < P.L.i0 || i >= P.L.i0 + P.L.ni || j < P.L.j0 || j >= P.L.j0 + P.L.nj || k < P.L.k0 || k >= P.L.k0 + P.L.nk) {
				atomicOr(P.err, 4u);
				continue;
			}
			const long long at = P.L.at(i, j, k);
			if (P.ex) {
				// a half world: the sum of the stored value and v, rounded with the plane's exponent
				const int e = P.ex[s.comp * P.L.ni + (i - P.L.i0)];
				((unsigned short *)F)[at] = halfOf(halfAt(F, at, pow2f(e)) + v, pow2f(-e));
			} else {
				F[at] += v;
			}
		}
		__syncthreads();
	}
}

__global__ void k_sources(const SourceParams P)
{
	sourcesBlock(P, 0);
}

// one group of independent ghost copies (reference src/update.c:182-191)
#define ALIS_GHOST_GROUP 4
struct GhostParams {
	int n;
	Layout L;
	float *F[2][3];
	int complexField;
	alisgpu_ghost_copy c[ALIS_GHOST_GROUP];
	int start[ALIS_GHOST_GROUP + 1];         // below 2^31 (checked on the host)
	unsigned int *err;
};

// one cell of ghost copy g: F = cos F' + sin G', G = cos G' - sin F'
// (G the imaginary set of a complex field), F = cos F' otherwise
__device__ __forceinline__ void ghostCell(const Layout &L, float *const F2[2][3], int complexField, const alisgpu_ghost_copy &g,
                                          int r, unsigned int *err)
{
	const int nk = 1 + g.k1 - g.k0, nj = 1 + g.j1 - g.j0;
	const int kk = r % nk, jj = (r / nk) % nj, ii = r / (nk * nj);
	const int i = g.i0 + ii, j = g.j0 + jj, k = g.k0 + kk;
	const int si = i + g.di, sj = j + g.dj, sk = k + g.dk;
	if (i < L.i0 || i >= L.i0 + L.ni || j < L.j0 || j >= L.j0 + L.nj || k < L.k0 || k >= L.k0 + L.nk ||
	    si < L.i0 || si >= L.i0 + L.ni || sj < L.j0 || sj >= L.j0 + L.nj || sk < L.k0 || sk >= L.k0 + L.nk) {
		atomicOr(err, 2u);
		return;
	}
	const long long d = L.at(i, j, k), s = L.at(si, sj, sk);
	float *F = F2[0][g.comp];
	if (complexField) {
		float *G = F2[1][g.comp];
		const float f = F[s], gg = G[s];
		F[d] = g.cosk * f + g.sink * gg;
		G[d] = g.cosk * gg - g.sink * f;
	} else {
		F[d] = g.cosk * F[s];
	}
}

__global__ void k_ghost(const GhostParams P)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= P.start[P.n]) return;
	int q = 0;
	while (t >= P.start[q + 1]) q++;
	ghostCell(P.L, P.F, P.complexField, P.c[q], t - P.start[q], P.err);
}

// All ghost copies of a half step in one cooperative launch: the host
// sorts the copies into dependency levels (a copy follows every earlier
// copy of the same component whose boxes it reads after, writes after or
// overwrites); copies of one level are independent and run together, and
// a grid-wide barrier separates the levels.  The driver guarantees that
// all blocks of a cooperative launch are resident, so the barrier ends.
#define ALIS_GHOST_MAX 48
#define ALIS_GHOST_NEAR 6
#define ALIS_GHOST_RED 16
struct GhostLevels {
	Layout L;
	float *F[2][3];
	int complexField;
	int n, nlev;
	alisgpu_ghost_copy c[ALIS_GHOST_MAX];     // in level order
	int start[ALIS_GHOST_MAX + 1];            // first cell of each copy (below 2^31)
	int levStart[ALIS_GHOST_MAX + 1];         // first copy of each level
	unsigned int *err;
	// one-launch form: per copy the copies of its component that can matter
	// to its cells -- later copies whose boxes meet its write box, earlier
	// copies whose boxes meet its read box (ALIS_GHOST_NEAR at most, else
	// -1: test every copy)
	signed char nLater[ALIS_GHOST_MAX], nEarlier[ALIS_GHOST_MAX];
	unsigned char later[ALIS_GHOST_MAX][ALIS_GHOST_NEAR], earlier[ALIS_GHOST_MAX][ALIS_GHOST_NEAR];
	// half storage: the exponents of the step as computed and as read, the
	// scales as read, and the (component, plane) whose read exponent the
	// copies take from another plane's computed one
	const signed char *exK;
	signed char *ex;
	float *sc;
	int nred;
	short red[ALIS_GHOST_RED][3];
};

__global__ void __launch_bounds__(256) k_ghost_levels(const __grid_constant__ GhostLevels P)
{
	cg::grid_group grid = cg::this_grid();
	const int stride = gridDim.x * blockDim.x;
	for (int l = 0; l < P.nlev; l++) {
		const int q0 = P.levStart[l], q1 = P.levStart[l + 1];
		for (int t = P.start[q0] + blockIdx.x * blockDim.x + threadIdx.x; t < P.start[q1]; t += stride) {
			int q = q0;
			while (t >= P.start[q + 1]) q++;
			ghostCell(P.L, P.F, P.complexField, P.c[q], t - P.start[q], P.err);
		}
		if (l + 1 < P.nlev) grid.sync();
	}
}

// All ghost copies of a half step in one plain launch.  The value a copy
// leaves in a cell comes down a short chain: the copy reads a cell that an
// earlier copy of the component wrote, that copy read another, and so on
// back to a root cell that no earlier copy wrote.  One thread per cell
// that keeps its value (no later copy of the component writes it) walks
// its chain back to the root and applies the copies forward, in the
// reference's order with the reference's arithmetic -- the bytes the
// sequential copies leave.  The list qualifies when no root is a cell that
// any copy writes (then no thread reads what another writes) and no chain
// is deeper than ALIS_GHOST_CHAIN; the CHECK instance tests that once per
// list, otherwise the list keeps the level-ordered cooperative launch.
#define ALIS_GHOST_CHAIN 8

__device__ __forceinline__ bool inCopy(const alisgpu_ghost_copy &c, int i, int j, int k)
{
	return c.i0 <= i && i <= c.i1 && c.j0 <= j && j <= c.j1 && c.k0 <= k && k <= c.k1;
}

template <bool CHECK, bool HALF = false>
__device__ __forceinline__ void ghostChainCell(const GhostLevels &P, int t, unsigned int *flag)
{
	if (HALF && t < P.nred) {
		const int ni = P.L.ni;
		const int e = P.exK[P.red[t][0] * ni + P.red[t][2]];
		P.ex[P.red[t][0] * ni + P.red[t][1]] = (signed char)e;
		P.sc[P.red[t][0] * ni + P.red[t][1]] = pow2f(e);
	}
	if (t >= P.start[P.n]) return;
	int q = 0;
	while (t >= P.start[q + 1]) q++;
	const alisgpu_ghost_copy &g = P.c[q];
	const int r = t - P.start[q];
	const int nk = 1 + g.k1 - g.k0, nj = 1 + g.j1 - g.j0;
	const int i = g.i0 + r / (nk * nj), j = g.j0 + (r / nk) % nj, k = g.k0 + r % nk;
	// kept by a later copy?  (the candidates are in increasing order)
	if (P.nLater[q] < 0) {
		for (int p = q + 1; p < P.n; p++) if (P.c[p].comp == g.comp && inCopy(P.c[p], i, j, k)) return;
	} else {
		for (int n = 0; n < P.nLater[q]; n++) if (inCopy(P.c[P.later[q][n]], i, j, k)) return;
	}
	const Layout &L = P.L;
	int chain[ALIS_GHOST_CHAIN], depth = 0, cur = q, ci = i, cj = j, ck = k;
	for (;;) {
		if (depth == ALIS_GHOST_CHAIN) {
			atomicOr(CHECK ? flag : P.err, CHECK ? 1u : 2u);
			return;
		}
		chain[depth++] = cur;
		const alisgpu_ghost_copy &c = P.c[cur];
		ci += c.di, cj += c.dj, ck += c.dk;
		// the last earlier copy that wrote the cell read (candidates in decreasing order)
		int prev = -1;
		if (P.nEarlier[cur] < 0) {
			for (int p = cur - 1; p >= 0; p--) if (P.c[p].comp == g.comp && inCopy(P.c[p], ci, cj, ck)) { prev = p; break; }
		} else {
			for (int n = 0; n < P.nEarlier[cur]; n++) if (inCopy(P.c[P.earlier[cur][n]], ci, cj, ck)) { prev = P.earlier[cur][n]; break; }
		}
		if (prev < 0) break;
		cur = prev;
	}
	if (i < L.i0 || i >= L.i0 + L.ni || j < L.j0 || j >= L.j0 + L.nj || k < L.k0 || k >= L.k0 + L.nk ||
	    ci < L.i0 || ci >= L.i0 + L.ni || cj < L.j0 || cj >= L.j0 + L.nj || ck < L.k0 || ck >= L.k0 + L.nk) {
		atomicOr(P.err, 2u);
		return;
	}
	if (CHECK) {
		for (int p = 0; p < P.n; p++) if (P.c[p].comp == g.comp && inCopy(P.c[p], ci, cj, ck)) { atomicOr(flag, 2u); return; }
		return;
	}
	const long long s = L.at(ci, cj, ck), d = L.at(i, j, k);
	float *F = P.F[0][g.comp];
	if (HALF) {
		// real fields: the root's value times the chain's factors (+-1, 0:
		// exact), stored with the exponent of the root's plane -- the plane
		// the destination plane reads its exponent from after the copies
		const int e = P.exK[g.comp * L.ni + (ci - L.i0)];
		float f = halfAt(F, s, pow2f(e));
		for (int l = depth - 1; l >= 0; l--) f = P.c[chain[l]].cosk * f;
		((unsigned short *)F)[d] = halfOf(f, pow2f(-e));
		return;
	}
	if (P.complexField) {
		float *G = P.F[1][g.comp];
		float f = F[s], gg = G[s];
		for (int l = depth - 1; l >= 0; l--) {
			const alisgpu_ghost_copy &c = P.c[chain[l]];
			const float nf = c.cosk * f + c.sink * gg, ng = c.cosk * gg - c.sink * f;
			f = nf, gg = ng;
		}
		F[d] = f, G[d] = gg;
	} else {
		float f = F[s];
		for (int l = depth - 1; l >= 0; l--) f = P.c[chain[l]].cosk * f;
		F[d] = f;
	}
}

template <bool CHECK, bool HALF = false>
__global__ void __launch_bounds__(256) k_ghost_chain(const __grid_constant__ GhostLevels P, unsigned int *flag)
{
	ghostChainCell<CHECK, HALF>(P, blockIdx.x * blockDim.x + threadIdx.x, flag);
}

// Small worlds (the TFSF auxiliary columns, tiny test worlds): the whole
// half step -- every cell of every m, then the source patches in list
// order, then the ghost copies one after another -- in one block, with a
// barrier between the dependent phases.  Same per-cell code as the large
// path; one launch instead of one per phase and ghost group.  The block
// is small so that it finds room beside a running large-world kernel.
#define ALIS_SMALL_CELLS 65536
// a world stepped on its own takes one block only up to this size: one
// block is one SM, so larger worlds run faster as a grid even with the
// extra source and ghost launches
#define ALIS_TINY_CELLS 4096
#define ALIS_SMALL_GHOSTS 48
struct SmallStepParams {
	HalfStepParams P[2];                      // per m
	int nm;                                   // 1 + complexField
	int nsrc, nghost;
	float *F[2][3];                           // the stepped field per m (m clamped)
	alisgpu_source_patch src[ALIS_MAXSRC];
	alisgpu_ghost_copy ghost[ALIS_SMALL_GHOSTS];
	const float *vdev;                        // values beyond the inline buffer
	float v[ALIS_MAXSRCV];
};

#define SMALL_THREADS 128
// the whole half step of a small world by the threads tid = 0..nth-1 of one block
template <int ALT>
__device__ __noinline__ void smallStepBlock(const SmallStepParams &S, int tid, int nth, const float *vals = 0)
{
	const Layout &L = S.P[0].L;
	for (int m = 0; m < S.nm; m++) {
		const HalfStepParams &P = S.P[m];
		const int nk = P.kMAX - P.kMIN + 1, nj = P.jMAX - P.jMIN + 1, ni = P.iMAX - P.iMIN + 1;
		const int cells = ni * nj * nk;
		for (int t = tid; t < cells; t += nth)
			stepCell<ALT>(P, P.iMIN + t / (nk * nj), P.jMIN + (t / nk) % nj, P.kMIN + t % nk, 0, P.nobj);
	}
	__syncthreads();
	// sources (reference src/update.c:161-179), later patches see earlier ones
	for (int q = 0; q < S.nsrc; q++) {
		const alisgpu_source_patch &p = S.src[q];
		const int nk = 1 + p.k1 - p.k0, nj = 1 + p.j1 - p.j0, ni = 1 + p.i1 - p.i0;
		float *F = S.F[p.m][p.comp];
		for (int t = tid; t < ni * nj * nk; t += nth) {
			const int i = p.i0 + t / (nk * nj), j = p.j0 + (t / nk) % nj, k = p.k0 + t % nk;
			if (i < L.i0 || i >= L.i0 + L.ni || j < L.j0 || j >= L.j0 + L.nj || k < L.k0 || k >= L.k0 + L.nk) {
				atomicOr(S.P[0].err, 4u);
				continue;
			}
			F[L.at(i, j, k)] += vals ? vals[p.voff + t] : S.vdev ? S.vdev[p.voff + t] : S.v[p.voff + t];
		}
		__syncthreads();
	}
	// ghost copies in list order (reference src/update.c:182-191)
	for (int q = 0; q < S.nghost; q++) {
		const alisgpu_ghost_copy &g = S.ghost[q];
		const int nk = 1 + g.k1 - g.k0, nj = 1 + g.j1 - g.j0, ni = 1 + g.i1 - g.i0;
		const int cells = (ni > 0 && nj > 0 && nk > 0) ? ni * nj * nk : 0;
		for (int t = tid; t < cells; t += nth) {
			const int i = g.i0 + t / (nk * nj), j = g.j0 + (t / nk) % nj, k = g.k0 + t % nk;
			const int si = i + g.di, sj = j + g.dj, sk = k + g.dk;
			if (i < L.i0 || i >= L.i0 + L.ni || j < L.j0 || j >= L.j0 + L.nj || k < L.k0 || k >= L.k0 + L.nk ||
			    si < L.i0 || si >= L.i0 + L.ni || sj < L.j0 || sj >= L.j0 + L.nj || sk < L.k0 || sk >= L.k0 + L.nk) {
				atomicOr(S.P[0].err, 2u);
				continue;
			}
			const long long d = L.at(i, j, k), src = L.at(si, sj, sk);
			float *F = S.F[0][g.comp];
			if (S.nm > 1) {
				float *G = S.F[1][g.comp];
				const float f = F[src], gg = G[src];
				F[d] = g.cosk * f + g.sink * gg;
				G[d] = g.cosk * gg - g.sink * f;
			} else {
				F[d] = g.cosk * F[src];
			}
		}
		__syncthreads();
	}
}

static void freeStaged(alisgpu_world *w)
{
	for (int f = 0; f < 2; f++) delete w->staged[f], w->staged[f] = 0;
}

// an auxiliary step handed over for a launch that did not take it runs on its own
template <int ALT> __global__ void k_small_step(const __grid_constant__ SmallStepParams S);
static int recordStaged(alisgpu_world *aux, int field);
static bool batchRecording(void);
static int runStagedAux(const alisgpu_half_step *s, int field)
{
	alisgpu_world *aux = s->ntfsf == 1 ? s->tfsf[0].aux : 0;
	if (!aux || !aux->stagedValid[field]) return ALISGPU_OK;
	if (batchRecording() && !aux->group) return recordStaged(aux, field);
	aux->stagedValid[field] = false;
	if (field == 0) k_small_step<1><<<1, SMALL_THREADS, 0, gStream>>>(*aux->staged[field]);
	else k_small_step<-1><<<1, SMALL_THREADS, 0, gStream>>>(*aux->staged[field]);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	return ALISGPU_OK;
}

template <int ALT>
__global__ void __launch_bounds__(SMALL_THREADS) k_small_step(const __grid_constant__ SmallStepParams S)
{
	smallStepBlock<ALT>(S, threadIdx.x, blockDim.x);
}

// A large world's half step with its TFSF auxiliary column in the same
// launch: the first plane of blocks is the column's (one block of
// TX x TY = SMALL_THREADS threads runs it, the rest return), the planes
// after it are the world's.  The column's step of this field reads and
// writes only the column, and the world's step reads the column's other
// field, so the two are independent within the launch; the launch order
// gives the reference's order across fields.
struct FusedStepParams {
	HalfStepParams P;
	SmallStepParams aux;
};

template <int ALT, int TY, bool HALF = false>
__global__ void __launch_bounds__(TX * TY, STEP_MINB(TY)) k_half_step_aux(const __grid_constant__ FusedStepParams F)
{
	if (blockIdx.z == 0) {
		if (blockIdx.x == 0 && blockIdx.y == 0) smallStepBlock<ALT>(F.aux, threadIdx.y * blockDim.x + threadIdx.x, blockDim.x * blockDim.y);
		return;
	}
	if constexpr (BLOCK_PLANES(HALF) == 1) {
		halfStepBlock<ALT, TY, HALF>(F.P, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z - 1);
	} else {
		const int np = F.P.iMAX - F.P.iMIN + 1;
#pragma unroll 1
		for (int q = 0; q < BLOCK_PLANES(HALF); q++) {
			const int plane = ((int)blockIdx.z - 1) * BLOCK_PLANES(HALF) + q;
			if (plane < np) halfStepBlock<ALT, TY, HALF>(F.P, (int)blockIdx.x, (int)blockIdx.y, plane);
		}
	}
}

// one half-step launch with block height kTyChoice[v] (v a runtime choice)
template <int ALT, bool HALF>
static void launchHalfStepAs(int ty, dim3 g, dim3 block, const HalfStepParams &P, const FusedStepParams *F, cudaStream_t st)
{
#define ALIS_LAUNCH(TY) do { if (F) k_half_step_aux<ALT, TY, HALF><<<g, block, 0, st>>>(*F); else k_half_step<ALT, TY, HALF><<<g, block, 0, st>>>(P); } while (0)
	if (ty == 2) ALIS_LAUNCH(2);
	else if (ty == 8) ALIS_LAUNCH(8);
	else ALIS_LAUNCH(4);
#undef ALIS_LAUNCH
}
template <int ALT>
static void launchHalfStep(int v, dim3 grid, const HalfStepParams &P, const FusedStepParams *F, cudaStream_t st, bool half = false)
{
	const int ty = kTyChoice[v];
	dim3 block(TX, ty, 1);
	dim3 g(grid.x, grid.y, grid.z + (F ? 1 : 0));
	if (half) launchHalfStepAs<ALT, true>(ty, g, block, P, F, st);
	else launchHalfStepAs<ALT, false>(ty, g, block, P, F, st);
}

// ---------------------------------------------------------------------
// Batched launches over many worlds (batch.cuh)
// ---------------------------------------------------------------------
// the tiles of a batched entry: nbx x nby tiles of 32 x BATCH_TY cells
// per i plane, planes in the half step's sweep order (2, 4 or 8; 4 unless
// the build defines it)
#ifndef BATCH_TY
#define BATCH_TY 4
#endif
static_assert(BATCH_TY == 2 || BATCH_TY == 4 || BATCH_TY == 8, "BATCH_TY divides the object tiles' 8 rows");
// n / d for 0 <= n < 2^31 as (n m) >> sh, with m = ceil(2^sh / d) and
// sh = 31 + ceil(log2 d): the product's error stays below 1/d for every
// such n (checked exhaustively over the divisors a launch uses)
struct FastDiv {
	unsigned m;
	int sh;
	__device__ __forceinline__ int div(int n) const { return (int)(((unsigned long long)(unsigned)n * m) >> sh); }
};
static FastDiv fastDiv(int d)
{
	int s = 0;
	while ((1LL << s) < d) s++;
	FastDiv f;
	f.sh = 31 + s;
	f.m = (unsigned)(((1ULL << f.sh) + (unsigned long long)d - 1) / (unsigned long long)d);
	return f;
}

struct BatchEntry {                    // the cells of one world (one m) in a batched launch
	int nbx, nby, planes;
	int itemStart;                     // its first tile in the launch
	FastDiv byRow, byPlane;            // division by nbx and by nbx nby
};
struct BatchBlock {                    // a half step run by one block (auxiliary column, tiny world)
	const SmallStepParams *S;          // its device slot
	int voff;                          // its source values in the group's values, or -1
};
struct BatchSource {                   // the source patches of one world
	const SourceParams *S;
	int voff;
};
struct BatchGhost {                    // the ghost copies of one world
	const GhostLevels *G;
	int start;                         // its first thread in the launch
};
// The launch parameters of a batched half step: the worlds' parameters
// travel in the kernel's parameter space, as those of a one-world launch
// do, so the cell code reads them through the constant cache.  Launches
// come in capacities of 1, 4, 8 and 16 entries, so that a launch carries
// about as many parameter bytes as it has worlds.
#define BATCH_WORLDS 16
struct BatchHead {
	int nE, nitems;                    // entries, tiles
	int nblk;                          // one-block steps: the first nblk blocks
	const BatchBlock *blk;
	const float *vals;
};
template <int CAP>
struct BatchStep {
	BatchHead h;
	BatchEntry E[CAP];
	HalfStepParams P[CAP];
};
static_assert(sizeof(BatchStep<BATCH_WORLDS>) <= 32000, "batched launch parameters exceed the parameter space");

// One launch over the worlds of a group: the first blocks run the
// one-block steps, each further block one tile of the concatenated
// worlds, in the order of a one-world launch (k tiles, then rows, then
// planes in the sweep direction), so the blocks resident at any time work
// on neighbouring tiles and planes.  A block finds its world from its
// index alone, and runs halfStepBlock, the code of the one-world launch,
// with the world's parameters from the launch's.
template <int ALT, int CAP>
__global__ void __launch_bounds__(TX * BATCH_TY, STEP_MINB(BATCH_TY)) k_step_batch(const __grid_constant__ BatchStep<CAP> B)
{
	if ((int)blockIdx.x < B.h.nblk) {
		const BatchBlock &b = B.h.blk[blockIdx.x];
		smallStepBlock<ALT>(*b.S, threadIdx.y * blockDim.x + threadIdx.x, blockDim.x * blockDim.y, b.voff >= 0 ? B.h.vals + b.voff : 0);
		return;
	}
	const int g = (int)blockIdx.x - B.h.nblk;
	int e = 0;
#pragma unroll
	for (int q = 1; q < CAP; q++) if (q < B.h.nE && B.E[q].itemStart <= g) e = q;
	const BatchEntry &E = B.E[e];
	const int t = g - E.itemStart, plane = E.byPlane.div(t), r = t - plane * E.nbx * E.nby, by = E.byRow.div(r);
	halfStepBlock<ALT, BATCH_TY>(B.P[e], r - by * E.nbx, by, plane);
}

__global__ void k_sources_batch(const BatchSource *T, const float *vals)
{
	const BatchSource &b = T[blockIdx.x];
	sourcesBlock(*b.S, b.voff >= 0 ? vals + b.voff : 0);
}

__global__ void __launch_bounds__(256) k_ghost_batch(const BatchGhost *T, int n, int total)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= total) return;
	int lo = 0, hi = n - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (T[mid].start <= t) lo = mid; else hi = mid - 1;
	}
	ghostChainCell<false>(*T[lo].G, t - T[lo].start, 0);
}

// the group a host thread is recording
struct SlotUpdate {
	void *dst;
	size_t off, bytes;                 // in the staged update bytes
};
struct Recorder {
	bool on = false;
	StreamGroup *group = nullptr;              // the thread's batch streams
	cudaEvent_t evBegin = nullptr, evEnd = nullptr;
	int kind = BATCH_NONE;
	unsigned long long stamp = 1;
	std::vector<BatchEntry> entries;
	std::vector<HalfStepParams> params;        // the entries' parameters
	std::vector<BatchBlock> blocks;
	std::vector<BatchSource> sources;
	std::vector<BatchGhost> ghosts;
	int nitems = 0, ghostTotal = 0;
	std::vector<float> values;
	std::vector<unsigned char> updates;        // new bytes of changed slots
	std::vector<SlotUpdate> updateList;
	void clear() {
		kind = BATCH_NONE;
		stamp++;
		entries.clear(), params.clear(), blocks.clear(), sources.clear(), ghosts.clear();
		nitems = 0, ghostTotal = 0;
		values.clear(), updates.clear(), updateList.clear();
	}
};
static thread_local Recorder gRec;
static bool batchRecording(void) { return gRec.on; }

// the staging blob: pinned host and device buffers in turn, each reused
// once the launches that read its last contents have finished
#define BLOB_RING 4
struct Blob {
	unsigned char *pin[BLOB_RING] = {};
	unsigned char *dev[BLOB_RING] = {};
	size_t cap[BLOB_RING] = {};
	cudaEvent_t done[BLOB_RING] = {};
	bool pending[BLOB_RING] = {};
	int cur = 0;
	size_t bytes = 0;
	bool open = false;
};
static thread_local Blob gBlob;

extern "C" int alisgpu__blob_take(size_t bytes, void **host, const void **dev)
{
	Blob &b = gBlob;
	if (b.open) return alisgpu__fail(ALISGPU_EINVAL, "batch: blob taken twice");
	const int q = b.cur;
	if (b.pending[q]) {
		ALIS_CUDA(cudaEventSynchronize(b.done[q]));
		b.pending[q] = false;
	}
	if (!b.done[q]) ALIS_CUDA(cudaEventCreateWithFlags(&b.done[q], cudaEventDisableTiming));
	if (bytes > b.cap[q]) {
		if (b.pin[q]) cudaFreeHost(b.pin[q]), b.pin[q] = 0;
		if (b.dev[q]) alisgpu__freeAsync(b.dev[q]), b.dev[q] = 0;
		b.cap[q] = 0;
		const size_t cap = std::max(bytes + bytes / 2, (size_t)1 << 16);
		ALIS_CUDA(cudaMallocHost(&b.pin[q], cap));
		ALIS_CUDA(alisgpu__mallocAsync(&b.dev[q], cap));
		b.cap[q] = cap;
	}
	b.bytes = bytes, b.open = true;
	*host = b.pin[q], *dev = b.dev[q];
	return ALISGPU_OK;
}

extern "C" int alisgpu__blob_send(void)
{
	Blob &b = gBlob;
	if (!b.open) return alisgpu__fail(ALISGPU_EINVAL, "batch: no blob taken");
	if (b.bytes) ALIS_CUDA(cudaMemcpyAsync(b.dev[b.cur], b.pin[b.cur], b.bytes, cudaMemcpyHostToDevice, gStream));
	return ALISGPU_OK;
}

// the launches reading the blob are issued: the next group takes the next buffer
extern "C" int alisgpu__blob_done(void)
{
	Blob &b = gBlob;
	if (!b.open) return ALISGPU_OK;
	ALIS_CUDA(cudaEventRecord(b.done[b.cur], gStream));
	b.pending[b.cur] = true;
	b.open = false;
	b.cur = (b.cur + 1) % BLOB_RING;
	return ALISGPU_OK;
}

extern "C" int alisgpu__slot_sync(ParamSlot *s, const void *src, size_t bytes, const void **dev)
{
	if (!s->dev || s->host.size() != bytes) {
		if (s->dev) alisgpu__freeAsync(s->dev), s->dev = nullptr;
		s->host.clear();
		ALIS_CUDA(alisgpu__mallocAsync((unsigned char **)&s->dev, bytes));
	}
	if (s->host.size() != bytes || memcmp(s->host.data(), src, bytes)) {
		s->host.assign((const unsigned char *)src, (const unsigned char *)src + bytes);
		// uploaded with the group, before its launches
		const size_t off = (gRec.updates.size() + 255) & ~(size_t)255;
		gRec.updates.resize(off + bytes);
		memcpy(gRec.updates.data() + off, src, bytes);
		gRec.updateList.push_back(SlotUpdate{ s->dev, off, bytes });
	}
	*dev = s->dev;
	return ALISGPU_OK;
}

extern "C" void alisgpu__slot_free(ParamSlot *s)
{
	if (s->dev) alisgpu__freeAsync(s->dev);
	s->dev = nullptr;
	s->host.clear();
}

template <int ALT, int CAP>
static int launchStepBatch(const BatchHead &h, const std::vector<BatchEntry> &E, const std::vector<HalfStepParams> &P, cudaStream_t st)
{
	static thread_local BatchStep<CAP> B;
	B.h = h;
	for (int q = 0; q < h.nE; q++) B.E[q] = E[q], B.P[q] = P[q];
	const unsigned blocks = (unsigned)h.nblk + (unsigned)h.nitems;
	if (blocks) k_step_batch<ALT, CAP><<<blocks, dim3(TX, BATCH_TY), 0, st>>>(B);
	return ALISGPU_OK;
}

template <int ALT>
static int launchStepBatch(const BatchHead &h, const std::vector<BatchEntry> &E, const std::vector<HalfStepParams> &P, cudaStream_t st)
{
	if (h.nE <= 1) return launchStepBatch<ALT, 1>(h, E, P, st);
	if (h.nE <= 4) return launchStepBatch<ALT, 4>(h, E, P, st);
	if (h.nE <= 8) return launchStepBatch<ALT, 8>(h, E, P, st);
	return launchStepBatch<ALT, BATCH_WORLDS>(h, E, P, st);
}

// launch the open half-step group: its tables and the changed slots go up
// in one copy, then the cells, the sources and the ghost copies of every
// world, each one launch
static int launchHalfGroup(int field)
{
	Recorder &R = gRec;
	auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
	const size_t oB = 0;
	const size_t oS = oB + al(R.blocks.size() * sizeof(BatchBlock));
	const size_t oG = oS + al(R.sources.size() * sizeof(BatchSource));
	const size_t oV = oG + al(R.ghosts.size() * sizeof(BatchGhost));
	const size_t oU = oV + al(R.values.size() * sizeof(float));
	const size_t total = oU + R.updates.size();
	void *hv = 0;
	const void *dv = 0;
	int rc = alisgpu__blob_take(total, &hv, &dv);
	if (rc) return rc;
	unsigned char *h = (unsigned char *)hv;
	const unsigned char *d = (const unsigned char *)dv;
	if (!R.blocks.empty()) memcpy(h + oB, R.blocks.data(), R.blocks.size() * sizeof(BatchBlock));
	if (!R.sources.empty()) memcpy(h + oS, R.sources.data(), R.sources.size() * sizeof(BatchSource));
	if (!R.ghosts.empty()) memcpy(h + oG, R.ghosts.data(), R.ghosts.size() * sizeof(BatchGhost));
	if (!R.values.empty()) memcpy(h + oV, R.values.data(), R.values.size() * sizeof(float));
	if (!R.updates.empty()) memcpy(h + oU, R.updates.data(), R.updates.size());
	if ((rc = alisgpu__blob_send())) return rc;
	for (const SlotUpdate &u : R.updateList)
		ALIS_CUDA(cudaMemcpyAsync(u.dst, d + oU + u.off, u.bytes, cudaMemcpyDeviceToDevice, gStream));
	const float *vals = (const float *)(d + oV);
	if (!R.entries.empty() || !R.blocks.empty()) {
		BatchHead h;
		h.nE = (int)R.entries.size(), h.nitems = R.nitems;
		h.blk = (const BatchBlock *)(d + oB), h.nblk = (int)R.blocks.size();
		h.vals = vals;
		int slot = alisgpu__prof_start();
		rc = field == 0 ? launchStepBatch<1>(h, R.entries, R.params, gStream) : launchStepBatch<-1>(h, R.entries, R.params, gStream);
		alisgpu__prof_stop(slot, field == 0 ? ALISGPU_K_STEP_E : ALISGPU_K_STEP_H);
		alisgpu__count_launch();
		if (rc) return rc;
		ALIS_CUDA(cudaGetLastError());
	}
	if (!R.sources.empty()) {
		int slot = alisgpu__prof_start();
		k_sources_batch<<<(unsigned)R.sources.size(), 256, 0, gStream>>>((const BatchSource *)(d + oS), vals);
		alisgpu__prof_stop(slot, ALISGPU_K_SOURCE);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}
	if (!R.ghosts.empty() && R.ghostTotal) {
		int slot = alisgpu__prof_start();
		k_ghost_batch<<<(unsigned)((R.ghostTotal + 255) / 256), 256, 0, gStream>>>((const BatchGhost *)(d + oG),
		                                                                        (int)R.ghosts.size(), R.ghostTotal);
		alisgpu__prof_stop(slot, ALISGPU_K_GHOST);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}
	return alisgpu__blob_done();
}

// launch the open group, whatever its kind
// launch the open group, whatever its kind, on the thread's batch streams
static int batchLaunch(void)
{
	Recorder &R = gRec;
	StreamGroup *prev = gGroup;
	gGroup = R.group;
	int rc = ALISGPU_OK;
	const bool updates = !R.updateList.empty();
	if (R.kind == BATCH_E || R.kind == BATCH_H) rc = launchHalfGroup(R.kind == BATCH_E ? 0 : 1);
	else if (R.kind == BATCH_PHASER) rc = alisgpu__phaser_batch_launch();
	else if (updates) rc = launchHalfGroup(0);
	R.clear();
	gGroup = prev;
	return rc;
}

// the shared streams wait for everything the batch streams were given
static int batchJoinShared(void)
{
	Recorder &R = gRec;
	ALIS_CUDA(cudaEventRecord(R.evEnd, R.group->main));
	ALIS_CUDA(cudaStreamWaitEvent(gDefaultGroup.main, R.evEnd, 0));
	return ALISGPU_OK;
}

// A recorded call runs the rest of its work (uploads of changed tables,
// launches of a group it closes) on the thread's batch streams.
extern "C" int alisgpu__batch_enter(int kind, const void *world)
{
	Recorder &R = gRec;
	if (!R.on) return 0;
	const alisgpu_world *w = (const alisgpu_world *)world;
	if (w && w->group) return 0;                      // worlds on streams of their own step as usual
	gGroup = R.group;
	if (kind == BATCH_NONE) return 1;
	if (R.kind != kind || (w && w->batchStamp == R.stamp)) {
		if (batchLaunch()) return -1;
		R.kind = kind;
	}
	if (w) const_cast<alisgpu_world *>(w)->batchStamp = R.stamp;
	return 1;
}

// Each recording thread has streams of its own, so that the groups of
// several threads overlap on the device; its batch starts after the work
// given to the shared streams so far, and that work's later calls start
// after the batch.
extern "C" int alisgpu_batch_begin(void)
{
	int rc = alisgpu_init();
	if (rc) return rc;
	Recorder &R = gRec;
	if (R.on) return alisgpu__fail(ALISGPU_EINVAL, "batch_begin: a batch is open already");
	if (!R.group) {
		StreamGroup *g = new StreamGroup();
		if ((rc = groupCreate(g))) { delete g; return rc; }
		ALIS_CUDA(cudaEventCreateWithFlags(&R.evBegin, cudaEventDisableTiming));
		ALIS_CUDA(cudaEventCreateWithFlags(&R.evEnd, cudaEventDisableTiming));
		R.group = g;
	}
	bindWorld(0);
	ALIS_CUDA(cudaEventRecord(R.evBegin, gDefaultGroup.main));
	ALIS_CUDA(cudaStreamWaitEvent(R.group->main, R.evBegin, 0));
	R.clear();
	R.on = true;
	return ALISGPU_OK;
}

extern "C" int alisgpu_batch_end(void)
{
	Recorder &R = gRec;
	if (!R.on) return ALISGPU_OK;
	int rc = batchLaunch();
	R.on = false;
	if (rc) alisgpu__phaser_batch_clear();
	const int rj = batchJoinShared();
	bindWorld(0);
	return rc ? rc : rj;
}

extern "C" int alisgpu__batch_flush(void)
{
	Recorder &R = gRec;
	if (!R.on || R.kind == BATCH_NONE) return ALISGPU_OK;
	int rc = batchLaunch();
	if (rc) return rc;
	return batchJoinShared();
}

// ---------------------------------------------------------------------
// host driver of one half step
// ---------------------------------------------------------------------
static void fillTfsf(DevTfsf &T, const alisgpu_tfsf &s, int field, const float *dtdMain[3], const alisgpu_geometry &g)
{
	T.iMin = s.iMin, T.iMax = s.iMax, T.jMin = s.jMin, T.jMax = s.jMax, T.kMin = s.kMin, T.kMax = s.kMax;
	T.iMIN = s.iMIN, T.iMAX = s.iMAX, T.jMIN = s.jMIN, T.jMAX = s.jMAX, T.kMIN = s.kMIN, T.kMAX = s.kMAX;
	T.auxIMAX = s.auxIMAX, T.auxJMAX = s.auxJMAX, T.aliasX = s.aliasX, T.aliasY = s.aliasY;
	T.L = s.aux->L;
	for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
		int mm = m <= s.aux->g.complexField ? m : 0;
		T.G[m][c] = field == 0 ? s.aux->H[mm][c] : s.aux->E[mm][c];
	}
	// dt/ds at the faces: E step uses iMin / iMax, H step iMin / iMax+1
	int lo[3] = { s.iMin, s.jMin, s.kMin };
	int hi[3] = { s.iMax + field, s.jMax + field, s.kMax + field };
	int base[3] = { g.iMIN, g.jMIN, g.kMIN };
	int top[3] = { g.iMAX, g.jMAX, g.kMAX };
	for (int a = 0; a < 3; a++) {
		float v0 = 0, v1 = 0;
		if (lo[a] >= base[a] && lo[a] <= top[a]) orderedCopy(&v0, dtdMain[a] + (lo[a] - base[a]), sizeof(float), cudaMemcpyDeviceToHost);
		if (hi[a] >= base[a] && hi[a] <= top[a]) orderedCopy(&v1, dtdMain[a] + (hi[a] - base[a]), sizeof(float), cudaMemcpyDeviceToHost);
		T.dtdMin[a] = v0, T.dtdMax[a] = v1;
	}
}

// cached dt/ds face values: the TFSF box is fixed once set up
// The device form of a world's TFSF boxes, kept per world (a world has a
// few); an epoch counter drops every world's entries when a box the host
// layer frees may have left its address for a new one.
static std::atomic<unsigned long long> gTfsfEpoch{1};

static DevTfsf tfsfFor(alisgpu_world *w, const alisgpu_tfsf &s, int field)
{
	const unsigned long long epoch = gTfsfEpoch.load();
	if (w->tfEpoch != epoch) w->tfCache.clear(), w->tfEpoch = epoch;
	for (alisgpu_world::TfsfCache &c : w->tfCache)
		if (c.key == &s && c.field == field && c.T.iMin == s.iMin && c.T.kMax == s.kMax && c.T.L.ni == s.aux->L.ni) return c.T;
	alisgpu_world::TfsfCache c;
	c.key = &s, c.field = field;
	const float *dtd[3] = { w->dtd[field][0], w->dtd[field][1], w->dtd[field][2] };
	fillTfsf(c.T, s, field, dtd, w->g);
	w->tfCache.push_back(c);
	return c.T;
}

extern "C" void alisgpu__forget_tfsf(const alisgpu_tfsf *s)
{
	(void)s;
	gTfsfEpoch++;
}

// ghost copies in list order; consecutive copies of distinct components
// share a launch (reference src/update.c:182-191)
static bool boxesMeet(const int a[6], const int b[6])
{
	return a[0] <= b[1] && b[0] <= a[1] && a[2] <= b[3] && b[2] <= a[3] && a[4] <= b[5] && b[4] <= a[5];
}

static int recordGhosts(alisgpu_world *w, int field, const GhostLevels &GL, long long total);

// The ghost copies of a half step.  With record set (a batch records the
// world's half step) the one-launch form joins the batch group; the other
// forms launch the group first and then run on their own.
// Ghost copies of a half world move values exactly: real copies by +-1 or
// 0, each stored with the exponent of the plane its chain starts in.  A
// copy between x planes takes its destination plane to the exponent of
// the plane it reads, so it must write the plane whole: every cell the
// half step updates there, and every cell an earlier copy of the component
// wrote there.  Fills the list's plane redirects; false when the list
// does not qualify.
static bool halfGhostPlan(const alisgpu_world *w, const alisgpu_ghost_copy *gl, int n, GhostLevels &GL)
{
	const Layout &L = w->L;
	const alisgpu_geometry &g = w->g;
	std::vector<int> es(3 * (size_t)L.ni);
	for (int q = 0; q < 3; q++) for (int p = 0; p < L.ni; p++) es[q * L.ni + p] = p;
	for (int c = 0; c < n; c++) {
		const alisgpu_ghost_copy &x = gl[c];
		if (x.i1 < x.i0 || x.j1 < x.j0 || x.k1 < x.k0) continue;
		if (x.comp < 0 || x.comp > 2 || !(x.cosk == 1.0f || x.cosk == -1.0f || x.cosk == 0.0f)) return false;
		if (x.di == 0) continue;
		if (x.i0 + x.di <= x.i1 && x.i1 + x.di >= x.i0) return false;
		const bool covers = x.j0 <= g.jMIN && x.j1 >= g.jMAX && x.k0 <= g.kMIN && x.k1 >= g.kMAX;
		for (int p = x.i0; p <= x.i1; p++) {
			if (p < L.i0 || p >= L.i0 + L.ni || p + x.di < L.i0 || p + x.di >= L.i0 + L.ni) return false;
			if (p >= g.iMIN && p <= g.iMAX && !covers) return false;
			for (int b = 0; b < c; b++) {
				const alisgpu_ghost_copy &y = gl[b];
				if (y.comp != x.comp || y.i1 < y.i0 || y.j1 < y.j0 || y.k1 < y.k0 || p < y.i0 || p > y.i1) continue;
				if (y.j0 < x.j0 || y.j1 > x.j1 || y.k0 < x.k0 || y.k1 > x.k1) return false;
			}
			es[x.comp * L.ni + (p - L.i0)] = es[x.comp * L.ni + (p + x.di - L.i0)];
		}
	}
	GL.nred = 0;
	for (int q = 0; q < 3; q++) for (int p = 0; p < L.ni; p++) {
		if (es[q * L.ni + p] == p) continue;
		if (GL.nred == ALIS_GHOST_RED) return false;
		GL.red[GL.nred][0] = (short)q, GL.red[GL.nred][1] = (short)p, GL.red[GL.nred][2] = (short)es[q * L.ni + p];
		GL.nred++;
	}
	return true;
}

static int runGhosts(alisgpu_world *w, int field, const alisgpu_ghost_copy *gl, int n, bool record = false)
{
	const alisgpu_geometry &g = w->g;
	if (n <= 0) return ALISGPU_OK;
	if (w->half && (record || n > ALIS_GHOST_MAX))
		return alisgpu__fail(ALISGPU_ENOTSUP, "ghost copies: %d copies of a half world", n);
	if (record && w->ghostChain[field] && w->bG[field].dev && w->ghostSeen[field].size() == (size_t)n &&
	    !memcmp(w->ghostSeen[field].data(), gl, n * sizeof *gl)) {
		// the list of the last recorded half step: its one-launch form is in the slot
		if (gRec.ghostTotal + w->ghostCells[field] >= (1ll << 31)) return alisgpu__fail(ALISGPU_ERANGE, "batch: ghost copies exceed 32-bit indexing");
		gRec.ghosts.push_back(BatchGhost{ (const GhostLevels *)w->bG[field].dev, gRec.ghostTotal });
		gRec.ghostTotal += (int)w->ghostCells[field];
		return ALISGPU_OK;
	}
	if (n <= ALIS_GHOST_MAX) {
		// dependency levels: written box W, read box R = W shifted
		int lev[ALIS_GHOST_MAX], nlev = 0;
		long long cells[ALIS_GHOST_MAX], total = 0;
		for (int q = 0; q < n; q++) {
			const alisgpu_ghost_copy &c = gl[q];
			const int Wq[6] = { c.i0, c.i1, c.j0, c.j1, c.k0, c.k1 };
			const int Rq[6] = { c.i0 + c.di, c.i1 + c.di, c.j0 + c.dj, c.j1 + c.dj, c.k0 + c.dk, c.k1 + c.dk };
			cells[q] = (c.i1 < c.i0 || c.j1 < c.j0 || c.k1 < c.k0) ? 0 : (long long)(1 + c.i1 - c.i0) * (1 + c.j1 - c.j0) * (1 + c.k1 - c.k0);
			total += cells[q];
			lev[q] = 0;
			for (int p = 0; p < q; p++) {
				const alisgpu_ghost_copy &e = gl[p];
				if (e.comp != c.comp || !cells[p] || !cells[q]) continue;
				const int Wp[6] = { e.i0, e.i1, e.j0, e.j1, e.k0, e.k1 };
				const int Rp[6] = { e.i0 + e.di, e.i1 + e.di, e.j0 + e.dj, e.j1 + e.dj, e.k0 + e.dk, e.k1 + e.dk };
				if (boxesMeet(Wp, Rq) || boxesMeet(Wp, Wq) || boxesMeet(Rp, Wq)) lev[q] = std::max(lev[q], lev[p] + 1);
			}
			nlev = std::max(nlev, lev[q] + 1);
		}
		if (total >= (1ll << 31)) return alisgpu__fail(ALISGPU_ERANGE, "ghost copies of %lld cells exceed 32-bit indexing", total);
		if (total == 0) return ALISGPU_OK;
		static thread_local GhostLevels GL;
		memset(&GL, 0, sizeof GL);
		GL.L = w->L;
		GL.err = gErrWord;
		GL.complexField = g.complexField;
		for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
			int mm = m <= g.complexField ? m : 0;
			GL.F[m][c] = field == 0 ? w->E[mm][c] : w->H[mm][c];
		}
		// the one-launch form, copies in the reference's order
		std::vector<alisgpu_ghost_copy> &seen = w->ghostSeen[field];
		const bool same = seen.size() == (size_t)n && !memcmp(seen.data(), gl, n * sizeof *gl);
		if (!same || w->ghostChain[field]) {
			int at = 0;
			for (int q = 0; q < n; q++) GL.c[q] = gl[q], GL.start[q] = at, at += (int)cells[q];
			GL.n = n, GL.start[n] = at;
			// candidate lists: copies of the component whose boxes meet the
			// write box (later) or the read box (earlier, nearest first)
			for (int q = 0; q < n; q++) {
				const alisgpu_ghost_copy &c = gl[q];
				const int Wq[6] = { c.i0, c.i1, c.j0, c.j1, c.k0, c.k1 };
				const int Rq[6] = { c.i0 + c.di, c.i1 + c.di, c.j0 + c.dj, c.j1 + c.dj, c.k0 + c.dk, c.k1 + c.dk };
				int nl = 0, ne = 0;
				for (int p = q + 1; p < n; p++) {
					const alisgpu_ghost_copy &e = gl[p];
					const int Wp[6] = { e.i0, e.i1, e.j0, e.j1, e.k0, e.k1 };
					if (e.comp != c.comp || !cells[p] || !boxesMeet(Wp, Wq)) continue;
					if (nl >= 0 && nl < ALIS_GHOST_NEAR) GL.later[q][nl++] = (unsigned char)p;
					else nl = -1;
				}
				for (int p = q - 1; p >= 0; p--) {
					const alisgpu_ghost_copy &e = gl[p];
					const int Wp[6] = { e.i0, e.i1, e.j0, e.j1, e.k0, e.k1 };
					if (e.comp != c.comp || !cells[p] || !boxesMeet(Wp, Rq)) continue;
					if (ne >= 0 && ne < ALIS_GHOST_NEAR) GL.earlier[q][ne++] = (unsigned char)p;
					else ne = -1;
				}
				GL.nLater[q] = (signed char)nl, GL.nEarlier[q] = (signed char)ne;
			}
			const unsigned blocks = (unsigned)((total + 255) / 256);
			if (!same) {
				seen.assign(gl, gl + n);
				unsigned int *flag = 0, h = 0;
				ALIS_CUDA(alisgpu__mallocAsync(&flag, sizeof h));
				ALIS_CUDA(cudaMemsetAsync(flag, 0, sizeof h, gStream));
				k_ghost_chain<true><<<blocks, 256, 0, gStream>>>(GL, flag);
				alisgpu__count_launch();
				ALIS_CUDA(cudaGetLastError());
				ALIS_CUDA(cudaMemcpyAsync(&h, flag, sizeof h, cudaMemcpyDeviceToHost, gStream));
				ALIS_CUDA(cudaStreamSynchronize(gStream));
				alisgpu__freeAsync(flag);
				w->ghostChain[field] = h == 0;
			}
			if (w->ghostChain[field] && record) return recordGhosts(w, field, GL, total);
			if (w->ghostChain[field] && w->half) {
				if (!halfGhostPlan(w, gl, n, GL))
					return alisgpu__fail(ALISGPU_ENOTSUP, "ghost copies: the list does not move whole planes of a half world");
				const int cur = (int)((w->nHalf[field] + 1) & 1);
				GL.exK = w->exK[field][cur], GL.ex = w->ex[field][cur], GL.sc = w->sc[field][cur];
				// the redirected scales are read by both fields' next steps
				if (GL.nred) w->tabFresh[0] = w->tabFresh[1] = false;
				const unsigned hb = (unsigned)((std::max<long long>(total, GL.nred) + 255) / 256);
				int slot = alisgpu__prof_start();
				k_ghost_chain<false, true><<<hb, 256, 0, gStream>>>(GL, nullptr);
				alisgpu__prof_stop(slot, ALISGPU_K_GHOST);
				alisgpu__count_launch();
				ALIS_CUDA(cudaGetLastError());
				return ALISGPU_OK;
			}
			if (w->ghostChain[field]) {
				int slot = alisgpu__prof_start();
				k_ghost_chain<false><<<blocks, 256, 0, gStream>>>(GL, nullptr);
				alisgpu__prof_stop(slot, ALISGPU_K_GHOST);
				alisgpu__count_launch();
				ALIS_CUDA(cudaGetLastError());
				return ALISGPU_OK;
			}
			memset(GL.c, 0, sizeof GL.c);
			memset(GL.start, 0, sizeof GL.start);
			GL.n = 0;
		}
		if (w->half) return alisgpu__fail(ALISGPU_ENOTSUP, "ghost copies: chains that a half world cannot run in one launch");
		if (record) {
			int rc = alisgpu__batch_flush();
			if (rc) return rc;
		}
		int at = 0;
		for (int l = 0; l < nlev; l++) {
			GL.levStart[l] = GL.n;
			for (int q = 0; q < n; q++) if (lev[q] == l) {
				GL.c[GL.n] = gl[q];
				GL.start[GL.n] = at;
				at += (int)cells[q];
				GL.n++;
			}
		}
		GL.levStart[nlev] = GL.n;
		GL.start[GL.n] = at;
		GL.nlev = nlev;
		// resident blocks of the cooperative launch, computed once (host
		// threads stepping several worlds may get here together)
		static std::atomic<int> blocksMaxAt{0};
		int blocksMax = blocksMaxAt.load();
		if (!blocksMax) {
			int dev = 0, sms = 0, per = 0;
			ALIS_CUDA(cudaGetDevice(&dev));
			ALIS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
			ALIS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ghost_levels, 256, 0));
			blocksMax = std::max(1, sms * per);
			blocksMaxAt.store(blocksMax);
		}
		const int blocks = (int)std::min<long long>((total + 255) / 256, blocksMax);
		void *args[] = { (void *)&GL };
		int slot = alisgpu__prof_start();
		ALIS_CUDA(cudaLaunchCooperativeKernel((const void *)k_ghost_levels, dim3(blocks), dim3(256), args, 0, gStream));
		alisgpu__prof_stop(slot, ALISGPU_K_GHOST);
		alisgpu__count_launch();
		return ALISGPU_OK;
	}
	if (record) {
		int rc = alisgpu__batch_flush();
		if (rc) return rc;
	}
	int q = 0;
	while (q < n) {
		GhostParams GP;
		memset(&GP, 0, sizeof GP);
		GP.L = w->L;
		GP.err = gErrWord;
		GP.complexField = g.complexField;
		for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
			int mm = m <= g.complexField ? m : 0;
			GP.F[m][c] = field == 0 ? w->E[mm][c] : w->H[mm][c];
		}
		int used = 0;
		long long total = 0;
		while (q < n && GP.n < ALIS_GHOST_GROUP && !(used & (1 << gl[q].comp))) {
			const alisgpu_ghost_copy &c = gl[q];
			used |= 1 << c.comp;
			GP.c[GP.n] = c;
			long long cells = (c.i1 < c.i0 || c.j1 < c.j0 || c.k1 < c.k0) ? 0 :
				(long long)(1 + c.i1 - c.i0) * (1 + c.j1 - c.j0) * (1 + c.k1 - c.k0);
			total += cells;
			if (total >= (1ll << 31)) return alisgpu__fail(ALISGPU_ERANGE, "ghost copies of %lld cells exceed 32-bit indexing", total);
			GP.start[GP.n + 1] = (int)total;
			GP.n++;
			q++;
		}
		if (total > 0) {
			int slot = alisgpu__prof_start();
			k_ghost<<<(unsigned)((total + 255) / 256), 256, 0, gStream>>>(GP);
			alisgpu__prof_stop(slot, ALISGPU_K_GHOST);
			alisgpu__count_launch();
			ALIS_CUDA(cudaGetLastError());
		}
	}
	return ALISGPU_OK;
}

static int applyPendingGhosts(alisgpu_world *w)
{
	if (w->pendingE.empty()) return ALISGPU_OK;
	int rc = runGhosts(w, 0, w->pendingE.data(), (int)w->pendingE.size());
	w->pendingE.clear();
	return rc;
}

// The block shape of this half step: while undecided, the first 3 x 3
// half steps of the field cycle through the shapes with events around
// them; once every one of them has completed, the shape with the least
// time (each shape's fastest run) stays.  ALISGPU_TUNE=0 keeps 32 x 4.
#define ALIS_TUNE_STEPS 9
#define ALIS_SHAPE_DEFAULT 1
#define ALIS_SHAPES ALIS_TY_CHOICES
static int tunedShape(alisgpu_world *w, int field, bool *timed)
{
	alisgpu_world::TyTuner &t = w->tune[field];
	*timed = false;
	if (t.choice >= 0) return t.choice;
	static int enabled = -1;
	if (enabled < 0) {
		const char *e = getenv("ALISGPU_TUNE");
		enabled = !(e && e[0] == '0');
	}
	static int forced = -2;
	if (forced == -2) {
		const char *e = getenv("ALISGPU_STEP_SHAPE");
		forced = e && atoi(e) >= 0 && atoi(e) < ALIS_SHAPES ? atoi(e) : -1;
	}
	if (forced >= 0) return t.choice = forced;
	if (!enabled) return t.choice = ALIS_SHAPE_DEFAULT;
	if (gProfOn) return ALIS_SHAPE_DEFAULT;
	if (t.seen < ALIS_TUNE_STEPS) {
		if (cudaEventCreate(&t.a[t.seen]) != cudaSuccess || cudaEventCreate(&t.b[t.seen]) != cudaSuccess)
			return t.choice = ALIS_SHAPE_DEFAULT;
		*timed = true;
		return t.seen % ALIS_SHAPES;
	}
	for (int q = 0; q < ALIS_TUNE_STEPS; q++) if (cudaEventQuery(t.b[q]) != cudaSuccess) return ALIS_SHAPE_DEFAULT;
	float best[ALIS_SHAPES];
	for (int c = 0; c < ALIS_SHAPES; c++) best[c] = 1e30f;
	for (int q = 0; q < ALIS_TUNE_STEPS; q++) {
		float ms = 0;
		if (cudaEventElapsedTime(&ms, t.a[q], t.b[q]) == cudaSuccess && ms < best[t.variant[q]]) best[t.variant[q]] = ms;
		cudaEventDestroy(t.a[q]), cudaEventDestroy(t.b[q]);
	}
	int c = ALIS_SHAPE_DEFAULT;
	for (int q = 0; q < ALIS_SHAPES; q++) if (best[q] < best[c]) c = q;
	return t.choice = c;
}

// Source values of a half step into the world's device buffer on stream
// st, through two pinned host buffers in turn: the copy is asynchronous
// and the consuming launch on st follows it.
static int stageValues(alisgpu_world *w, const float *vals, int n, cudaStream_t st, const float **dev)
{
	if (n > w->vcap) {
		// ordered on the stream that uses the buffer
		if (w->vbuf) ALIS_CUDA(cudaFreeAsync(w->vbuf, st));
		w->vbuf = 0, w->vcap = 0;
		ALIS_CUDA(cudaMallocAsync((void **)&w->vbuf, n * sizeof(float), st));
		w->vcap = n;
	}
	if (n > w->vpinCap) {
		for (int b = 0; b < 2; b++) {
			if (w->vpin[b]) {
				ALIS_CUDA(cudaEventSynchronize(w->vpinFree[b]));
				ALIS_CUDA(cudaFreeHost(w->vpin[b]));
				w->vpin[b] = 0;
			} else {
				ALIS_CUDA(cudaEventCreateWithFlags(&w->vpinFree[b], cudaEventDisableTiming));
				ALIS_CUDA(cudaEventRecord(w->vpinFree[b], st));
			}
			ALIS_CUDA(cudaMallocHost(&w->vpin[b], n * sizeof(float)));
		}
		w->vpinCap = n;
	}
	const int b = w->vpinNext;
	w->vpinNext ^= 1;
	ALIS_CUDA(cudaEventSynchronize(w->vpinFree[b]));
	memcpy(w->vpin[b], vals, n * sizeof(float));
	ALIS_CUDA(cudaMemcpyAsync(w->vbuf, w->vpin[b], n * sizeof(float), cudaMemcpyHostToDevice, st));
	ALIS_CUDA(cudaEventRecord(w->vpinFree[b], st));
	*dev = w->vbuf;
	return ALISGPU_OK;
}

// ---- recording a half step into the open batch group ----
static int recordStaged(alisgpu_world *aux, int field)
{
	aux->stagedValid[field] = false;
	const void *dS = 0;
	int rc = alisgpu__slot_sync(&aux->bS[field], aux->staged[field], sizeof(SmallStepParams), &dS);
	if (rc) return rc;
	const std::vector<float> &v = aux->stagedVals[field];
	const int voff = v.empty() ? -1 : (int)gRec.values.size();
	gRec.values.insert(gRec.values.end(), v.begin(), v.end());
	gRec.blocks.push_back(BatchBlock{ (const SmallStepParams *)dS, voff });
	return ALISGPU_OK;
}

static int recordGhosts(alisgpu_world *w, int field, const GhostLevels &GL, long long total)
{
	const void *dG = 0;
	int rc = alisgpu__slot_sync(&w->bG[field], &GL, sizeof GL, &dG);
	if (rc) return rc;
	w->ghostCells[field] = total;
	if (gRec.ghostTotal + total >= (1ll << 31)) return alisgpu__fail(ALISGPU_ERANGE, "batch: ghost copies exceed 32-bit indexing");
	gRec.ghosts.push_back(BatchGhost{ (const GhostLevels *)dG, gRec.ghostTotal });
	gRec.ghostTotal += (int)total;
	return ALISGPU_OK;
}

// A large world's half step in the open batch group: an entry per
// field set m, the TFSF auxiliary column's staged step as a one-block
// entry, the source patches and the ghost copies (H; E's wait for the
// next host read as usual).  P: the step's parameters with the per-world
// parts filled in.
static int recordHalfStep(alisgpu_world *w, const alisgpu_half_step *s, HalfStepParams &P)
{
	const alisgpu_geometry &g = w->g;
	const int field = s->field;
	if ((int)gRec.entries.size() + 1 + g.complexField > BATCH_WORLDS) {
		// the group is full: launch it and go on with a new one of the same kind
		const int kind = gRec.kind;
		int rc = batchLaunch();
		if (rc) return rc;
		gRec.kind = kind;
		w->batchStamp = gRec.stamp;
	}
	for (int m = 0; m <= g.complexField; m++) {
		P.m = m;
		for (int c = 0; c < 3; c++) {
			P.F[c] = field == 0 ? w->E[m][c] : w->H[m][c];
			P.G[c] = field == 0 ? w->H[m][c] : w->E[m][c];
			P.C[c] = field == 0 ? w->C[c] : 0;
			P.Fother[c] = w->E[m][c];
		}
		P.matIdx = field == 0 ? w->matIdx : 0;
		P.matTab = field == 0 ? w->matTab : 0;
		P.matWide = w->matWide;
		for (int f = 0; f < 6; f++) for (int q = 0; q < 2; q++) P.psi[f][q] = w->psi[field][m][f][q];
		const int nbx = (g.kMAX - g.kMIN + TX) / TX, nby = (g.jMAX - g.jMIN + BATCH_TY) / BATCH_TY, planes = g.iMAX - g.iMIN + 1;
		gRec.entries.push_back(BatchEntry{ nbx, nby, planes, gRec.nitems, fastDiv(nbx), fastDiv(nbx * nby) });
		gRec.params.push_back(P);
		const long long items = (long long)gRec.nitems + (long long)nbx * nby * planes;
		if (items >= (1ll << 31)) return alisgpu__fail(ALISGPU_ERANGE, "batch: too many items");
		gRec.nitems = (int)items;
	}
	int rc = runStagedAux(s, field);
	if (rc) return rc;
	if (s->nsrc > 0) {
		if (s->nsrc > ALIS_MAXSRC) return alisgpu__fail(ALISGPU_ERANGE, "half_step: %d source patches (max %d)", s->nsrc, ALIS_MAXSRC);
		static thread_local SourceParams SP;
		memset(&SP, 0, sizeof SP);
		SP.n = s->nsrc;
		SP.L = w->L;
		for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
			int mm = m <= g.complexField ? m : 0;
			SP.F[m][c] = field == 0 ? w->E[mm][c] : w->H[mm][c];
		}
		memcpy(SP.p, s->src, s->nsrc * sizeof(alisgpu_source_patch));
		SP.err = gErrWord;
		const void *dS = 0;
		if ((rc = alisgpu__slot_sync(&w->bSrc[field], &SP, sizeof SP, &dS))) return rc;
		const int voff = s->nvalues ? (int)gRec.values.size() : -1;
		gRec.values.insert(gRec.values.end(), s->values, s->values + s->nvalues);
		gRec.sources.push_back(BatchSource{ (const SourceParams *)dS, voff });
	}
	if (field == 0) {
		w->pendingE.assign(s->ghost, s->ghost + s->nghost);
	} else {
		w->hGhosts.assign(s->ghost, s->ghost + s->nghost);
		if ((rc = runGhosts(w, 1, s->ghost, s->nghost, true))) return rc;
	}
	w->hRecorded = false;
	gMainRec[field] = 0;
	return ALISGPU_OK;
}

// The scale table of a half world's field X for its next step: per
// updated plane, the other field's scales at the plane and at the plane +
// ALT of X (as read now), X's scales as read now, X's inverse scales.
struct HalfTableParams {
	const float *scG, *scOld, *inv;
	float *tab;
	int ni, p0, p1, alt;
};

__device__ __forceinline__ void halfTableEntry(const HalfTableParams &T, int t)
{
	if (t >= T.ni * HALF_TAB) return;
	const int pl = t / HALF_TAB, k = t % HALF_TAB, q = k % 3;
	if (pl < T.p0 || pl > T.p1) return;
	const int at = q * T.ni + pl;
	T.tab[t] = k < 3 ? T.scG[at] : k < 6 ? T.scG[at + T.alt] : k < 9 ? T.scOld[at] : T.inv[at];
}

__global__ void k_half_table(const HalfTableParams T)
{
	halfTableEntry(T, blockIdx.x * blockDim.x + threadIdx.x);
}

// The objects of each tile of ALIS_TILE_K x ALIS_TILE_J x 1 cells that
// their boxes (clipped to the updated cells, as the per-cell test clips
// them) meet, in list order: counted per tile, then filled object by
// object.  Made again only when the object boxes change.
static int objectTiles(alisgpu_world *w, HalfStepParams &P)
{
	const alisgpu_geometry &g = w->g;
	const int nI = g.iMAX - g.iMIN + 1, nJ = g.jMAX - g.jMIN + 1, nK = g.kMAX - g.kMIN + 1;
	P.tjn = (nJ + ALIS_TILE_J - 1) / ALIS_TILE_J, P.tkn = (nK + ALIS_TILE_K - 1) / ALIS_TILE_K;
	static thread_local std::vector<int> key;
	key.assign({ g.iMIN, g.iMAX, g.jMIN, g.jMAX, g.kMIN, g.kMAX });
	for (const DevObj &o : w->objs) key.insert(key.end(), { o.i0, o.i1, o.j0, o.j1, o.k0, o.k1 });
	if (key != w->tileKey || !w->tileStart) {
		const size_t nt = (size_t)nI * P.tjn * P.tkn;
		if (nt >= (1u << 31)) return alisgpu__fail(ALISGPU_ERANGE, "object tiles: %zu tiles", nt);
		std::vector<int> start(nt + 1, 0), at;
		// the tile ranges of each object's clipped box (empty: none)
		auto span = [&](const DevObj &o, int r[6]) {
			const int i0 = std::max(o.i0, g.iMIN), i1 = std::min(o.i1, g.iMAX);
			const int j0 = std::max(o.j0, g.jMIN), j1 = std::min(o.j1, g.jMAX);
			const int k0 = std::max(o.k0, g.kMIN), k1 = std::min(o.k1, g.kMAX);
			if (i1 < i0 || j1 < j0 || k1 < k0) return false;
			r[0] = i0 - g.iMIN, r[1] = i1 - g.iMIN;
			r[2] = (j0 - g.jMIN) / ALIS_TILE_J, r[3] = (j1 - g.jMIN) / ALIS_TILE_J;
			r[4] = (k0 - g.kMIN) / ALIS_TILE_K, r[5] = (k1 - g.kMIN) / ALIS_TILE_K;
			return true;
		};
		int r[6];
		for (const DevObj &o : w->objs)
			if (span(o, r))
				for (int a = r[0]; a <= r[1]; a++) for (int b = r[2]; b <= r[3]; b++) for (int c = r[4]; c <= r[5]; c++)
					start[((size_t)a * P.tjn + b) * P.tkn + c + 1]++;
		for (size_t t = 0; t < nt; t++) start[t + 1] += start[t];
		if ((size_t)start[nt] >= (1u << 31)) return alisgpu__fail(ALISGPU_ERANGE, "object tiles: %d entries", start[nt]);
		std::vector<int> list(std::max(start[nt], 1)), fill(start.begin(), start.end() - 1);
		for (size_t n = 0; n < w->objs.size(); n++)
			if (span(w->objs[n], r))
				for (int a = r[0]; a <= r[1]; a++) for (int b = r[2]; b <= r[3]; b++) for (int c = r[4]; c <= r[5]; c++)
					list[fill[((size_t)a * P.tjn + b) * P.tkn + c]++] = (int)n;
		alisgpu__freeAsync(w->tileStart), alisgpu__freeAsync(w->tileObj);
		w->tileStart = w->tileObj = 0;
		w->tileKey.clear();
		ALIS_CUDA(alisgpu__mallocAsync(&w->tileStart, (nt + 1) * sizeof(int)));
		ALIS_CUDA(alisgpu__mallocAsync(&w->tileObj, list.size() * sizeof(int)));
		ALIS_CUDA(orderedCopy(w->tileStart, start.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice));
		ALIS_CUDA(orderedCopy(w->tileObj, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice));
		w->tileKey = key;
	}
	P.tileStart = w->tileStart, P.tileObj = w->tileObj;
	return ALISGPU_OK;
}

// After a half step of a half world's field F, per (component, plane) of
// the planes it updated: the largest magnitude over the plane's slots
// gives F's next exponent, which becomes the next parity's exponent as
// read and as computed, its scale and the inverse scale F's next step
// stores with; the slots F's next step fills are zeroed (one warp per
// (component, plane)).  The threads after those make the other field's
// scale table from F's scales as read now.
struct HalfNextParams {
	const unsigned *m;
	unsigned *mZero;
	signed char *ex, *exK;
	float *sc, *inv;
	int ni, p0, p1;                            // layout planes the half step updates
	HalfTableParams other;
};

__global__ void k_half_next(const HalfNextParams P)
{
	const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
	const int w = t / 32, lane = (int)(threadIdx.x & 31);
	if (w >= 3 * P.ni) {
		halfTableEntry(P.other, t - 3 * P.ni * 32);
		return;
	}
	const int pl = w % P.ni;
	P.mZero[(size_t)w * HALF_SLOTS + lane] = 0;
	if (pl < P.p0 || pl > P.p1) return;
	const unsigned m = __reduce_max_sync(0xffffffffu, P.m[(size_t)w * HALF_SLOTS + lane]);
	if (lane == 0) {
		const int e = halfExponent(m);
		P.ex[w] = P.exK[w] = (signed char)e;
		P.sc[w] = pow2f(e);
		P.inv[w] = pow2f(-e);
	}
}

static HalfTableParams halfTableFor(const alisgpu_world *w, int field)
{
	HalfTableParams T;
	T.scG = halfScales(w, 1 - field), T.scOld = halfScales(w, field), T.inv = w->inv[field], T.tab = w->tab[field];
	T.ni = w->L.ni, T.p0 = w->g.iMIN - w->L.i0, T.p1 = w->g.iMAX - w->L.i0, T.alt = field == 0 ? 1 : -1;
	return T;
}

// the scale table of a field whose table is not current
static int halfTable(alisgpu_world *w, int field)
{
	const HalfTableParams T = halfTableFor(w, field);
	k_half_table<<<(T.ni * HALF_TAB + 255) / 256, 256, 0, gStream>>>(T);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	w->tabFresh[field] = true;
	return ALISGPU_OK;
}

static int halfNext(alisgpu_world *w, int field)
{
	const int next = (int)(w->nHalf[field] & 1);
	HalfNextParams P;
	P.m = w->mx[field][next ^ 1], P.mZero = w->mx[field][next];
	P.ex = w->ex[field][next], P.exK = w->exK[field][next], P.sc = w->sc[field][next], P.inv = w->inv[field];
	P.ni = w->L.ni, P.p0 = w->g.iMIN - w->L.i0, P.p1 = w->g.iMAX - w->L.i0;
	P.other = halfTableFor(w, 1 - field);
	const int threads = 3 * P.ni * 32 + P.ni * HALF_TAB;
	k_half_next<<<(threads + 255) / 256, 256, 0, gStream>>>(P);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	w->tabFresh[1 - field] = true;
	return ALISGPU_OK;
}

extern "C" int alisgpu_half_step_run(alisgpu_world *w, const alisgpu_half_step *s)
{
	bindWorld(w);
	if (!w || !s || s->field < 0 || s->field > 1) return alisgpu__fail(ALISGPU_EINVAL, "half_step: bad argument");
	if (s->ntfsf > ALIS_MAXTFSF) return alisgpu__fail(ALISGPU_ERANGE, "half_step: %d TFSF boxes (max %d)", s->ntfsf, ALIS_MAXTFSF);
	const alisgpu_geometry &g = w->g;
	const int field = s->field;
	if (!w->dtd[field][0]) return alisgpu__fail(ALISGPU_EINVAL, "half_step: line tables not set");
	HalfStepParams P;
	memset(&P, 0, sizeof P);
	P.iMIN = g.iMIN, P.iMAX = g.iMAX, P.jMIN = g.jMIN, P.jMAX = g.jMAX, P.kMIN = g.kMIN, P.kMAX = g.kMAX;
	P.iMin = g.iMin, P.iMax = g.iMax, P.jMin = g.jMin, P.jMax = g.jMax, P.kMin = g.kMin, P.kMax = g.kMax;
	P.L = w->L;
	for (int a = 0; a < 3; a++) P.dtd[a] = w->dtd[field][a];
	for (int q = 0; q < 9; q++) P.cp[q] = w->cp[field][q];
	int mins[3] = { g.iMin, g.jMin, g.kMin }, maxs[3] = { g.iMax, g.jMax, g.kMax };
	int MINs[3] = { g.iMIN, g.jMIN, g.kMIN }, MAXs[3] = { g.iMAX, g.jMAX, g.kMAX };
	const int Alt = field == 0 ? 1 : -1;
	for (int f = 0; f < 6; f++) {
		int a = f % 3;
		bool on = f < 3 ? MINs[a] < mins[a] : MAXs[a] > maxs[a];
		if (!on) continue;
		if (!w->psi[field][0][f][0].p) continue;
		P.slabOn[f] = 1;
		if (f < 3) P.slabLo[f] = MINs[a] - (Alt - 1) / 2, P.slabHi[f] = mins[a] - (Alt + 3) / 2;
		else P.slabLo[f] = maxs[a] + 2, P.slabHi[f] = MAXs[a];
	}
	P.nobj = (int)w->objs.size();
	P.obj = w->dObjs;
	if (P.nobj > 8) {
		int rc = objectTiles(w, P);
		if (rc) return rc;
	}
	P.ntfsf = s->ntfsf;
	for (int q = 0; q < s->ntfsf; q++) P.tf[q] = tfsfFor(w, s->tfsf[q], field);
	P.err = gErrWord;

	// a batch records the call (its uploads then go to the batch streams):
	// an auxiliary column's step is staged for its parent's entry, any
	// other step joins the group of its field
	const long long cells = (long long)(g.iMAX - g.iMIN + 1) * (g.jMAX - g.jMIN + 1) * (g.kMAX - g.kMIN + 1);
	// a half world takes the grid launch, unrecorded, with its source
	// patches inside the cells the step updates
	if (w->half) {
		if (batchRecording()) return alisgpu__fail(ALISGPU_ENOTSUP, "half_step: batched recording of a half world");
		for (int q = 0; q < s->nsrc; q++) {
			const alisgpu_source_patch &p = s->src[q];
			if (p.m != 0 || p.comp < 0 || p.comp > 2 || p.i0 < g.iMIN || p.i1 > g.iMAX || p.j0 < g.jMIN || p.j1 > g.jMAX ||
			    p.k0 < g.kMIN || p.k1 > g.kMAX)
				return alisgpu__fail(ALISGPU_ENOTSUP, "half_step: a source patch of a half world outside the updated cells");
		}
	}
	const bool smallPath = !w->half && cells <= (s->concurrent ? ALIS_SMALL_CELLS : ALIS_TINY_CELLS) && s->nsrc <= ALIS_MAXSRC &&
	                       s->nghost <= ALIS_SMALL_GHOSTS;
	const int rec = alisgpu__batch_enter(smallPath && s->concurrent && s->attach ? BATCH_NONE : (field == 0 ? BATCH_E : BATCH_H), w);
	if (rec < 0) return alisgpu__fail(ALISGPU_ECUDA, "half_step: batch launch failed: %s", gErr);
	// per-axis classification: CPML slabs, TFSF planes, object ranges
	// (made again only when one of them changed)
	static thread_local std::vector<int> key;
	key.clear();
	for (int f = 0; f < 6; f++) key.push_back(P.slabOn[f]), key.push_back(P.slabLo[f]), key.push_back(P.slabHi[f]);
	for (int q = 0; q < P.ntfsf; q++) {
		const DevTfsf &T = P.tf[q];
		const int b[12] = { T.iMin, T.iMax, T.jMin, T.jMax, T.kMin, T.kMax, T.iMIN, T.iMAX, T.jMIN, T.jMAX, T.kMIN, T.kMAX };
		key.insert(key.end(), b, b + 12);
	}
	for (const DevObj &o : w->objs) {
		const int b[6] = { o.i0, o.i1, o.j0, o.j1, o.k0, o.k1 };
		key.insert(key.end(), b, b + 6);
	}
	if (key == w->clsKey[field] && w->cls[field][0] && w->cls[field][1] && w->cls[field][2]) {
		for (int a = 0; a < 3; a++) P.cls[a] = w->cls[field][a];
	} else {
		w->clsKey[field] = key;
		int n[3] = { g.iMAX - g.iMIN + 1, g.jMAX - g.jMIN + 1, g.kMAX - g.kMIN + 1 };
		int lo0[3] = { g.iMIN, g.jMIN, g.kMIN }, hi0[3] = { g.iMAX, g.jMAX, g.kMAX };
		std::vector<unsigned short> t[3];
		for (int a = 0; a < 3; a++) t[a].assign(n[a], 0);
		auto mark = [&](int a, int lo, int hi, unsigned short bit) {
			for (int q = max(lo, lo0[a]); q <= min(hi, hi0[a]); q++) t[a][q - lo0[a]] |= bit;
		};
		for (int f = 0; f < 6; f++) if (P.slabOn[f]) mark(f % 3, P.slabLo[f], P.slabHi[f], f < 3 ? CLS_PML_LO : CLS_PML_HI);
		for (int q = 0; q < P.ntfsf; q++) {
			const DevTfsf &T = P.tf[q];
			int mn[3] = { T.iMin, T.jMin, T.kMin }, mx[3] = { T.iMax, T.jMax, T.kMax };
			int MN[3] = { T.iMIN, T.jMIN, T.kMIN }, MX[3] = { T.iMAX, T.jMAX, T.kMAX };
			for (int a = 0; a < 3; a++) {
				if (mn[a] > lo0[a]) mark(a, mn[a], mn[a], CLS_TFSF);
				if (mx[a] < hi0[a]) mark(a, mx[a] + field, mx[a] + field, CLS_TFSF);
				// the index range of the faces' corrections: every face
				// plane and every range tfsfCell tests along this axis
				mark(a, min(mn[a], MN[a]) - 1, max(mx[a], MX[a]) + 1, CLS_TFSF_IN);
			}
		}
		for (size_t q = 0; q < w->objs.size(); q++) {
			const DevObj &o = w->objs[q];
			unsigned short bit = q < 8 ? (unsigned short)(1u << q) : (unsigned short)CLS_OBJ8;
			mark(0, o.i0, o.i1, bit), mark(1, o.j0, o.j1, bit), mark(2, o.k0, o.k1, bit);
		}
		for (int a = 0; a < 3; a++) {
			if (!w->cls[field][a]) ALIS_CUDA(alisgpu__mallocAsync(&w->cls[field][a], n[a] * sizeof(unsigned short)));
			if (w->clsHost[field][a] != t[a]) {
				w->clsHost[field][a] = t[a];
				ALIS_CUDA(cudaMemcpyAsync(w->cls[field][a], w->clsHost[field][a].data(), n[a] * sizeof(unsigned short), cudaMemcpyHostToDevice, gStream));
			}
			P.cls[a] = w->cls[field][a];
		}
	}
	if (w->L.elems() >= (1ull << 31))
		return alisgpu__fail(ALISGPU_ERANGE, "half_step: %zu elements per field exceed 32-bit indexing", w->L.elems());
	// an auxiliary world runs on the side stream (not while timing kernels
	// one by one); any other world first waits for the auxiliary step of
	// the other field, whose fields its TFSF corrections read
	const bool side = s->concurrent && !gProfOn;
	if (!side && gAuxRec[1 - field]) ALIS_CUDA(cudaStreamWaitEvent(gStream, gEvAuxDone[1 - field], 0));
	if (smallPath) {
		static thread_local SmallStepParams S;
		S.nm = 1 + g.complexField;
		for (int m = 0; m < S.nm; m++) {
			S.P[m] = P;
			HalfStepParams &Q = S.P[m];
			Q.m = m;
			for (int c = 0; c < 3; c++) {
				Q.F[c] = field == 0 ? w->E[m][c] : w->H[m][c];
				Q.G[c] = field == 0 ? w->H[m][c] : w->E[m][c];
				Q.C[c] = field == 0 ? w->C[c] : 0;
				Q.Fother[c] = w->E[m][c];
			}
			for (int f = 0; f < 6; f++) for (int q = 0; q < 2; q++) Q.psi[f][q] = w->psi[field][m][f][q];
		}
		for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
			int mm = m <= g.complexField ? m : 0;
			S.F[m][c] = field == 0 ? w->E[mm][c] : w->H[mm][c];
		}
		S.nsrc = s->nsrc, S.nghost = s->nghost;
		if (s->nsrc) memcpy(S.src, s->src, s->nsrc * sizeof(alisgpu_source_patch));
		if (s->nghost) memcpy(S.ghost, s->ghost, s->nghost * sizeof(alisgpu_ghost_copy));
		// recorded by a batch: staged for the parent's entry, or an entry of its own
		if (rec) {
			S.vdev = 0;
			memset(S.v, 0, sizeof S.v);
			if (s->attach && s->concurrent) {
				if (!w->staged[field]) w->staged[field] = new SmallStepParams();
				*w->staged[field] = S;
				w->stagedValid[field] = true;
				w->stagedVals[field].assign(s->values, s->values + s->nvalues);
				return ALISGPU_OK;
			}
			if (!s->concurrent) {
				int rc = runStagedAux(s, field);
				if (rc) return rc;
			}
			const void *dS = 0;
			int rc = alisgpu__slot_sync(&w->bS[field], &S, sizeof S, &dS);
			if (rc) return rc;
			const int voff = s->nvalues ? (int)gRec.values.size() : -1;
			gRec.values.insert(gRec.values.end(), s->values, s->values + s->nvalues);
			gRec.blocks.push_back(BatchBlock{ (const SmallStepParams *)dS, voff });
			gMainRec[field] = 0;
			return ALISGPU_OK;
		}
		// on the side stream: after the parent's last step of the other
		// field, or after everything when a join asked for that
		cudaStream_t st = gStream;
		if (side) {
			st = gSide;
			if (gSideWaitsAll || !gMainRec[1 - field]) {
				// (no record of the parent's last step of the other field: wait for everything)
				ALIS_CUDA(cudaEventRecord(gEvJoin, gStream));
				ALIS_CUDA(cudaStreamWaitEvent(gSide, gEvJoin, 0));
				gSideWaitsAll = 0;
			} else {
				ALIS_CUDA(cudaStreamWaitEvent(gSide, gEvMainDone[1 - field], 0));
			}
		}
		S.vdev = 0;
		if (s->attach && s->concurrent && !gProfOn) {
			// runs inside the parent's next launch of this field, on the main stream
			if (s->nvalues > ALIS_MAXSRCV) {
				int rc = stageValues(w, s->values, s->nvalues, gStream, &S.vdev);
				if (rc) return rc;
			} else if (s->nvalues) {
				memcpy(S.v, s->values, s->nvalues * sizeof(float));
			}
			if (!w->staged[field]) w->staged[field] = new SmallStepParams();
			*w->staged[field] = S;
			w->stagedValid[field] = true;
			return ALISGPU_OK;
		}
		if (s->nvalues > ALIS_MAXSRCV) {
			int rc = stageValues(w, s->values, s->nvalues, st, &S.vdev);
			if (rc) return rc;
		} else if (s->nvalues) {
			memcpy(S.v, s->values, s->nvalues * sizeof(float));
		}
		if (!s->concurrent) {
			int rc = runStagedAux(s, field);
			if (rc) return rc;
		}
		int slot = alisgpu__prof_start();
		if (field == 0) k_small_step<1><<<1, SMALL_THREADS, 0, st>>>(S);
		else k_small_step<-1><<<1, SMALL_THREADS, 0, st>>>(S);
		alisgpu__prof_stop(slot, ALISGPU_K_STEP_AUX);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
		if (side) {
			ALIS_CUDA(cudaEventRecord(gEvAuxDone[field], gSide));
			gAuxRec[field] = 1, gSideUsed = 1;
		} else if (s->ntfsf > 0) {
			ALIS_CUDA(cudaEventRecord(gEvMainDone[field], gStream));
			gMainRec[field] = 1;
		} else {
			gMainRec[field] = 0;
		}
		return ALISGPU_OK;
	}
	if (rec) return recordHalfStep(w, s, P);
	if (w->half && !w->tabFresh[field]) {
		int rc = halfTable(w, field);
		if (rc) return rc;
	}
	const int ni = g.iMAX - g.iMIN + 1;
	bool timed = false, fused = false;
	const int v = tunedShape(w, field, &timed);
	const int ty = kTyChoice[v];
	const int bp = w->half ? BLOCK_PLANES(true) : BLOCK_PLANES(false);
	dim3 grid((g.kMAX - g.kMIN + TX) / TX, (g.jMAX - g.jMIN + ty) / ty, (ni + bp - 1) / bp);
	if (timed) ALIS_CUDA(cudaEventRecord(w->tune[field].a[w->tune[field].seen], gStream));
	for (int m = 0; m <= g.complexField; m++) {
		P.m = m;
		for (int c = 0; c < 3; c++) {
			P.F[c] = field == 0 ? w->E[m][c] : w->H[m][c];
			P.G[c] = field == 0 ? w->H[m][c] : w->E[m][c];
			P.C[c] = field == 0 ? w->C[c] : 0;
			P.Fother[c] = w->E[m][c];
		}
		P.matIdx = field == 0 ? w->matIdx : 0;
		P.matTab = field == 0 ? w->matTab : 0;
		P.matWide = w->matWide;
		for (int f = 0; f < 6; f++) for (int q = 0; q < 2; q++) P.psi[f][q] = w->psi[field][m][f][q];
		if (w->half) {
			// step n stores with the inverse scales made from the maxima of
			// step n - 1 and accumulates its own
			P.h.tab = w->tab[field];
			P.h.mCur = w->mx[field][w->nHalf[field] & 1];
		}
		int slot = alisgpu__prof_start();
		alisgpu_world *aux = s->ntfsf == 1 && m == 0 ? s->tfsf[0].aux : 0;
		if (aux && aux->stagedValid[field]) {
			// with the auxiliary column's step of this field as the first plane of blocks
			static thread_local FusedStepParams FP;
			FP.P = P;
			FP.aux = *aux->staged[field];
			aux->stagedValid[field] = false;
			fused = true;
			if (field == 0) launchHalfStep<1>(v, grid, P, &FP, gStream, w->half);
			else launchHalfStep<-1>(v, grid, P, &FP, gStream, w->half);
		} else if (field == 0) launchHalfStep<1>(v, grid, P, 0, gStream, w->half);
		else launchHalfStep<-1>(v, grid, P, 0, gStream, w->half);
		alisgpu__prof_stop(slot, field == 0 ? ALISGPU_K_STEP_E : ALISGPU_K_STEP_H);
		alisgpu__count_launch();
	}
	ALIS_CUDA(cudaGetLastError());
	if (w->half) w->nHalf[field]++, w->tabFresh[field] = false;
	if (timed) {
		alisgpu_world::TyTuner &t = w->tune[field];
		ALIS_CUDA(cudaEventRecord(t.b[t.seen], gStream));
		t.variant[t.seen++] = v;
	}
	{
		int rc = runStagedAux(s, field);
		if (rc) return rc;
	}

	// sources
	if (s->nsrc > 0) {
		if (s->nsrc > ALIS_MAXSRC) return alisgpu__fail(ALISGPU_ERANGE, "half_step: %d source patches (max %d)", s->nsrc, ALIS_MAXSRC);
		static thread_local SourceParams SP;
		SP.n = s->nsrc;
		SP.L = w->L;
		for (int m = 0; m < 2; m++) for (int c = 0; c < 3; c++) {
			int mm = m <= g.complexField ? m : 0;
			SP.F[m][c] = field == 0 ? w->E[mm][c] : w->H[mm][c];
		}
		memcpy(SP.p, s->src, s->nsrc * sizeof(alisgpu_source_patch));
		SP.vdev = 0;
		SP.err = gErrWord;
		SP.ex = w->half ? halfRead(w, field) : 0;
		if (s->nvalues <= ALIS_MAXSRCV) {
			memcpy(SP.v, s->values, s->nvalues * sizeof(float));
		} else {
			int rc = stageValues(w, s->values, s->nvalues, gStream, &SP.vdev);
			if (rc) return rc;
		}
		int slot = alisgpu__prof_start();
		k_sources<<<1, 256, 0, gStream>>>(SP);
		alisgpu__prof_stop(slot, ALISGPU_K_SOURCE);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}

	// ghost copies: E's wait for the next host read, H's run now
	if (field == 0) {
		w->pendingE.assign(s->ghost, s->ghost + s->nghost);
		w->hRecorded = false;
	} else {
		if (!w->evHCells) ALIS_CUDA(cudaEventCreateWithFlags(&w->evHCells, cudaEventDisableTiming));
		ALIS_CUDA(cudaEventRecord(w->evHCells, gStream));
		w->hGhosts.assign(s->ghost, s->ghost + s->nghost);
		int rc = runGhosts(w, 1, s->ghost, s->nghost);
		if (rc) return rc;
		if (w->half && (rc = halfNext(w, 1))) return rc;
		w->hOps = gOps, w->hRecorded = true;
	}
	if (field == 0 && w->half) {
		int rc = halfNext(w, 0);
		if (rc) return rc;
	}
	// an auxiliary world stepped on the side stream waits for this record;
	// none is needed when there is no box or its column ran in this launch
	if (s->ntfsf > 0 && !fused) {
		ALIS_CUDA(cudaEventRecord(gEvMainDone[field], gStream));
		gMainRec[field] = 1;
	} else {
		gMainRec[field] = 0;
	}
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// Instantaneous Poynting flux through an axis-normal plane (reference
// src/output.c:233-356) with the reference's arithmetic in its order as
// one OpenMP thread runs it: two sums, each an outer loop over one
// in-plane index of (H-grid spacing x inner sum), the inner sum over the
// other index with half-weight edge terms in double and float interior
// terms; H is averaged across the plane.  One block: its threads compute
// the inner sums, one thread adds the outer loops in order.
// ---------------------------------------------------------------------
// an observer's read of element c of a field component: float storage, or
// (ex: the component's exponents per plane of a half world) a half value
// times its plane's power of two (plane = c / si, the layout's plane pitch)
__device__ __forceinline__ float fieldAt(const float *p, const signed char *ex, long long si, long long c)
{
	return ex ? halfAt(p, c, pow2f(ex[c / si])) : p[c];
}

struct PlaneParams {
	Layout L;
	const float *E[3], *H[3];
	const signed char *exE[3], *exH[3];          // half storage (else null)
	int axis, pos;
	int lo[2], hi[2];                          // in-plane axes u < v
	const float *wE[2], *wH[2];                // spacings over [lo, hi], indexed by index
	float *out;
};

// One warp per inner sum: the warp stages the row's terms in shared
// memory with coalesced loads, lane 0 then adds them in the reference's
// order.  Rows of the first loop come first in inner[], then the second.
#define PF_WARPS 8
#define PF_CHUNK 256                           // row cells staged at a time
__global__ void __launch_bounds__(32 * PF_WARPS) k_plane_rows(const PlaneParams P)
{
	__shared__ float se[PF_WARPS][PF_CHUNK], sh[PF_WARPS][PF_CHUNK];   // a chunk of each warp's row
	const int a = P.axis;
	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const int n1 = P.hi[a == 1 ? 1 : 0] - P.lo[a == 1 ? 1 : 0];
	const int n2 = P.hi[a == 1 ? 0 : 1] - P.lo[a == 1 ? 0 : 1];
	const int row = blockIdx.x * PF_WARPS + warp;
	if (row >= n1 + n2) return;
	const int l = row < n1 ? 0 : 1, t = l == 0 ? row : row - n1;
	// x plane (u=j, v=k): Ey (Hz) over k for each j, then -Ez (Hy) over j for each k;
	// y plane (u=i, v=k): Ez (Hx) over i for each k, then -Ex (Hz) over k for each i;
	// z plane (u=i, v=j): Ex (Hy) over j for each i, then -Ey (Hx) over i for each j
	const int oAx = (a == 1) == (l == 0) ? 1 : 0, nAx = 1 - oAx;
	const int ec = a == 0 ? (l == 0 ? 1 : 2) : a == 1 ? (l == 0 ? 2 : 0) : (l == 0 ? 0 : 1);
	const int hc = a == 0 ? (l == 0 ? 2 : 1) : a == 1 ? (l == 0 ? 0 : 2) : (l == 0 ? 1 : 0);
	const int o = P.lo[oAx] + 1 + t, m0 = P.lo[nAx], m1 = P.hi[nAx];
	const float *wN = P.wE[nAx];
	const float *Ec = P.E[ec], *Hc = P.H[hc];
	const signed char *xE = P.exE[ec], *xH = P.exH[hc];
	const long long si = P.L.si;
	const long long dn = a == 0 ? P.L.si : a == 1 ? P.L.sj : 1;  // H across the plane
	auto cell = [&](int n) -> long long {
		const int u = oAx == 0 ? o : n, v = oAx == 0 ? n : o;
		return a == 0 ? P.L.at(P.pos, u, v) : a == 1 ? P.L.at(u, P.pos, v) : P.L.at(u, v, P.pos);
	};
	float sum = 0;
	// edge terms: `sum +/-= 0.5 * w * E * (H + H')` in double
	for (int e = 0; e < 2; e++) {
		const int n = e ? m1 : m0;
		const long long c = cell(n);
		const double hw = 0.5 * (double)wN[n];
		const double term = __dmul_rn(hw * (double)fieldAt(Ec, xE, si, c), (double)__fadd_rn(fieldAt(Hc, xH, si, c), fieldAt(Hc, xH, si, c + dn)));
		sum = __double2float_rn(l == 0 ? __dadd_rn((double)sum, term) : __dsub_rn((double)sum, term));
	}
	// interior terms in float, a chunk of the row at a time
	for (int base = m0 + 1; base < m1; base += PF_CHUNK) {
		const int cnt = min(PF_CHUNK, m1 - base);
		__syncwarp();
		for (int q = lane; q < cnt; q += 32) {
			const long long c = cell(base + q);
			se[warp][q] = __fmul_rn(wN[base + q], fieldAt(Ec, xE, si, c));
			sh[warp][q] = __fadd_rn(fieldAt(Hc, xH, si, c), fieldAt(Hc, xH, si, c + dn));
		}
		__syncwarp();
		if (lane == 0)
			for (int q = 0; q < cnt; q++) {
				const float term = __fmul_rn(se[warp][q], sh[warp][q]);
				sum = l == 0 ? __fadd_rn(sum, term) : __fsub_rn(sum, term);
			}
	}
	if (lane == 0) P.out[1 + row] = sum;
}

// the outer loops in order: inner sums staged in shared memory first
__global__ void __launch_bounds__(256) k_plane_total(const PlaneParams P)
{
	extern __shared__ float inner[];
	const int a = P.axis;
	const int n1 = P.hi[a == 1 ? 1 : 0] - P.lo[a == 1 ? 1 : 0];
	const int n2 = P.hi[a == 1 ? 0 : 1] - P.lo[a == 1 ? 0 : 1];
	for (int q = threadIdx.x; q < n1 + n2; q += blockDim.x) inner[q] = P.out[1 + q];
	__syncthreads();
	if (threadIdx.x) return;
	float Sum = 0, Part = 0;
	for (int l = 0; l < 2; l++) {
		const int oAx = (a == 1) == (l == 0) ? 1 : 0;
		const int o0 = P.lo[oAx], o1 = P.hi[oAx];
		const float *wO = P.wH[oAx];
		float acc = 0;
		for (int o = o0 + 1; o <= o1; o++) acc = __fadd_rn(acc, __fmul_rn(wO[o], inner[(l == 0 ? 0 : n1) + (o - o0 - 1)]));
		if (l == 0) Sum = acc; else Part = acc;
	}
	P.out[0] = __fadd_rn(Sum, Part);
}

extern "C" int alisgpu_plane_flux(alisgpu_world *w, int axis, int pos, const int lo[2], const int hi[2], float *out)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	if (!w || axis < 0 || axis > 2 || !lo || !hi || !out) return alisgpu__fail(ALISGPU_EINVAL, "plane_flux: bad argument");
	if (!w->sp[0][0]) return alisgpu__fail(ALISGPU_EINVAL, "plane_flux: spacing tables not set");
	const alisgpu_geometry &g = w->g;
	const int MINs[3] = { g.iMIN, g.jMIN, g.kMIN }, MAXs[3] = { g.iMAX, g.jMAX, g.kMAX };
	const int ua = axis == 0 ? 1 : 0, va = axis == 2 ? 1 : 2;
	if (pos < MINs[axis] - 1 || pos > MAXs[axis] || lo[0] < MINs[ua] || hi[0] > MAXs[ua] || lo[1] < MINs[va] ||
	    hi[1] > MAXs[va] || hi[0] < lo[0] || hi[1] < lo[1])
		return alisgpu__fail(ALISGPU_ERANGE, "plane_flux: plane or range outside the world");
	// E's upper halo is written by the deferred ghost copies
	if (pos > MAXs[axis] - 1 || hi[0] > MAXs[ua] || hi[1] > MAXs[va]) {
		int rc = applyPendingGhosts(w);
		if (rc) return rc;
	}
	const int n1 = axis == 1 ? hi[1] - lo[1] : hi[0] - lo[0];
	const int n2 = axis == 1 ? hi[0] - lo[0] : hi[1] - lo[1];
	const size_t floats = 1 + (size_t)n1 + n2;
	if (floats > w->planeTabFloats) {
		ALIS_CUDA(cudaStreamSynchronize(gStream));
		if (w->planeTab) alisgpu__freeAsync(w->planeTab);
		w->planeTab = 0, w->planeTabFloats = 0;
		ALIS_CUDA(alisgpu__mallocAsync(&w->planeTab, floats * sizeof(float)));
		w->planeTabFloats = floats;
	}
	PlaneParams P;
	memset(&P, 0, sizeof P);
	P.L = w->L;
	for (int c = 0; c < 3; c++) P.E[c] = w->E[0][c], P.H[c] = w->H[0][c];
	if (w->half)
		for (int c = 0; c < 3; c++) P.exE[c] = halfRead(w, 0) + c * w->L.ni, P.exH[c] = halfRead(w, 1) + c * w->L.ni;
	P.axis = axis, P.pos = pos;
	const int axes[2] = { ua, va };
	for (int q = 0; q < 2; q++) {
		P.lo[q] = lo[q], P.hi[q] = hi[q];
		P.wE[q] = w->sp[0][axes[q]] - MINs[axes[q]];
		P.wH[q] = w->sp[1][axes[q]] - MINs[axes[q]];
	}
	P.out = w->planeTab;
	const size_t smem = (size_t)(n1 + n2 + 1) * sizeof(float);
	if (smem > 48 * 1024) return alisgpu__fail(ALISGPU_ERANGE, "plane_flux: plane of %d + %d rows too large", n1, n2);
	int slot = alisgpu__prof_start();
	if (n1 + n2 > 0) {
		k_plane_rows<<<(n1 + n2 + PF_WARPS - 1) / PF_WARPS, 32 * PF_WARPS, 0, gStream>>>(P);
		alisgpu__count_launch();
	}
	k_plane_total<<<1, 256, smem, gStream>>>(P);
	alisgpu__prof_stop(slot, ALISGPU_K_FLUX);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	ALIS_CUDA(cudaMemcpyAsync(out, P.out, sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// E and H over a small index box, for observers that read a few cells
// (get): one gather launch and one copy instead of whole arrays
// ---------------------------------------------------------------------
struct BoxGatherParams {
	Layout L;
	const float *F[2][2][3];                   // [E/H][m][comp]
	int nm;
	int i0, j0, k0, ni, nj, nk;
	float *out;                                // [E/H][m][comp][ni][nj][nk]
	const signed char *ex[2];                  // half storage: the fields' exponents (else null)
};

__global__ void k_box_gather(const BoxGatherParams P)
{
	const int cells = P.ni * P.nj * P.nk;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= cells * 6 * P.nm) return;
	const int r = t % cells, fc = t / cells;           // fc = (field * nm + m) * 3 + comp
	const int comp = fc % 3, m = (fc / 3) % P.nm, f = fc / (3 * P.nm);
	const int k = P.k0 + r % P.nk, j = P.j0 + (r / P.nk) % P.nj, i = P.i0 + r / (P.nk * P.nj);
	if (P.ex[0]) P.out[t] = halfAt(P.F[f][m][comp], P.L.at(i, j, k), pow2f(P.ex[f][comp * P.L.ni + (i - P.L.i0)]));
	else P.out[t] = P.F[f][m][comp][P.L.at(i, j, k)];
}

extern "C" int alisgpu_field_box_download(alisgpu_world *w, int i0, int i1, int j0, int j1, int k0, int k1, float *host)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	if (!w || !host || i1 < i0 || j1 < j0 || k1 < k0) return alisgpu__fail(ALISGPU_EINVAL, "field_box_download: bad argument");
	const Layout &L = w->L;
	if (i0 < L.i0 || i1 >= L.i0 + L.ni || j0 < L.j0 || j1 >= L.j0 + L.nj || k0 < L.k0 || k1 >= L.k0 + L.nk)
		return alisgpu__fail(ALISGPU_ERANGE, "field_box_download: box outside the halo'd grid");
	const alisgpu_geometry &g = w->g;
	// E's upper halo is written by the deferred ghost copies
	if (i1 > g.iMAX || j1 > g.jMAX || k1 > g.kMAX) {
		int rc = applyPendingGhosts(w);
		if (rc) return rc;
	}
	BoxGatherParams P;
	memset(&P, 0, sizeof P);
	P.L = L;
	P.nm = 1 + g.complexField;
	for (int m = 0; m < P.nm; m++) for (int c = 0; c < 3; c++) P.F[0][m][c] = w->E[m][c], P.F[1][m][c] = w->H[m][c];
	if (w->half) P.ex[0] = halfRead(w, 0), P.ex[1] = halfRead(w, 1);
	P.i0 = i0, P.j0 = j0, P.k0 = k0, P.ni = 1 + i1 - i0, P.nj = 1 + j1 - j0, P.nk = 1 + k1 - k0;
	const size_t n = (size_t)P.ni * P.nj * P.nk * 6 * P.nm;
	if (n >= (1u << 31)) return alisgpu__fail(ALISGPU_ERANGE, "field_box_download: box of %zu values too large", n);
	if (n > w->planeTabFloats) {
		ALIS_CUDA(cudaStreamSynchronize(gStream));
		if (w->planeTab) alisgpu__freeAsync(w->planeTab);
		w->planeTab = 0, w->planeTabFloats = 0;
		ALIS_CUDA(alisgpu__mallocAsync(&w->planeTab, n * sizeof(float)));
		w->planeTabFloats = n;
	}
	P.out = w->planeTab;
	int slot = alisgpu__prof_start();
	k_box_gather<<<(unsigned)((n + 255) / 256), 256, 0, gStream>>>(P);
	alisgpu__prof_stop(slot, ALISGPU_K_GATHER);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	ALIS_CUDA(cudaMemcpyAsync(host, P.out, n * sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// Running DFT of sliceFreqDom (reference src/slices.c:326-356) over a box:
// F += f(i,j,k) * re, G += f(i,j,k) * im with f one of the E/H samples of
// the field functions (reference src/fields.c:130-291): a raw component,
// E averaged over its two samples, H over its four, with the mirror
// parities of symmetry planes, in their float arithmetic.  The sums stay
// on the device until the slice is written.
// ---------------------------------------------------------------------
struct alisgpu_slice_dft {
	alisgpu_world *w;
	int i0, i1, j0, j1, k0, k1;
	float *acc;                                // F then G, box arrays (k fastest)
};

struct SliceDftParams {
	Layout L;
	const float *F;                            // the sampled component (E or H, m)
	const signed char *ex;                     // its exponents per plane (half storage; else null)
	int kind;                                  // 0 raw, 1 E pair, 2 H quad; -1: zero (imaginary part of a real field)
	int d1, d2;                                // offsets of the second (and third) sample
	float base;                                // 1, 0.5, 0.25
	int sym[3];
	float par[3];
	int i0, j0, k0, ni, nj, nk;
	float re, im;
	float *acc;
};

__global__ void k_slice_dft(const SliceDftParams P)
{
	const int cells = P.ni * P.nj * P.nk;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= cells) return;
	int k = P.k0 + t % P.nk, j = P.j0 + (t / P.nk) % P.nj, i = P.i0 + t / (P.nk * P.nj);
	float v = 0;
	if (P.kind >= 0) {
		float p = P.base;
		if (P.sym[0] && i < 0) i = -i, p *= P.par[0];
		if (P.sym[1] && j < 0) j = -j, p *= P.par[1];
		if (P.sym[2] && k < 0) k = -k, p *= P.par[2];
		const long long c = P.L.at(i, j, k);
		const long long si = P.L.si;
		if (P.kind == 0) v = p * fieldAt(P.F, P.ex, si, c);
		else if (P.kind == 1) v = p * (fieldAt(P.F, P.ex, si, c) + fieldAt(P.F, P.ex, si, c + P.d1));
		else v = p * (fieldAt(P.F, P.ex, si, c) + fieldAt(P.F, P.ex, si, c + P.d1) + fieldAt(P.F, P.ex, si, c + P.d2) +
		              fieldAt(P.F, P.ex, si, c + P.d1 + P.d2));
	}
	P.acc[t] += v * P.re;
	P.acc[t + cells] += v * P.im;
}

extern "C" int alisgpu_slice_dft_create(alisgpu_world *w, const int box[6], alisgpu_slice_dft **out)
{
	bindWorld(w);
	if (!w || !box || !out || box[1] < box[0] || box[3] < box[2] || box[5] < box[4])
		return alisgpu__fail(ALISGPU_EINVAL, "slice_dft_create: bad argument");
	const size_t cells = (size_t)(1 + box[1] - box[0]) * (1 + box[3] - box[2]) * (1 + box[5] - box[4]);
	if (2 * cells >= (1u << 31)) return alisgpu__fail(ALISGPU_ERANGE, "slice_dft_create: box of %zu cells too large", cells);
	alisgpu_slice_dft *d = new alisgpu_slice_dft();
	d->w = w;
	d->i0 = box[0], d->i1 = box[1], d->j0 = box[2], d->j1 = box[3], d->k0 = box[4], d->k1 = box[5];
	cudaError_t e = alisgpu__mallocAsync(&d->acc, 2 * cells * sizeof(float));
	if (e == cudaSuccess) e = cudaMemsetAsync(d->acc, 0, 2 * cells * sizeof(float), gStream);
	if (e != cudaSuccess) {
		alisgpu__freeAsync(d->acc);
		delete d;
		return alisgpu__check(e, "slice_dft_create");
	}
	*out = d;
	return ALISGPU_OK;
}

extern "C" int alisgpu_slice_dft_add(alisgpu_slice_dft *d, int field, int m, int comp, int avg, const int sym[3], const float par[3],
                                     float re, float im)
{
	ALIS_BATCH_GUARD();
	if (d) bindWorld(d->w);
	if (!d || field < 0 || field > 1 || m < 0 || m > 1 || comp < 0 || comp > 2 || avg < 0 || avg > 1 || !sym || !par)
		return alisgpu__fail(ALISGPU_EINVAL, "slice_dft_add: bad argument");
	alisgpu_world *w = d->w;
	const alisgpu_geometry &g = w->g;
	const Layout &L = w->L;
	SliceDftParams P;
	memset(&P, 0, sizeof P);
	P.L = L;
	// the indices read, after mirroring, and one cell beyond: inside the halo'd grid
	const int lo[3] = { d->i0, d->j0, d->k0 }, hi[3] = { d->i1, d->j1, d->k1 };
	const int L0[3] = { L.i0, L.j0, L.k0 }, LN[3] = { L.ni, L.nj, L.nk };
	for (int a = 0; a < 3; a++) {
		P.sym[a] = sym[a] != 0, P.par[a] = par[a];
		int mn = lo[a], mx = hi[a];
		if (P.sym[a] && lo[a] < 0) {
			if (hi[a] < 0) mn = -hi[a], mx = -lo[a];
			else mn = 0, mx = std::max(hi[a], -lo[a]);
		}
		if (mn < L0[a] || mx + 1 >= L0[a] + LN[a]) return alisgpu__fail(ALISGPU_ERANGE, "slice_dft_add: box outside the grid");
	}
	if (m > g.complexField) {
		P.kind = -1;
	} else {
		P.F = field == 0 ? w->E[m][comp] : w->H[m][comp];
		P.ex = w->half ? halfRead(w, field) + comp * L.ni : 0;
		const long long st[3] = { L.si, L.sj, 1 };
		if (!avg) P.kind = 0, P.base = 1.0f;
		else if (field == 0) P.kind = 1, P.base = 0.5f, P.d1 = (int)st[comp];
		else {
			// H: the two axes other than its own, in the reference's order
			const int a1 = comp == 0 ? 1 : comp == 1 ? 2 : 0, a2 = comp == 0 ? 2 : comp == 1 ? 0 : 1;
			P.kind = 2, P.base = 0.25f, P.d1 = (int)st[a1], P.d2 = (int)st[a2];
		}
	}
	// E's upper halo (written by the deferred ghost copies) is read at the box's upper edge
	if (field == 0 && P.kind >= 0 && (d->i1 >= g.iMAX || d->j1 >= g.jMAX || d->k1 >= g.kMAX || P.sym[0] || P.sym[1] || P.sym[2])) {
		int rc = applyPendingGhosts(w);
		if (rc) return rc;
	}
	P.i0 = d->i0, P.j0 = d->j0, P.k0 = d->k0;
	P.ni = 1 + d->i1 - d->i0, P.nj = 1 + d->j1 - d->j0, P.nk = 1 + d->k1 - d->k0;
	P.re = re, P.im = im;
	P.acc = d->acc;
	const int cells = P.ni * P.nj * P.nk;
	int slot = alisgpu__prof_start();
	k_slice_dft<<<(unsigned)((cells + 255) / 256), 256, 0, gStream>>>(P);
	alisgpu__prof_stop(slot, ALISGPU_K_GATHER);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	return ALISGPU_OK;
}

extern "C" int alisgpu_slice_dft_download(alisgpu_slice_dft *d, float *F, float *G)
{
	ALIS_BATCH_GUARD();
	if (d) bindWorld(d->w);
	if (!d || !F || !G) return alisgpu__fail(ALISGPU_EINVAL, "slice_dft_download: bad argument");
	const size_t cells = (size_t)(1 + d->i1 - d->i0) * (1 + d->j1 - d->j0) * (1 + d->k1 - d->k0);
	ALIS_CUDA(cudaMemcpyAsync(F, d->acc, cells * sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaMemcpyAsync(G, d->acc + cells, cells * sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

extern "C" int alisgpu_slice_dft_destroy(alisgpu_slice_dft *d)
{
	if (d) bindWorld(d->w);
	if (!d) return ALISGPU_OK;
	cudaStreamSynchronize(gStream);
	alisgpu__freeAsync(d->acc);
	delete d;
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// Power absorbed by dispersive object n (reference src/output.c:359-435):
// J . E over the object's box with the reference's arithmetic in its
// order as one OpenMP thread runs it.  The three column sums along k of
// each (i, j) do not depend on the column's edge weights: one thread per
// column computes them, one thread then combines the columns in the
// reference's call order.
// ---------------------------------------------------------------------
struct AbsorbParams {
	Layout L;
	const float *E[3], *C[3];
	const signed char *exE[3];                // half storage (else null)
	DevObj o;
	int iMIN, iMAX, jMIN, jMAX, kMIN, kMAX;
	int i0, i1, j0, j1, k0, k1;               // box clipped to the world
	const float *dxE, *dxH, *dyE, *dyH, *dzE, *dzH;   // spacings indexed by index
	float *cols;                              // [columns][3]
	float *out;
};

// polarisation + conduction current density / eps of axis a at a cell of the box
__device__ __forceinline__ float objCurrent(const AbsorbParams &P, int a, int i, int j, int k, long long c)
{
	const DevObj &o = P.o;
	const int b = (i - o.i0) * (int)o.si + (j - o.j0) * (int)o.sj + (k - o.k0);
	float f = 0;
	if (o.a[a]) f = __fadd_rn(f, __fdiv_rn(__fmul_rn(__fmul_rn(2.0f, o.fill[a][b]), fieldAt(P.E[a], P.exE[a], P.L.si, c)), __fadd_rn(1.0f, __fdiv_rn(1.0f, o.a[a]))));
	for (int p = 0; p < o.NK; p++) f = __fadd_rn(f, o.J[0][p][a][b]);
	return __fdiv_rn(f, P.C[a][c]);
}

__global__ void k_absorb_columns(const AbsorbParams P)
{
	const int nj = 1 + P.j1 - P.j0;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (1 + P.i1 - P.i0) * nj) return;
	const int i = P.i0 + t / nj, j = P.j0 + t % nj;
	float xs = 0, ys = 0, zs = 0;
	for (int k = P.k0; k <= P.k1; k++) {
		const long long c = P.L.at(i, j, k);
		if (P.C[0][c] != 0) xs = __fadd_rn(xs, __fmul_rn(__fmul_rn(P.dzE[k], fieldAt(P.E[0], P.exE[0], P.L.si, c)), objCurrent(P, 0, i, j, k, c)));
		if (P.C[1][c] != 0) ys = __fadd_rn(ys, __fmul_rn(__fmul_rn(P.dzE[k], fieldAt(P.E[1], P.exE[1], P.L.si, c)), objCurrent(P, 1, i, j, k, c)));
		if (P.C[2][c] != 0) zs = __fadd_rn(zs, __fmul_rn(__fmul_rn(P.dzH[k], fieldAt(P.E[2], P.exE[2], P.L.si, c)), objCurrent(P, 2, i, j, k, c)));
	}
	// half weights where the box meets the world's k edges; `* 0.5` is a
	// double product, the difference rounds back to float
	auto halfOff = [](float s, float v) { return __double2float_rn(__dsub_rn((double)s, (double)v * 0.5)); };
	if (P.k0 == P.kMIN) {
		const int k = P.kMIN;
		const long long c = P.L.at(i, j, k);
		if (P.C[0][c] != 0) xs = halfOff(xs, __fmul_rn(__fmul_rn(P.dzE[k], fieldAt(P.E[0], P.exE[0], P.L.si, c)), objCurrent(P, 0, i, j, k, c)));
		if (P.C[1][c] != 0) ys = halfOff(ys, __fmul_rn(__fmul_rn(P.dzE[k], fieldAt(P.E[1], P.exE[1], P.L.si, c)), objCurrent(P, 1, i, j, k, c)));
		if (P.C[2][c] != 0) zs = __fsub_rn(zs, __fmul_rn(__fmul_rn(P.dzH[k], fieldAt(P.E[2], P.exE[2], P.L.si, c)), objCurrent(P, 2, i, j, k, c)));
	}
	if (P.k1 == P.kMAX) {
		const int k = P.kMAX;
		const long long c = P.L.at(i, j, k);
		if (P.C[0][c] != 0) xs = halfOff(xs, __fmul_rn(__fmul_rn(P.dzE[k], fieldAt(P.E[0], P.exE[0], P.L.si, c)), objCurrent(P, 0, i, j, k, c)));
		if (P.C[1][c] != 0) ys = halfOff(ys, __fmul_rn(__fmul_rn(P.dzE[k], fieldAt(P.E[1], P.exE[1], P.L.si, c)), objCurrent(P, 1, i, j, k, c)));
	}
	P.cols[3 * t] = xs, P.cols[3 * t + 1] = ys, P.cols[3 * t + 2] = zs;
}

__device__ __forceinline__ float absorbColumn(const AbsorbParams &P, const float *cols, int i, int j, float x, float y, float z)
{
	const int t = (i - P.i0) * (1 + P.j1 - P.j0) + (j - P.j0);
	const float xs = cols[3 * t], ys = cols[3 * t + 1], zs = cols[3 * t + 2];
	float S = 0;
	S = __fadd_rn(S, __fmul_rn(__fmul_rn(__fmul_rn(x, xs), P.dxH[i]), P.dyE[j]));
	S = __fadd_rn(S, __fmul_rn(__fmul_rn(__fmul_rn(y, ys), P.dxE[i]), P.dyH[j]));
	S = __fadd_rn(S, __fmul_rn(__fmul_rn(__fmul_rn(z, zs), P.dxE[i]), P.dyE[j]));
	return S;
}

__global__ void __launch_bounds__(256) k_absorb_total(const AbsorbParams P)
{
	// the column sums staged in shared memory, then added in order
	extern __shared__ float cols[];
	const int ncols = 3 * (1 + P.i1 - P.i0) * (1 + P.j1 - P.j0);
	for (int q = threadIdx.x; q < ncols; q += blockDim.x) cols[q] = P.cols[q];
	__syncthreads();
	if (threadIdx.x || blockIdx.x) return;
	float Sum = 0;
	for (int i = P.i0; i <= P.i1; i++) {
		for (int j = P.j0; j <= P.j1; j++) Sum = __fadd_rn(Sum, absorbColumn(P, cols, i, j, 1, 1, 1));
		if (P.j0 == P.jMIN) Sum = __fadd_rn(Sum, absorbColumn(P, cols, i, P.jMIN, -0.5f, -1, -0.5f));
		if (P.j1 == P.jMAX) Sum = __fadd_rn(Sum, absorbColumn(P, cols, i, P.jMAX, -0.5f, 0, -0.5f));
	}
	if (P.i0 == P.iMIN) {
		float part = 0;
		for (int j = P.j0; j <= P.j1; j++) part = __fadd_rn(part, absorbColumn(P, cols, P.iMIN, j, -1, -0.5f, -0.5f));
		Sum = __fadd_rn(Sum, part);
		if (P.j0 == P.jMIN) Sum = __fadd_rn(Sum, absorbColumn(P, cols, P.iMIN, P.jMIN, 0.5f, 0.5f, 0.25f));
		if (P.j1 == P.jMAX) Sum = __fadd_rn(Sum, absorbColumn(P, cols, P.iMIN, P.jMAX, 0.5f, 0.0f, 0.25f));
	}
	if (P.i1 == P.iMAX) {
		float part = 0;
		for (int j = P.j0; j <= P.j1; j++) part = __fadd_rn(part, absorbColumn(P, cols, P.iMAX, j, 0, -0.5f, -0.5f));
		Sum = __fadd_rn(Sum, part);
		if (P.j0 == P.jMIN) Sum = __fadd_rn(Sum, absorbColumn(P, cols, P.iMAX, P.jMIN, 0.0f, 0.5f, 0.25f));
		if (P.j1 == P.jMAX) Sum = __fadd_rn(Sum, absorbColumn(P, cols, P.iMAX, P.jMAX, 0.0f, 0.0f, 0.25f));
	}
	P.out[0] = Sum;
}

extern "C" int alisgpu_object_absorption(alisgpu_world *w, int n, float *out)
{
	ALIS_BATCH_GUARD();
	bindWorld(w);
	if (!w || !out || n < 0 || n >= (int)w->objs.size()) return alisgpu__fail(ALISGPU_EINVAL, "object_absorption: bad argument");
	if (!w->sp[0][0]) return alisgpu__fail(ALISGPU_EINVAL, "object_absorption: spacing tables not set");
	if (!w->C[0]) return alisgpu__fail(ALISGPU_EINVAL, "object_absorption: world has no eps maps");
	const alisgpu_geometry &g = w->g;
	AbsorbParams P;
	memset(&P, 0, sizeof P);
	P.L = w->L;
	for (int c = 0; c < 3; c++) P.E[c] = w->E[0][c], P.C[c] = w->C[c];
	if (w->half)
		for (int c = 0; c < 3; c++) P.exE[c] = halfRead(w, 0) + c * w->L.ni;
	P.o = w->objs[n];
	P.iMIN = g.iMIN, P.iMAX = g.iMAX, P.jMIN = g.jMIN, P.jMAX = g.jMAX, P.kMIN = g.kMIN, P.kMAX = g.kMAX;
	P.i0 = std::max(g.iMIN, P.o.i0), P.i1 = std::min(g.iMAX, P.o.i1);
	P.j0 = std::max(g.jMIN, P.o.j0), P.j1 = std::min(g.jMAX, P.o.j1);
	P.k0 = std::max(g.kMIN, P.o.k0), P.k1 = std::min(g.kMAX, P.o.k1);
	if (P.i1 < P.i0 || P.j1 < P.j0 || P.k1 < P.k0) { *out = 0; return ALISGPU_OK; }
	const long long cols = (long long)(1 + P.i1 - P.i0) * (1 + P.j1 - P.j0);
	const size_t floats = 3 * cols + 1;
	if (floats > w->planeTabFloats) {
		ALIS_CUDA(cudaStreamSynchronize(gStream));
		if (w->planeTab) alisgpu__freeAsync(w->planeTab);
		w->planeTab = 0, w->planeTabFloats = 0;
		ALIS_CUDA(alisgpu__mallocAsync(&w->planeTab, floats * sizeof(float)));
		w->planeTabFloats = floats;
	}
	float *t = w->planeTab;
	P.dxE = w->sp[0][0] - g.iMIN, P.dyE = w->sp[0][1] - g.jMIN, P.dzE = w->sp[0][2] - g.kMIN;
	P.dxH = w->sp[1][0] - g.iMIN, P.dyH = w->sp[1][1] - g.jMIN, P.dzH = w->sp[1][2] - g.kMIN;
	P.cols = t, t += 3 * cols;
	P.out = t;
	int slot = alisgpu__prof_start();
	k_absorb_columns<<<(unsigned)((cols + 127) / 128), 128, 0, gStream>>>(P);
	const size_t smem = 3 * (size_t)cols * sizeof(float);
	if (smem <= 48 * 1024) k_absorb_total<<<1, 256, smem, gStream>>>(P);
	else {
		ALIS_CUDA(cudaFuncSetAttribute(k_absorb_total, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
		if (smem > 200 * 1024) return alisgpu__fail(ALISGPU_ERANGE, "object_absorption: %lld columns too many", cols);
		k_absorb_total<<<1, 256, smem, gStream>>>(P);
	}
	alisgpu__prof_stop(slot, ALISGPU_K_FLUX);
	alisgpu__count_launch();
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	ALIS_CUDA(cudaMemcpyAsync(out, P.out, sizeof(float), cudaMemcpyDeviceToHost, gStream));
	ALIS_CUDA(cudaStreamSynchronize(gStream));
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// Second-order (chi2) coupling of a signal world to pump fields over the
// box of dispersive object n (reference src/update.c:343-411): E_a +=
// 2 Alt d C_a fill_a (G1_b G2_c) for the 9 terms of each axis a, with the
// pump components averaged onto the a-grid (0.25 x a 4-cell sum, a double
// product) where they sit elsewhere.  One launch per axis: within it a
// cell takes its 9 terms in the reference's order, and a later axis reads
// the finished earlier one (as the reference's term-by-term sweeps do,
// also when the signal world is its own pump).
// ---------------------------------------------------------------------
struct TwmParams {
	Layout L;
	float *F[3];
	const float *G1[3], *G2[3];
	const float *C[3];
	const float *fill[3];
	int oi0, oj0, ok0;                     // object box origin (fill indexing)
	long long osj, osi;
	int i0, i1, j0, j1, k0, k1;            // coupled range
	float coef[6];                         // 2 Alt d[a][q] per term kind
	unsigned active;                       // d[a][q] non-zero
};

// component c of a pump field on the grid of axis a: the cell itself
// (float) or the reference's 4-cell average (double)
__device__ __forceinline__ double pumpAt(const float *const G[3], const Layout &L, int c, int a, int i, int j, int k, bool &isDouble)
{
	if (c == a) { isDouble = false; return (double)G[c][L.at(i, j, k)]; }
	isDouble = true;
	int o[4][3];
	if (a == 0 && c == 1) { int t[4][3] = {{0,0,0},{-1,0,0},{0,1,0},{-1,1,0}}; memcpy(o, t, sizeof t); }
	else if (a == 0) { int t[4][3] = {{0,0,0},{-1,0,0},{0,0,1},{-1,0,1}}; memcpy(o, t, sizeof t); }
	else if (a == 1 && c == 2) { int t[4][3] = {{0,0,0},{0,-1,0},{0,0,1},{0,-1,1}}; memcpy(o, t, sizeof t); }
	else if (a == 1) { int t[4][3] = {{0,0,0},{0,-1,0},{1,0,0},{1,-1,0}}; memcpy(o, t, sizeof t); }
	else if (c == 0) { int t[4][3] = {{0,0,0},{0,0,-1},{1,0,0},{1,0,-1}}; memcpy(o, t, sizeof t); }
	else { int t[4][3] = {{0,0,0},{0,0,-1},{0,1,0},{0,1,-1}}; memcpy(o, t, sizeof t); }
	float sum = G[c][L.at(i + o[0][0], j + o[0][1], k + o[0][2])];
	for (int q = 1; q < 4; q++) sum = __fadd_rn(sum, G[c][L.at(i + o[q][0], j + o[q][1], k + o[q][2])]);
	return 0.25 * (double)sum;
}

template <int A>
__global__ void k_twm(const TwmParams P)
{
	const int nj = 1 + P.j1 - P.j0, nk = 1 + P.k1 - P.k0;
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long long)(1 + P.i1 - P.i0) * nj * nk) return;
	const int i = P.i0 + (int)(t / ((long long)nj * nk)), j = P.j0 + (int)((t / nk) % nj), k = P.k0 + (int)(t % nk);
	const long long c = P.L.at(i, j, k);
	const long long b = (long long)(i - P.oi0) * P.osi + (long long)(j - P.oj0) * P.osj + (k - P.ok0);
	// the terms of axis A: (d index, G1 component, G2 component)
	const int T[9][3] = {{0,0,0},{1,1,1},{2,2,2},{3,1,2},{3,2,1},{4,2,0},{4,0,2},{5,0,1},{5,1,0}};
	float f = P.F[A][c];
	const float cv = P.C[A][c], fl = P.fill[A][b];
	// a pump that is the signal itself reads this cell's running value
	const bool self1 = P.G1[A] == P.F[A], self2 = P.G2[A] == P.F[A];
#pragma unroll
	for (int q = 0; q < 9; q++) {
		const int di = T[q][0];
		if (!((P.active >> di) & 1u)) continue;
		bool d1, d2;
		double v1 = pumpAt(P.G1, P.L, T[q][1], A, i, j, k, d1);
		double v2 = pumpAt(P.G2, P.L, T[q][2], A, i, j, k, d2);
		if (T[q][1] == A && self1) v1 = (double)f;
		if (T[q][2] == A && self2) v2 = (double)f;
		const float lead = __fmul_rn(__fmul_rn(P.coef[di], cv), fl);
		if (!d1 && !d2) f = __fadd_rn(f, __fmul_rn(lead, __fmul_rn((float)v1, (float)v2)));
		else f = __double2float_rn(__dadd_rn((double)f, __dmul_rn((double)lead, __dmul_rn(v1, v2))));
	}
	P.F[A][c] = f;
}

// Order the signal world's stream after (before = false) or the pump
// world's stream before (before = true) the other when they are in
// different stream groups.
static int crossGroup(const alisgpu_world *ws, const alisgpu_world *wp, bool pumpFirst)
{
	StreamGroup *gs = ws->group ? ws->group : &gDefaultGroup, *gp = wp->group ? wp->group : &gDefaultGroup;
	if (gs == gp) return ALISGPU_OK;
	StreamGroup *from = pumpFirst ? gp : gs, *to = pumpFirst ? gs : gp;
	StreamGroup *keep = gGroup;
	gGroup = from;
	fullJoin();
	ALIS_CUDA(cudaEventRecord(from->evJoin, from->main));
	ALIS_CUDA(cudaStreamWaitEvent(to->main, from->evJoin, 0));
	gGroup = keep;
	return ALISGPU_OK;
}

extern "C" int alisgpu_nonlinear_twm(alisgpu_world *ws, const alisgpu_world *wp1, const alisgpu_world *wp2, int n, int m,
                                     const float d[3][6], float Alt)
{
	ALIS_BATCH_GUARD();
	if (!ws || !wp1 || !wp2 || !d || n < 0 || n >= (int)ws->objs.size() || m < 0 || m > ws->g.complexField ||
	    m > wp1->g.complexField || m > wp2->g.complexField)
		return alisgpu__fail(ALISGPU_EINVAL, "nonlinear_twm: bad argument");
	if (ws->half || wp1->half || wp2->half) return alisgpu__fail(ALISGPU_ENOTSUP, "nonlinear_twm: a world stores half values");
	// the pumps' fields are read on the signal world's stream
	int rc = crossGroup(ws, wp1, true);
	if (!rc) rc = crossGroup(ws, wp2, true);
	if (rc) return rc;
	bindWorld(ws);
	fullJoin();
	if (!ws->C[0]) return alisgpu__fail(ALISGPU_EINVAL, "nonlinear_twm: signal world has no eps maps");
	if (memcmp(&ws->L, &wp1->L, sizeof(Layout)) || memcmp(&ws->L, &wp2->L, sizeof(Layout)))
		return alisgpu__fail(ALISGPU_EINVAL, "nonlinear_twm: pump and signal worlds differ in grid");
	const DevObj &o = ws->objs[n];
	TwmParams P;
	memset(&P, 0, sizeof P);
	P.L = ws->L;
	for (int c = 0; c < 3; c++) {
		P.F[c] = ws->E[m][c], P.G1[c] = wp1->E[m][c], P.G2[c] = wp2->E[m][c];
		P.C[c] = ws->C[c], P.fill[c] = o.fill[c];
	}
	P.oi0 = o.i0, P.oj0 = o.j0, P.ok0 = o.k0, P.osj = o.sj, P.osi = o.si;
	// the reference couples [box min, box max - 1] on every axis
	P.i0 = o.i0, P.i1 = o.i1 - 1, P.j0 = o.j0, P.j1 = o.j1 - 1, P.k0 = o.k0, P.k1 = o.k1 - 1;
	if (P.i1 < P.i0 || P.j1 < P.j0 || P.k1 < P.k0) return ALISGPU_OK;
	const long long cells = (long long)(1 + P.i1 - P.i0) * (1 + P.j1 - P.j0) * (1 + P.k1 - P.k0);
	for (int a = 0; a < 3; a++) {
		P.active = 0;
		for (int q = 0; q < 6; q++) {
			P.coef[q] = (2.0f * Alt) * d[a][q];
			if (d[a][q]) P.active |= 1u << q;
		}
		if (!P.active) continue;
		int slot = alisgpu__prof_start();
		const unsigned blocks = (unsigned)((cells + 255) / 256);
		if (a == 0) k_twm<0><<<blocks, 256, 0, gStream>>>(P);
		else if (a == 1) k_twm<1><<<blocks, 256, 0, gStream>>>(P);
		else k_twm<2><<<blocks, 256, 0, gStream>>>(P);
		alisgpu__prof_stop(slot, ALISGPU_K_STEP_AUX);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}
	// the pumps' next steps overwrite what was read
	rc = crossGroup(ws, wp1, false);
	if (!rc) rc = crossGroup(ws, wp2, false);
	bindWorld(ws);
	return rc;
}

// field pointers of set m for the phaser gather kernel
// The stream of a phaser gather on world w that reads H over the boxes
// box[n] (i0, i1, j0, j1, k0, k1, each already widened by the cells the
// gather reads): the side stream, after w's last H cell updates, when
// nothing has changed world data since that half step's ghost launch and
// none of its ghost copies writes H there -- the gather then runs beside
// the ghost copies; else the main stream.  gatherEnd joins the streams.
extern "C" cudaStream_t alisgpu__gather_begin(alisgpu_world *w, const int (*box)[6], int n)
{
	if (gProfOn || !w || !w->hRecorded || gOps != w->hOps) return gStream;
	for (const alisgpu_ghost_copy &c : w->hGhosts) {
		const int W[6] = { c.i0, c.i1, c.j0, c.j1, c.k0, c.k1 };
		for (int q = 0; q < n; q++) if (boxesMeet(W, box[q])) return gStream;
	}
	if (cudaStreamWaitEvent(gGather, w->evHCells, 0) != cudaSuccess) return gStream;
	return gGather;
}

extern "C" int alisgpu__gather_end(alisgpu_world *w, cudaStream_t st)
{
	if (st == gStream) return ALISGPU_OK;
	ALIS_CUDA(cudaEventRecord(gEvGatherDone, gGather));
	ALIS_CUDA(cudaStreamWaitEvent(gStream, gEvGatherDone, 0));
	// a gather changes no world data: a further phaser may also run beside
	w->hOps = gOps;
	return ALISGPU_OK;
}

extern "C" int alisgpu__world_fields(alisgpu_world *w, int m, const float **E, const float **H, Layout *L)
{
	if (!w || m < 0 || m > w->g.complexField) return alisgpu__fail(ALISGPU_EINVAL, "world_fields: bad argument");
	for (int c = 0; c < 3; c++) E[c] = w->E[m][c], H[c] = w->H[m][c];
	*L = w->L;
	return ALISGPU_OK;
}

// the exponents E and H are read with now (null for float storage)
extern "C" void alisgpu__world_half(const alisgpu_world *w, const signed char **exE, const signed char **exH)
{
	*exE = w && w->half ? halfRead(w, 0) : 0;
	*exH = w && w->half ? halfRead(w, 1) : 0;
}
