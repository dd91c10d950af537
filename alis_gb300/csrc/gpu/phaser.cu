// phaser.cu -- time-blocked running DFT on phaser faces.
//
// The reference adds, every step and for every frequency f,
//   A_E += exp(2 pi i f t_E) * E          (float complex)
//   A_H += exp(2 pi i f t_H) * (H + H') * 0.5
// to four tangential accumulators per face cell (src/phaser.c:83-110):
// 64 B of accumulator traffic per face cell, frequency and step.  Here a
// gather kernel copies the face samples of each step (E1, E2, H1 + H1',
// H2 + H2') into a ring buffer on the device; every `ring` steps a flush
// kernel loads each accumulator once, applies the buffered steps in time
// order with exactly the reference's float operations, and stores it
// once.  Results are bit-identical to the per-step reference sums, with
// accumulator traffic divided by the ring length.
//
// The H term rounds as the reference's double expression
// fl(A + (p * Hs) * 0.5): for any float p*Hs whose half is exact the float
// add gives the same result (double rounding is innocuous for float
// operands); when halving is inexact (p*Hs subnormal) the add is done in
// double.  Optional Kahan compensation keeps a second accumulator.
#include <cstring>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "batch.cuh"

struct alisgpu_phaser {
	alisgpu_world *w;
	int nfreq, nface, ring, kahan;
	std::vector<alisgpu_face> faces;
	std::vector<long long> faceStart;     // cell offset of each face
	long long cells;                      // total face cells
	float *buf;                           // [ring][cells][4]
	float2 *acc;                          // [nfreq][cells][4]
	float2 *comp;                         // Kahan compensation (or null)
	float2 *phase;                        // [ring][nfreq][2] (E, H)
	std::vector<float2> hostPhase;        // phases of buffered steps
	// pinned staging of the phases, two in turn, so that their upload is
	// asynchronous (a pageable copy may wait for the stream to drain)
	float2 *pinned[2];
	cudaEvent_t pinnedFree[2];
	size_t pinnedCap;
	int pinnedNext;
	int *faceInfo;                        // per face: axis, box
	int used;                             // buffered steps
	float *fluxTab;                       // spacing tables and sums of the flux kernels
	size_t fluxTabBytes;
};

// world layout and field pointers needed by the gather kernel
struct GatherParams {
	Layout L;
	const float *E[3], *H[3];
	int nface;
	long long start[7];
	int box[6][7];                        // axis, i0, i1, j0, j1, k0, k1
	float *out;                           // ring slot
	const signed char *exE, *exH;         // half storage: the exponents per (component, plane) (else null)
};

extern "C" int alisgpu__world_fields(alisgpu_world *w, int m, const float **E, const float **H, Layout *L);
extern "C" void alisgpu__world_half(const alisgpu_world *w, const signed char **exE, const signed char **exH);
extern "C" cudaStream_t alisgpu__gather_begin(alisgpu_world *w, const int (*box)[6], int n);
extern "C" void alisgpu__bind(alisgpu_world *w);
extern "C" int alisgpu__gather_end(alisgpu_world *w, cudaStream_t st);

__device__ __forceinline__ void gatherCell(const GatherParams &P, long long t)
{
	if (t >= P.start[P.nface]) return;
	int f = 0;
	while (t >= P.start[f + 1]) f++;
	const int *b = P.box[f];
	long long r = t - P.start[f];
	int nk = 1 + b[6] - b[5], nj = 1 + b[4] - b[3];
	int k = b[5] + (int)(r % nk), j = b[3] + (int)((r / nk) % nj), i = b[1] + (int)(r / ((long long)nk * nj));
	int axis = b[0];
	// tangential components of the face: x (y, z), y (z, x), z (x, y)
	int c1 = axis == 0 ? 1 : axis == 1 ? 2 : 0;
	int c2 = axis == 0 ? 2 : axis == 1 ? 0 : 1;
	long long c = P.L.at(i, j, k);
	long long n = c + (axis == 0 ? P.L.si : axis == 1 ? P.L.sj : 1);
	float4 v;
	if (P.exE) {
		// a half world: each sample times its plane's power of two
		const int ni = P.L.ni, pl = i - P.L.i0, pn = pl + (axis == 0);
		v.x = halfAt(P.E[c1], c, pow2f(P.exE[c1 * ni + pl]));
		v.y = halfAt(P.E[c2], c, pow2f(P.exE[c2 * ni + pl]));
		v.z = halfAt(P.H[c1], c, pow2f(P.exH[c1 * ni + pl])) + halfAt(P.H[c1], n, pow2f(P.exH[c1 * ni + pn]));
		v.w = halfAt(P.H[c2], c, pow2f(P.exH[c2 * ni + pl])) + halfAt(P.H[c2], n, pow2f(P.exH[c2 * ni + pn]));
	} else {
		v.x = P.E[c1][c];
		v.y = P.E[c2][c];
		v.z = P.H[c1][c] + P.H[c1][n];
		v.w = P.H[c2][c] + P.H[c2][n];
	}
	reinterpret_cast<float4 *>(P.out)[t] = v;
}

__global__ void k_phaser_gather(const GatherParams P)
{
	gatherCell(P, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// fl(a + p * 0.5) with the rounding of the reference's double expression
// (float)((double)a + (double)p * 0.5): p * 0.5 is exact in double and
// the double sum of two floats rounds innocuously to float, so the result
// is the exactly rounded a + p/2 -- which is what one fused multiply-add
// computes, including when p/2 is subnormal.
__device__ __forceinline__ float addHalf(float a, float p)
{
	return __fmaf_rn(p, 0.5f, a);
}

#define FLUSH_THREADS 128
#define FLUSH_FREQ 8
#define FLUSH_SUB 8                              // ring steps per compensated add

// the phase factors of frequency group by (FLUSH_FREQ frequencies) for
// every ring step, into shared memory: [steps][FLUSH_FREQ][E, H]
__device__ __forceinline__ void flushPhases(const float2 *phase, int nfreq, int steps, int by, float2 *sph)
{
	const int f0 = by * FLUSH_FREQ;
	const int nf = min(FLUSH_FREQ, nfreq - f0);
	for (int q = threadIdx.x; q < steps * FLUSH_FREQ * 2; q += blockDim.x) {
		int s = q / (FLUSH_FREQ * 2), r = q % (FLUSH_FREQ * 2), ff = r / 2, h = r % 2;
		sph[q] = ff < nf ? phase[((long long)s * nfreq + f0 + ff) * 2 + h] : make_float2(0, 0);
	}
}

// one (face cell, component) t over frequency group by: ring step s of
// the cell is buf[s * xs]
template <bool KAHAN>
__device__ __forceinline__ void flushCell(const float *buf, long long xs, float2 *acc, float2 *comp, long long n4,
                                          int nfreq, int steps, long long t, int by, const float2 *sph)
{
	const int f0 = by * FLUSH_FREQ;
	const int nf = min(FLUSH_FREQ, nfreq - f0);
	const bool isH = (t & 3) >= 2;
	float2 a[FLUSH_FREQ], cc[FLUSH_FREQ];
#pragma unroll
	for (int ff = 0; ff < FLUSH_FREQ; ff++) {
		a[ff] = cc[ff] = make_float2(0, 0);
		if (ff < nf) {
			a[ff] = acc[(long long)(f0 + ff) * n4 + t];
			if (KAHAN) cc[ff] = comp[(long long)(f0 + ff) * n4 + t];
		}
	}
	if (!KAHAN) {
		// the reference's sums, term by term in its rounding
		for (int s = 0; s < steps; s++) {
			const float x = buf[(long long)s * xs];
#pragma unroll
			for (int ff = 0; ff < FLUSH_FREQ; ff++) {
				if (ff >= nf) break;
				const float2 p = sph[(s * FLUSH_FREQ + ff) * 2 + (isH ? 1 : 0)];
				const float pr = p.x * x, pi = p.y * x;
				if (isH) a[ff].x = addHalf(a[ff].x, pr), a[ff].y = addHalf(a[ff].y, pi);
				else a[ff].x = a[ff].x + pr, a[ff].y = a[ff].y + pi;
			}
		}
	} else {
		// compensated: the terms of FLUSH_SUB steps summed with fused
		// multiply-adds, then one Kahan step (y = part - c; s' = s + y;
		// c = (s' - s) - y) per frequency
		for (int s0 = 0; s0 < steps; s0 += FLUSH_SUB) {
			float2 part[FLUSH_FREQ];
#pragma unroll
			for (int ff = 0; ff < FLUSH_FREQ; ff++) part[ff] = make_float2(0, 0);
			const int s1 = min(s0 + FLUSH_SUB, steps);
			for (int s = s0; s < s1; s++) {
				const float x = isH ? 0.5f * buf[(long long)s * xs] : buf[(long long)s * xs];
#pragma unroll
				for (int ff = 0; ff < FLUSH_FREQ; ff++) {
					const float2 p = sph[(s * FLUSH_FREQ + ff) * 2 + (isH ? 1 : 0)];
					part[ff].x = __fmaf_rn(p.x, x, part[ff].x), part[ff].y = __fmaf_rn(p.y, x, part[ff].y);
				}
			}
#pragma unroll
			for (int ff = 0; ff < FLUSH_FREQ; ff++) {
				const float yr = __fsub_rn(part[ff].x, cc[ff].x), yi = __fsub_rn(part[ff].y, cc[ff].y);
				const float sr = __fadd_rn(a[ff].x, yr), sI = __fadd_rn(a[ff].y, yi);
				cc[ff].x = __fsub_rn(__fsub_rn(sr, a[ff].x), yr), cc[ff].y = __fsub_rn(__fsub_rn(sI, a[ff].y), yi);
				a[ff].x = sr, a[ff].y = sI;
			}
		}
	}
#pragma unroll
	for (int ff = 0; ff < FLUSH_FREQ; ff++) {
		if (ff < nf) {
			acc[(long long)(f0 + ff) * n4 + t] = a[ff];
			if (KAHAN) comp[(long long)(f0 + ff) * n4 + t] = cc[ff];
		}
	}
}

// thread = one (face cell, component) of cell block bx; frequency group by
template <bool KAHAN>
__device__ __forceinline__ void flushBlock(const float *buf, float2 *acc, float2 *comp, const float2 *phase,
                                           long long n4, int nfreq, int steps, long long bx, int by, float2 *sph)
{
	flushPhases(phase, nfreq, steps, by, sph);
	__syncthreads();
	const long long t = bx * blockDim.x + threadIdx.x;
	if (t < n4) flushCell<KAHAN>(buf + t, n4, acc, comp, n4, nfreq, steps, t, by, sph);
}

template <bool KAHAN>
__global__ void __launch_bounds__(FLUSH_THREADS) k_phaser_flush(const float *buf, float2 *acc, float2 *comp, const float2 *phase,
                                                                long long n4, int nfreq, int steps)
{
	extern __shared__ float2 sph[];                 // [steps][FLUSH_FREQ][2]
	flushBlock<KAHAN>(buf, acc, comp, phase, n4, nfreq, steps, blockIdx.x, blockIdx.y, sph);
}

// The flush with the block's ring entries staged once: each block reads
// the ring steps of its FLUSH_THREADS (cell, component) pairs into shared
// memory and runs every frequency group from there, so the ring is read
// from memory once instead of once per group.  Each accumulator sums the
// same terms in the same order as k_phaser_flush.
template <bool KAHAN>
__global__ void __launch_bounds__(FLUSH_THREADS) k_phaser_flush_staged(const float *buf, float2 *acc, float2 *comp,
                                                                       const float2 *phase, long long n4, int nfreq, int steps)
{
	extern __shared__ float2 sph[];                 // [steps][FLUSH_FREQ][2], then the ring [steps][FLUSH_THREADS]
	float *ring = (float *)(sph + steps * FLUSH_FREQ * 2);
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	for (int st = 0; st < steps; st++) ring[st * blockDim.x + threadIdx.x] = t < n4 ? buf[(long long)st * n4 + t] : 0.0f;
	const int groups = (nfreq + FLUSH_FREQ - 1) / FLUSH_FREQ;
	for (int by = 0; by < groups; by++) {
		__syncthreads();                            // the previous group's phases are no longer read
		flushPhases(phase, nfreq, steps, by, sph);
		__syncthreads();
		if (t < n4) flushCell<KAHAN>(ring + threadIdx.x, blockDim.x, acc, comp, n4, nfreq, steps, t, by, sph);
	}
}

// ---- batched phaser work (batch.cuh): every recorded phaser's flush in
// one launch, then every phaser's gather in one launch ----
struct FlushItem {
	const float *buf;
	float2 *acc, *comp;
	const float2 *phase;
	long long n4;
	int nfreq, steps, kahan;
	int bx, blocks;                       // cell blocks; blocks of the item (bx x frequency groups)
	int start;                            // its first block in the launch
};
struct GatherItem {
	const GatherParams *G;
	long long start;                      // its first thread in the launch
};

__global__ void __launch_bounds__(FLUSH_THREADS) k_phaser_flush_batch(const FlushItem *T, int n)
{
	extern __shared__ float2 sph[];
	int lo = 0, hi = n - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (T[mid].start <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
	}
	const FlushItem &F = T[lo];
	const int b = (int)blockIdx.x - F.start;
	if (F.kahan) flushBlock<true>(F.buf, F.acc, F.comp, F.phase, F.n4, F.nfreq, F.steps, b % F.bx, b / F.bx, sph);
	else flushBlock<false>(F.buf, F.acc, F.comp, F.phase, F.n4, F.nfreq, F.steps, b % F.bx, b / F.bx, sph);
}

__global__ void k_phaser_gather_batch(const GatherItem *T, int n, long long total)
{
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= total) return;
	int lo = 0, hi = n - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (T[mid].start <= t) lo = mid; else hi = mid - 1;
	}
	gatherCell(*T[lo].G, t - T[lo].start);
}

extern "C" int alisgpu_phaser_create(alisgpu_world *w, int nfreq, int nface, const alisgpu_face *faces, int ring, int kahan, alisgpu_phaser **out)
{
	alisgpu__bind(w);
	if (!w || nfreq <= 0 || nface < 0 || nface > 6 || (nface && !faces) || !out || ring <= 0)
		return alisgpu__fail(ALISGPU_EINVAL, "phaser_create: bad argument");
	alisgpu_phaser *p = new alisgpu_phaser();
	p->w = w, p->nfreq = nfreq, p->nface = nface, p->ring = ring, p->kahan = kahan;
	p->cells = 0;
	for (int f = 0; f < nface; f++) {
		const alisgpu_face &a = faces[f];
		p->faces.push_back(a);
		p->faceStart.push_back(p->cells);
		p->cells += (long long)(1 + a.i1 - a.i0) * (1 + a.j1 - a.j0) * (1 + a.k1 - a.k0);
	}
	p->faceStart.push_back(p->cells);
	long long n4 = p->cells * 4;
	cudaStream_t st = alisgpu__stream();
	if (p->cells) {
		ALIS_CUDA(alisgpu__mallocAsync(&p->buf, (size_t)ring * n4 * sizeof(float)));
		ALIS_CUDA(alisgpu__mallocAsync(&p->acc, (size_t)nfreq * n4 * sizeof(float2)));
		ALIS_CUDA(cudaMemsetAsync(p->acc, 0, (size_t)nfreq * n4 * sizeof(float2), st));
		if (kahan) {
			ALIS_CUDA(alisgpu__mallocAsync(&p->comp, (size_t)nfreq * n4 * sizeof(float2)));
			ALIS_CUDA(cudaMemsetAsync(p->comp, 0, (size_t)nfreq * n4 * sizeof(float2), st));
		}
	}
	ALIS_CUDA(alisgpu__mallocAsync(&p->phase, (size_t)ring * nfreq * 2 * sizeof(float2)));
	p->used = 0;
	*out = p;
	return ALISGPU_OK;
}

// Pinned staging buffers outlive their phasers: freeing pinned memory
// waits for the whole device, which a served loop of many worlds avoids.
static std::vector<std::pair<float2 *, size_t>> gPinnedSpare;
static std::mutex gPinnedLock;

static float2 *pinnedTake(size_t n)
{
	std::lock_guard<std::mutex> lock(gPinnedLock);
	for (size_t q = 0; q < gPinnedSpare.size(); q++)
		if (gPinnedSpare[q].second >= n) {
			float2 *b = gPinnedSpare[q].first;
			gPinnedSpare.erase(gPinnedSpare.begin() + q);
			return b;
		}
	float2 *b = 0;
	return cudaMallocHost(&b, n * sizeof(float2)) == cudaSuccess ? b : 0;
}

static void pinnedRelease(float2 *b, size_t n)
{
	std::lock_guard<std::mutex> lock(gPinnedLock);
	if (b) gPinnedSpare.push_back(std::make_pair(b, n));
}

extern "C" int alisgpu_phaser_destroy(alisgpu_phaser *p)
{
	ALIS_BATCH_GUARD();
	if (p) alisgpu__bind(p->w);
	if (!p) return ALISGPU_OK;
	cudaStreamSynchronize(alisgpu__stream());
	if (p->buf) alisgpu__freeAsync(p->buf);
	if (p->acc) alisgpu__freeAsync(p->acc);
	if (p->comp) alisgpu__freeAsync(p->comp);
	if (p->phase) alisgpu__freeAsync(p->phase);
	if (p->fluxTab) alisgpu__freeAsync(p->fluxTab);
	for (int b = 0; b < 2; b++)
		if (p->pinned[b]) cudaEventSynchronize(p->pinnedFree[b]), pinnedRelease(p->pinned[b], p->pinnedCap), cudaEventDestroy(p->pinnedFree[b]);
	delete p;
	return ALISGPU_OK;
}

// the phase factors of the buffered steps to the device, through pinned
// staging (two buffers in turn)
static int uploadPhases(alisgpu_phaser *p)
{
	cudaStream_t st = alisgpu__stream();
	const size_t nph = p->hostPhase.size();
	if (nph > p->pinnedCap) {
		for (int b = 0; b < 2; b++) {
			if (p->pinned[b]) {
				ALIS_CUDA(cudaEventSynchronize(p->pinnedFree[b]));
				pinnedRelease(p->pinned[b], p->pinnedCap);
				p->pinned[b] = 0;
			} else {
				ALIS_CUDA(cudaEventCreateWithFlags(&p->pinnedFree[b], cudaEventDisableTiming));
				ALIS_CUDA(cudaEventRecord(p->pinnedFree[b], st));
			}
			p->pinned[b] = pinnedTake(nph);
			if (!p->pinned[b]) return alisgpu__fail(ALISGPU_ENOMEM, "phaser_flush: no pinned host memory");
		}
		p->pinnedCap = nph;
	}
	// the buffer's last upload (two flushes back) has left it
	const int b = p->pinnedNext;
	p->pinnedNext ^= 1;
	ALIS_CUDA(cudaEventSynchronize(p->pinnedFree[b]));
	memcpy(p->pinned[b], p->hostPhase.data(), nph * sizeof(float2));
	ALIS_CUDA(cudaMemcpyAsync(p->phase, p->pinned[b], nph * sizeof(float2), cudaMemcpyHostToDevice, st));
	ALIS_CUDA(cudaEventRecord(p->pinnedFree[b], st));
	return ALISGPU_OK;
}

extern "C" int alisgpu_phaser_flush(alisgpu_phaser *p)
{
	if (p) alisgpu__bind(p->w);
	if (!p) return alisgpu__fail(ALISGPU_EINVAL, "phaser_flush: null phaser");
	if (!p->used || !p->cells) { p->used = 0; p->hostPhase.clear(); return ALISGPU_OK; }
	// a batch's recorded gathers into the ring come first
	int rc = alisgpu__batch_flush();
	if (rc) return rc;
	if ((rc = uploadPhases(p))) return rc;
	cudaStream_t st = alisgpu__stream();
	long long n4 = p->cells * 4;
	dim3 grid((unsigned)((n4 + FLUSH_THREADS - 1) / FLUSH_THREADS), (p->nfreq + FLUSH_FREQ - 1) / FLUSH_FREQ);
	size_t smem = (size_t)p->used * FLUSH_FREQ * 2 * sizeof(float2);
	int slot = alisgpu__prof_start();
	// the ring staged per block where phases and ring fit 48 KB (a ring of
	// up to 64 steps), else one block per cell block and frequency group
	const size_t staged = smem + (size_t)p->used * FLUSH_THREADS * sizeof(float);
	if (staged <= 48 * 1024) {
		if (p->kahan) k_phaser_flush_staged<true><<<grid.x, FLUSH_THREADS, staged, st>>>(p->buf, p->acc, p->comp, p->phase, n4, p->nfreq, p->used);
		else k_phaser_flush_staged<false><<<grid.x, FLUSH_THREADS, staged, st>>>(p->buf, p->acc, p->comp, p->phase, n4, p->nfreq, p->used);
	} else if (p->kahan) k_phaser_flush<true><<<grid, FLUSH_THREADS, smem, st>>>(p->buf, p->acc, p->comp, p->phase, n4, p->nfreq, p->used);
	else k_phaser_flush<false><<<grid, FLUSH_THREADS, smem, st>>>(p->buf, p->acc, p->comp, p->phase, n4, p->nfreq, p->used);
	alisgpu__prof_stop(slot, ALISGPU_K_FLUSH);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	p->used = 0;
	p->hostPhase.clear();
	return ALISGPU_OK;
}

static thread_local std::vector<FlushItem> gBatchFlush;
static thread_local std::vector<GatherParams> gBatchGather;

extern "C" void alisgpu__phaser_batch_clear(void)
{
	gBatchFlush.clear();
	gBatchGather.clear();
}

// the face samples of the current fields into ring slot `used`
static void gatherParams(alisgpu_phaser *p, GatherParams &G)
{
	memset(&G, 0, sizeof G);
	alisgpu__world_fields(p->w, 0, G.E, G.H, &G.L);
	alisgpu__world_half(p->w, &G.exE, &G.exH);
	G.nface = p->nface;
	for (int f = 0; f <= p->nface; f++) G.start[f] = p->faceStart[f];
	for (int f = 0; f < p->nface; f++) {
		const alisgpu_face &a = p->faces[f];
		int b[7] = { a.axis, a.i0, a.i1, a.j0, a.j1, a.k0, a.k1 };
		memcpy(G.box[f], b, sizeof b);
	}
	G.out = p->buf + (size_t)p->used * p->cells * 4;
}

// a phaser's step in the open batch group: its ring flush when the ring
// is full, then its gather
static int recordPhaser(alisgpu_phaser *p, const float *phaseE, const float *phaseH)
{
	if (p->used == p->ring) {
		if (p->cells) {
			int rc = uploadPhases(p);
			if (rc) return rc;
			FlushItem F;
			memset(&F, 0, sizeof F);
			F.buf = p->buf, F.acc = p->acc, F.comp = p->comp, F.phase = p->phase;
			F.n4 = p->cells * 4, F.nfreq = p->nfreq, F.steps = p->used, F.kahan = p->kahan;
			F.bx = (int)((F.n4 + FLUSH_THREADS - 1) / FLUSH_THREADS);
			F.blocks = F.bx * ((p->nfreq + FLUSH_FREQ - 1) / FLUSH_FREQ);
			if (F.blocks > 0) gBatchFlush.push_back(F);
		}
		p->used = 0;
		p->hostPhase.clear();
	}
	if (p->cells) {
		GatherParams G;
		gatherParams(p, G);
		gBatchGather.push_back(G);
	}
	for (int f = 0; f < p->nfreq; f++) {
		p->hostPhase.push_back(make_float2(phaseE[2 * f], phaseE[2 * f + 1]));
		p->hostPhase.push_back(make_float2(phaseH[2 * f], phaseH[2 * f + 1]));
	}
	p->used++;
	return ALISGPU_OK;
}

extern "C" int alisgpu__phaser_batch_launch(void)
{
	auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
	std::vector<FlushItem> &F = gBatchFlush;
	std::vector<GatherParams> &G = gBatchGather;
	if (F.empty() && G.empty()) return ALISGPU_OK;
	int blocks = 0, steps = 0;
	for (FlushItem &f : F) {
		f.start = blocks;
		if ((long long)blocks + f.blocks >= (1ll << 31)) return alisgpu__fail(ALISGPU_ERANGE, "batch: flush blocks exceed 2^31");
		blocks += f.blocks;
		steps = std::max(steps, f.steps);
	}
	const size_t oF = 0, oG = al(F.size() * sizeof(FlushItem)), oI = oG + al(G.size() * sizeof(GatherParams));
	const size_t total = oI + G.size() * sizeof(GatherItem);
	void *hv = 0;
	const void *dv = 0;
	int rc = alisgpu__blob_take(total, &hv, &dv);
	if (rc) return rc;
	unsigned char *h = (unsigned char *)hv;
	const unsigned char *d = (const unsigned char *)dv;
	if (!F.empty()) memcpy(h + oF, F.data(), F.size() * sizeof(FlushItem));
	if (!G.empty()) memcpy(h + oG, G.data(), G.size() * sizeof(GatherParams));
	long long threads = 0;
	GatherItem *items = (GatherItem *)(h + oI);
	for (size_t q = 0; q < G.size(); q++) {
		items[q].G = (const GatherParams *)(d + oG) + q;
		items[q].start = threads;
		threads += G[q].start[G[q].nface];
	}
	if ((rc = alisgpu__blob_send())) return rc;
	cudaStream_t st = alisgpu__stream();
	if (blocks) {
		const size_t smem = (size_t)steps * FLUSH_FREQ * 2 * sizeof(float2);
		int slot = alisgpu__prof_start();
		k_phaser_flush_batch<<<(unsigned)blocks, FLUSH_THREADS, smem, st>>>((const FlushItem *)(d + oF), (int)F.size());
		alisgpu__prof_stop(slot, ALISGPU_K_FLUSH);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}
	if (threads) {
		int slot = alisgpu__prof_start();
		k_phaser_gather_batch<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>((const GatherItem *)(d + oI), (int)G.size(), threads);
		alisgpu__prof_stop(slot, ALISGPU_K_GATHER);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}
	F.clear(), G.clear();
	return alisgpu__blob_done();
}

extern "C" int alisgpu_phaser_record(alisgpu_phaser *p, const float *phaseE, const float *phaseH)
{
	if (p) alisgpu__bind(p->w);
	if (!p || !phaseE || !phaseH) return alisgpu__fail(ALISGPU_EINVAL, "phaser_record: bad argument");
	{
		const int rec = alisgpu__batch_enter(BATCH_PHASER, p->w);
		if (rec < 0) return alisgpu__fail(ALISGPU_ECUDA, "phaser_record: batch launch failed");
		if (rec) return recordPhaser(p, phaseE, phaseH);
	}
	if (p->used == p->ring) {
		int rc = alisgpu_phaser_flush(p);
		if (rc) return rc;
	}
	if (p->cells) {
		GatherParams G;
		memset(&G, 0, sizeof G);
		int rc = alisgpu__world_fields(p->w, 0, G.E, G.H, &G.L);
		if (rc) return rc;
		alisgpu__world_half(p->w, &G.exE, &G.exH);
		G.nface = p->nface;
		for (int f = 0; f <= p->nface; f++) G.start[f] = p->faceStart[f];
		for (int f = 0; f < p->nface; f++) {
			const alisgpu_face &a = p->faces[f];
			int b[7] = { a.axis, a.i0, a.i1, a.j0, a.j1, a.k0, a.k1 };
			memcpy(G.box[f], b, sizeof b);
		}
		G.out = p->buf + (size_t)p->used * p->cells * 4;
		// H is read on each face and one cell beyond it along the face axis
		int reads[6][6];
		for (int f = 0; f < p->nface; f++) {
			const alisgpu_face &a = p->faces[f];
			int b[6] = { a.i0, a.i1, a.j0, a.j1, a.k0, a.k1 };
			b[2 * a.axis + 1]++;
			memcpy(reads[f], b, sizeof b);
		}
		cudaStream_t st = alisgpu__gather_begin(p->w, reads, p->nface);
		int slot = alisgpu__prof_start();
		k_phaser_gather<<<(unsigned)((p->cells + 255) / 256), 256, 0, st>>>(G);
		alisgpu__prof_stop(slot, ALISGPU_K_GATHER);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
		int rc2 = alisgpu__gather_end(p->w, st);
		if (rc2) return rc2;
	}
	for (int f = 0; f < p->nfreq; f++) {
		p->hostPhase.push_back(make_float2(phaseE[2 * f], phaseE[2 * f + 1]));
		p->hostPhase.push_back(make_float2(phaseH[2 * f], phaseH[2 * f + 1]));
	}
	p->used++;
	return ALISGPU_OK;
}

extern "C" int alisgpu_phaser_download(alisgpu_phaser *p, int f, int face, int q, float *host)
{
	ALIS_BATCH_GUARD();
	if (p) alisgpu__bind(p->w);
	if (!p || !host || f < 0 || f >= p->nfreq || face < 0 || face >= p->nface || q < 0 || q > 3)
		return alisgpu__fail(ALISGPU_EINVAL, "phaser_download: bad argument");
	long long n = p->faceStart[face + 1] - p->faceStart[face];
	// strided gather of one component: (float2 at stride 4)
	const float2 *src = p->acc + (size_t)f * p->cells * 4 + p->faceStart[face] * 4 + q;
	ALIS_CUDA(cudaMemcpy2DAsync(host, sizeof(float2), src, 4 * sizeof(float2), sizeof(float2), n, cudaMemcpyDeviceToHost, alisgpu__stream()));
	ALIS_CUDA(cudaStreamSynchronize(alisgpu__stream()));
	return ALISGPU_OK;
}

extern "C" int alisgpu_phaser_zero(alisgpu_phaser *p)
{
	ALIS_BATCH_GUARD();
	if (p) alisgpu__bind(p->w);
	if (!p) return alisgpu__fail(ALISGPU_EINVAL, "phaser_zero: null phaser");
	p->used = 0;
	p->hostPhase.clear();
	if (!p->cells) return ALISGPU_OK;
	size_t bytes = (size_t)p->nfreq * p->cells * 4 * sizeof(float2);
	ALIS_CUDA(cudaMemsetAsync(p->acc, 0, bytes, alisgpu__stream()));
	if (p->comp) ALIS_CUDA(cudaMemsetAsync(p->comp, 0, bytes, alisgpu__stream()));
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// Poynting flux of every face at every frequency (reference
// src/phaser.c:156-219), with the reference's arithmetic in its order as
// one OpenMP thread runs it: each face has two sums, each an outer loop
// over one in-plane index of (spacing x inner sum), the inner sum running
// over the other index with half-weight edge terms in double and interior
// terms in float complex.  One thread computes one inner sum; one thread
// per (frequency, face) then adds the outer loops in order.
// ---------------------------------------------------------------------
struct FluxLoop {
	int face, oIsU, eq, hq, sign;          // outer index is the face's slow in-plane axis u
	int o0, o1, n0, n1;                    // outer range [o0, o1], inner edges n0, n1
	const float *wN, *wO;                  // inner (E grid) and outer (H grid) spacings, indexed by index
	long long start;                       // first inner-sum slot of this loop
};
struct FluxParams {
	int nloop;
	FluxLoop loop[12];
	long long perFreq;                     // inner sums per frequency
	int nface;
	int nv[6];                             // fast in-plane extent of each face
	long long faceStart[6];                // first cell of each face
	long long cells;                       // cells of all faces
	const float2 *acc;                     // [nfreq][cells][4]
	float *inner;                          // [nfreq][perFreq]
	float *out;                            // [nfreq][nface]
	int nfreq;
};

// the reference's `sum +/-= 0.5 * w * E * conjf(H)`: double complex product,
// the float sum widened, the real part rounded back to float
__device__ __forceinline__ float edgeTerm(float sum, int sign, float w, float2 e, float2 h)
{
	const double hw = 0.5 * (double)w;
	const double ar = hw * (double)e.x, ai = hw * (double)e.y;
	const double br = (double)h.x, bi = -(double)h.y;
	const double re = __dsub_rn(__dmul_rn(ar, br), __dmul_rn(ai, bi));
	return __double2float_rn(sign > 0 ? __dadd_rn((double)sum, re) : __dsub_rn((double)sum, re));
}

// `sum +/-= w * E * conjf(H)` in float complex arithmetic
__device__ __forceinline__ float midTerm(float sum, int sign, float w, float2 e, float2 h)
{
	const float ar = __fmul_rn(w, e.x), ai = __fmul_rn(w, e.y);
	const float re = __fsub_rn(__fmul_rn(ar, h.x), __fmul_rn(ai, -h.y));
	return sign > 0 ? __fadd_rn(sum, re) : __fsub_rn(sum, re);
}

__global__ void k_phaser_flux_inner(const FluxParams P)
{
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= P.perFreq * P.nfreq) return;
	const int f = (int)(t / P.perFreq);
	const long long r = t % P.perFreq;
	int l = 0;
	while (l + 1 < P.nloop && r >= P.loop[l + 1].start) l++;
	const FluxLoop &L = P.loop[l];
	const int o = L.o0 + 1 + (int)(r - L.start);   // outer index in (o0, o1]
	const float2 *acc = P.acc + ((long long)f * P.cells + P.faceStart[L.face]) * 4;
	const int nv = P.nv[L.face];
	// cell (u, v) of the face at acc[((u - u0) * nv + (v - v0)) * 4 + q]
	auto at = [&](int n) -> long long {
		const long long u = L.oIsU ? o - L.o0 : n - L.n0;
		const long long v = L.oIsU ? n - L.n0 : o - L.o0;
		return (u * nv + v) * 4;
	};
	float sum = 0;
	sum = edgeTerm(sum, L.sign, L.wN[L.n0], acc[at(L.n0) + L.eq], acc[at(L.n0) + L.hq]);
	sum = edgeTerm(sum, L.sign, L.wN[L.n1], acc[at(L.n1) + L.eq], acc[at(L.n1) + L.hq]);
	for (int n = L.n0 + 1; n < L.n1; n++)
		sum = midTerm(sum, L.sign, L.wN[n], acc[at(n) + L.eq], acc[at(n) + L.hq]);
	P.inner[t] = sum;
}

__global__ void k_phaser_flux_outer(const FluxParams P)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= P.nfreq * P.nface) return;
	const int f = t / P.nface, face = t % P.nface;
	const float *inner = P.inner + (long long)f * P.perFreq;
	float Sum = 0, Part = 0;
	int seen = 0;
	for (int l = 0; l < P.nloop; l++) {
		const FluxLoop &L = P.loop[l];
		if (L.face != face) continue;
		float acc = 0;
		for (int o = L.o0 + 1; o <= L.o1; o++) acc = __fadd_rn(acc, __fmul_rn(L.wO[o], inner[L.start + (o - L.o0 - 1)]));
		if (seen++ == 0) Sum = acc; else Part = acc;
	}
	P.out[t] = __fadd_rn(Sum, Part);
}

extern "C" int alisgpu_phaser_face_flux(alisgpu_phaser *p, const float *const wE[3], const float *const wH[3],
                                        const int lo[3], const int hi[3], float *out)
{
	ALIS_BATCH_GUARD();
	if (p) alisgpu__bind(p->w);
	if (!p || !wE || !wH || !lo || !hi || !out) return alisgpu__fail(ALISGPU_EINVAL, "phaser_face_flux: bad argument");
	int rc = alisgpu_phaser_flush(p);
	if (rc) return rc;
	if (!p->nface || !p->nfreq) return ALISGPU_OK;
	cudaStream_t st = alisgpu__stream();
	int len[3];
	size_t tabFloats = 0;
	for (int a = 0; a < 3; a++) {
		if (hi[a] < lo[a]) return alisgpu__fail(ALISGPU_EINVAL, "phaser_face_flux: empty box");
		len[a] = 1 + hi[a] - lo[a];
		tabFloats += 2 * (size_t)len[a];
	}
	FluxParams P;
	memset(&P, 0, sizeof P);
	P.nface = p->nface, P.nfreq = p->nfreq, P.cells = p->cells, P.acc = p->acc;
	// inner-sum slots
	long long per = 0;
	for (int q = 0; q < p->nface; q++) {
		const alisgpu_face &fc = p->faces[q];
		for (int a = 0; a < 3; a++) {
			const int b0 = a == 0 ? fc.i0 : a == 1 ? fc.j0 : fc.k0, b1 = a == 0 ? fc.i1 : a == 1 ? fc.j1 : fc.k1;
			if (b0 < lo[a] || b1 > hi[a]) return alisgpu__fail(ALISGPU_EINVAL, "phaser_face_flux: face outside the table box");
		}
		const int ua = fc.axis == 0 ? 1 : 0, va = fc.axis == 2 ? 1 : 2;
		const int u0 = ua == 0 ? fc.i0 : fc.j0, u1 = ua == 0 ? fc.i1 : fc.j1;
		const int v0 = va == 1 ? fc.j0 : fc.k0, v1 = va == 1 ? fc.j1 : fc.k1;
		P.nv[q] = 1 + v1 - v0;
		P.faceStart[q] = p->faceStart[q];
		// (outer axis is u, E comp, H comp, sign) of the two loops: x face
		// (u=j, v=k) L1 j-outer Ey Hz +, L2 k-outer Ez Hy -; y face (u=i,
		// v=k) L1 k-outer Ez Hx +, L2 i-outer Ex Hz -; z face (u=i, v=j) L1
		// i-outer Ex Hy +, L2 j-outer Ey Hx -.  Components per cell: E1 E2 H1 H2.
		const int oIsU[2] = { fc.axis == 1 ? 0 : 1, fc.axis == 1 ? 1 : 0 };
		for (int l = 0; l < 2; l++) {
			FluxLoop &L = P.loop[P.nloop++];
			L.face = q, L.oIsU = oIsU[l];
			L.eq = l == 0 ? 0 : 1, L.hq = l == 0 ? 3 : 2, L.sign = l == 0 ? 1 : -1;
			L.o0 = L.oIsU ? u0 : v0, L.o1 = L.oIsU ? u1 : v1;
			L.n0 = L.oIsU ? v0 : u0, L.n1 = L.oIsU ? v1 : u1;
			L.start = per;
			per += L.o1 - L.o0;
		}
	}
	P.perFreq = per;
	// device tables: wE[3], wH[3] (each over [lo, hi] of its axis), then the inner sums and the output
	size_t innerFloats = (size_t)per * p->nfreq, outFloats = (size_t)p->nfreq * p->nface;
	size_t bytes = (tabFloats + innerFloats + outFloats) * sizeof(float);
	if (bytes > p->fluxTabBytes) {
		ALIS_CUDA(cudaStreamSynchronize(st));
		if (p->fluxTab) alisgpu__freeAsync(p->fluxTab);
		p->fluxTab = 0, p->fluxTabBytes = 0;
		ALIS_CUDA(alisgpu__mallocAsync(&p->fluxTab, bytes));
		p->fluxTabBytes = bytes;
	}
	float *tab = p->fluxTab;
	const float *dE[3], *dH[3];
	for (int a = 0; a < 3; a++) {
		ALIS_CUDA(cudaMemcpyAsync(tab, wE[a], len[a] * sizeof(float), cudaMemcpyHostToDevice, st));
		dE[a] = tab - lo[a], tab += len[a];
		ALIS_CUDA(cudaMemcpyAsync(tab, wH[a], len[a] * sizeof(float), cudaMemcpyHostToDevice, st));
		dH[a] = tab - lo[a], tab += len[a];
	}
	P.inner = tab, tab += innerFloats;
	P.out = tab;
	for (int l = 0; l < P.nloop; l++) {
		FluxLoop &L = P.loop[l];
		const alisgpu_face &fc = p->faces[L.face];
		const int ua = fc.axis == 0 ? 1 : 0, va = fc.axis == 2 ? 1 : 2;
		const int oa = L.oIsU ? ua : va, na = L.oIsU ? va : ua;
		L.wN = dE[na], L.wO = dH[oa];
	}
	if (per > 0) {
		long long threads = per * p->nfreq;
		int slot = alisgpu__prof_start();
		k_phaser_flux_inner<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(P);
		k_phaser_flux_outer<<<(p->nfreq * p->nface + 127) / 128, 128, 0, st>>>(P);
		alisgpu__prof_stop(slot, ALISGPU_K_FLUX);
		alisgpu__count_launch();
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
		ALIS_CUDA(cudaMemcpyAsync(out, P.out, outFloats * sizeof(float), cudaMemcpyDeviceToHost, st));
	} else {
		memset(out, 0, outFloats * sizeof(float));
	}
	ALIS_CUDA(cudaStreamSynchronize(st));
	return ALISGPU_OK;
}

// accessors for the far-field kernel
extern "C" const float2 *alisgpu__phaser_acc(alisgpu_phaser *p, int f, int face, long long *cells)
{
	*cells = p->faceStart[face + 1] - p->faceStart[face];
	return p->acc + (size_t)f * p->cells * 4 + p->faceStart[face] * 4;
}
extern "C" int alisgpu__phaser_nface(alisgpu_phaser *p) { return p->nface; }
extern "C" int alisgpu__phaser_nfreq(alisgpu_phaser *p) { return p->nfreq; }
extern "C" void alisgpu__bind_phaser(alisgpu_phaser *p) { if (p) alisgpu__bind(p->w); }
extern "C" const alisgpu_face *alisgpu__phaser_face(alisgpu_phaser *p, int face) { return &p->faces[face]; }
