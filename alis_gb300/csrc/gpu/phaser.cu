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
#include <vector>
#include "common.cuh"

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
	int *faceInfo;                        // per face: axis, box
	int used;                             // buffered steps
};

// world layout and field pointers needed by the gather kernel
struct GatherParams {
	Layout L;
	const float *E[3], *H[3];
	int nface;
	long long start[7];
	int box[6][7];                        // axis, i0, i1, j0, j1, k0, k1
	float *out;                           // ring slot
};

extern "C" int alisgpu__world_fields(alisgpu_world *w, int m, const float **E, const float **H, Layout *L);

__global__ void k_phaser_gather(const GatherParams P)
{
	long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
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
	v.x = P.E[c1][c];
	v.y = P.E[c2][c];
	v.z = P.H[c1][c] + P.H[c1][n];
	v.w = P.H[c2][c] + P.H[c2][n];
	reinterpret_cast<float4 *>(P.out)[t] = v;
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

// thread = one (face cell, component); loops over a chunk of frequencies
template <bool KAHAN>
__global__ void __launch_bounds__(FLUSH_THREADS) k_phaser_flush(const float *buf, float2 *acc, float2 *comp, const float2 *phase,
                                                                long long n4, int nfreq, int steps)
{
	extern __shared__ float2 sph[];                 // [steps][FLUSH_FREQ][2]
	const int f0 = blockIdx.y * FLUSH_FREQ;
	const int nf = min(FLUSH_FREQ, nfreq - f0);
	for (int q = threadIdx.x; q < steps * FLUSH_FREQ * 2; q += blockDim.x) {
		int s = q / (FLUSH_FREQ * 2), r = q % (FLUSH_FREQ * 2), ff = r / 2, h = r % 2;
		sph[q] = ff < nf ? phase[((long long)s * nfreq + f0 + ff) * 2 + h] : make_float2(0, 0);
	}
	__syncthreads();
	long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n4) return;
	const bool isH = (t & 3) >= 2;
	float2 a[FLUSH_FREQ], cc[FLUSH_FREQ];
#pragma unroll
	for (int ff = 0; ff < FLUSH_FREQ; ff++) {
		if (ff < nf) {
			a[ff] = acc[(long long)(f0 + ff) * n4 + t];
			cc[ff] = KAHAN ? comp[(long long)(f0 + ff) * n4 + t] : make_float2(0, 0);
		}
	}
	for (int s = 0; s < steps; s++) {
		const float x = buf[(long long)s * n4 + t];
#pragma unroll
		for (int ff = 0; ff < FLUSH_FREQ; ff++) {
			if (ff >= nf) break;
			const float2 p = sph[(s * FLUSH_FREQ + ff) * 2 + (isH ? 1 : 0)];
			const float pr = p.x * x, pi = p.y * x;
			if (!KAHAN) {
				if (isH) a[ff].x = addHalf(a[ff].x, pr), a[ff].y = addHalf(a[ff].y, pi);
				else a[ff].x = a[ff].x + pr, a[ff].y = a[ff].y + pi;
			} else {
				// Kahan: y = term - c; s' = s + y; c = (s' - s) - y
				float yr = (isH ? pr * 0.5f : pr) - cc[ff].x, yi = (isH ? pi * 0.5f : pi) - cc[ff].y;
				float sr = a[ff].x + yr, sI = a[ff].y + yi;
				cc[ff].x = (sr - a[ff].x) - yr, cc[ff].y = (sI - a[ff].y) - yi;
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

extern "C" int alisgpu_phaser_create(alisgpu_world *w, int nfreq, int nface, const alisgpu_face *faces, int ring, int kahan, alisgpu_phaser **out)
{
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
		ALIS_CUDA(cudaMalloc(&p->buf, (size_t)ring * n4 * sizeof(float)));
		ALIS_CUDA(cudaMalloc(&p->acc, (size_t)nfreq * n4 * sizeof(float2)));
		ALIS_CUDA(cudaMemsetAsync(p->acc, 0, (size_t)nfreq * n4 * sizeof(float2), st));
		if (kahan) {
			ALIS_CUDA(cudaMalloc(&p->comp, (size_t)nfreq * n4 * sizeof(float2)));
			ALIS_CUDA(cudaMemsetAsync(p->comp, 0, (size_t)nfreq * n4 * sizeof(float2), st));
		}
	}
	ALIS_CUDA(cudaMalloc(&p->phase, (size_t)ring * nfreq * 2 * sizeof(float2)));
	p->used = 0;
	*out = p;
	return ALISGPU_OK;
}

extern "C" int alisgpu_phaser_destroy(alisgpu_phaser *p)
{
	if (!p) return ALISGPU_OK;
	cudaStreamSynchronize(alisgpu__stream());
	if (p->buf) cudaFree(p->buf);
	if (p->acc) cudaFree(p->acc);
	if (p->comp) cudaFree(p->comp);
	if (p->phase) cudaFree(p->phase);
	delete p;
	return ALISGPU_OK;
}

extern "C" int alisgpu_phaser_flush(alisgpu_phaser *p)
{
	if (!p) return alisgpu__fail(ALISGPU_EINVAL, "phaser_flush: null phaser");
	if (!p->used || !p->cells) { p->used = 0; p->hostPhase.clear(); return ALISGPU_OK; }
	cudaStream_t st = alisgpu__stream();
	ALIS_CUDA(cudaMemcpyAsync(p->phase, p->hostPhase.data(), p->hostPhase.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
	long long n4 = p->cells * 4;
	dim3 grid((unsigned)((n4 + FLUSH_THREADS - 1) / FLUSH_THREADS), (p->nfreq + FLUSH_FREQ - 1) / FLUSH_FREQ);
	size_t smem = (size_t)p->used * FLUSH_FREQ * 2 * sizeof(float2);
	int slot = alisgpu__prof_start();
	if (p->kahan) k_phaser_flush<true><<<grid, FLUSH_THREADS, smem, st>>>(p->buf, p->acc, p->comp, p->phase, n4, p->nfreq, p->used);
	else k_phaser_flush<false><<<grid, FLUSH_THREADS, smem, st>>>(p->buf, p->acc, p->comp, p->phase, n4, p->nfreq, p->used);
	alisgpu__prof_stop(slot, ALISGPU_K_FLUSH);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	p->used = 0;
	p->hostPhase.clear();
	return ALISGPU_OK;
}

extern "C" int alisgpu_phaser_record(alisgpu_phaser *p, const float *phaseE, const float *phaseH)
{
	if (!p || !phaseE || !phaseH) return alisgpu__fail(ALISGPU_EINVAL, "phaser_record: bad argument");
	if (p->used == p->ring) {
		int rc = alisgpu_phaser_flush(p);
		if (rc) return rc;
	}
	if (p->cells) {
		GatherParams G;
		memset(&G, 0, sizeof G);
		int rc = alisgpu__world_fields(p->w, 0, G.E, G.H, &G.L);
		if (rc) return rc;
		G.nface = p->nface;
		for (int f = 0; f <= p->nface; f++) G.start[f] = p->faceStart[f];
		for (int f = 0; f < p->nface; f++) {
			const alisgpu_face &a = p->faces[f];
			int b[7] = { a.axis, a.i0, a.i1, a.j0, a.j1, a.k0, a.k1 };
			memcpy(G.box[f], b, sizeof b);
		}
		G.out = p->buf + (size_t)p->used * p->cells * 4;
		int slot = alisgpu__prof_start();
		k_phaser_gather<<<(unsigned)((p->cells + 255) / 256), 256, 0, alisgpu__stream()>>>(G);
		alisgpu__prof_stop(slot, ALISGPU_K_GATHER);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
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
	if (!p) return alisgpu__fail(ALISGPU_EINVAL, "phaser_zero: null phaser");
	p->used = 0;
	p->hostPhase.clear();
	if (!p->cells) return ALISGPU_OK;
	size_t bytes = (size_t)p->nfreq * p->cells * 4 * sizeof(float2);
	ALIS_CUDA(cudaMemsetAsync(p->acc, 0, bytes, alisgpu__stream()));
	if (p->comp) ALIS_CUDA(cudaMemsetAsync(p->comp, 0, bytes, alisgpu__stream()));
	return ALISGPU_OK;
}

// accessors for the far-field kernel
extern "C" const float2 *alisgpu__phaser_acc(alisgpu_phaser *p, int f, int face, long long *cells)
{
	*cells = p->faceStart[face + 1] - p->faceStart[face];
	return p->acc + (size_t)f * p->cells * 4 + p->faceStart[face] * 4;
}
extern "C" int alisgpu__phaser_nface(alisgpu_phaser *p) { return p->nface; }
extern "C" const alisgpu_face *alisgpu__phaser_face(alisgpu_phaser *p, int face) { return &p->faces[face]; }
