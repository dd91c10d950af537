// farfield.cu -- near-to-far-field face sums in FP64.
//
// For one phaser frequency and a batch of directions, each face of the
// phaser box contributes four bilinear forms
//     sum_u sum_v alpha(u) beta(v) S(u, v)
// of a DFT accumulator S with per-direction weights: lateral Bloch
// factors exp(i k x) times cell spacings on one in-plane axis, and the
// 1-D reciprocity test field times spacings on the other, with trapezoid
// end weights (reference src/farfld.c:248-459).  One block handles one
// (direction, face): the weight vectors go to shared memory in double,
// every thread sums a strided share of the face cells in double, and a
// block reduction combines them.  The accumulators themselves are the
// float sums of the phaser kernels.  This file is built with FMA
// contraction on: it is an FP64 computation checked to a tolerance against
// an FP64 restatement, not a bit-exact replica of the FP32 reference.
#include <cstring>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "batch.cuh"

extern "C" const float2 *alisgpu__phaser_acc(alisgpu_phaser *p, int f, int face, long long *cells);
extern "C" int alisgpu__phaser_nface(alisgpu_phaser *p);
extern "C" int alisgpu__phaser_nfreq(alisgpu_phaser *p);
extern "C" void alisgpu__bind_phaser(alisgpu_phaser *p);
extern "C" const alisgpu_face *alisgpu__phaser_face(alisgpu_phaser *p, int face);

struct FFFace {
	int axis, side;                      // side 0 min, 1 max
	int i0, i1, j0, j1, k0, k1;
	const float2 *acc;                   // [cells][4] (E1, E2, H1, H2)
};

struct FFParams {
	int nface;
	FFFace face[6];
	alisgpu_farfield_geom g;
	int nk;
	const double2 *T;                    // [nA][6][nk]
	const unsigned char *present;        // [nA][6]
	const double *kx, *ky;
	double2 *part;                       // [nA][6]
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x*b.x - a.y*b.y, a.x*b.y + a.y*b.x); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cexpi(double t) { double s, c; sincos(t, &s, &c); return make_double2(c, s); }

// trapezoid weight of index u in [lo, hi]
__device__ __forceinline__ double trap(int u, int lo, int hi)
{
	if (u < lo || u > hi) return 0;
	return (u == lo ? 0.5 : 0.0) + (u == hi ? 0.5 : 0.0) + (u > lo && u < hi ? 1.0 : 0.0);
}

// lateral weights: 0 -> E-grid (dxE e^{ik x(i)}, mirror -conj cos), 1 ->
// H-grid (dxH e^{ik x(i-1/2)}, mirror +conj cos), axis 0 (x) or 1 (y)
__device__ double2 lateral(const alisgpu_farfield_geom &g, int axis, int grid, int u, double kk)
{
	const double *coord = axis == 0 ? (grid ? g.xH : g.xE) : (grid ? g.yH : g.yE);
	const double *sp = axis == 0 ? (grid ? g.dxH : g.dxE) : (grid ? g.dyH : g.dyE);
	int base = axis == 0 ? g.iMin : g.jMin;
	double2 w = cscale(cexpi(kk * coord[u - base]), sp[u - base]);
	if (g.sym[axis]) {
		double2 m = cscale(cconj(w), g.cosk[axis]);
		w = grid ? cadd(w, m) : csub(w, m);
	}
	return w;
}

// z weights from the test field component c: integer-k components (Ex,
// Ey, Hz) use E-grid dz and mirror -T[-k]; half-k ones (Ez, Hx, Hy) use
// H-grid dz and mirror +T[1-k]
__device__ double2 zweight(const alisgpu_farfield_geom &g, const double2 *T, int nk, int c, int k)
{
	bool integer = c == 0 || c == 1 || c == 5;
	const double *dz = integer ? g.dzE : g.dzH;
	double d = dz[k - g.kMIN];
	double2 w = cscale(T[c * nk + (k - g.kMIN)], d);
	if (g.sym[2]) {
		int mk = integer ? -k : 1 - k;
		double2 m = cscale(cscale(T[c * nk + (mk - g.kMIN)], d), g.cosk[2]);
		w = integer ? csub(w, m) : cadd(w, m);
	}
	return w;
}

#define FF_THREADS 256

__global__ void __launch_bounds__(FF_THREADS) k_farfield(const FFParams P)
{
	extern __shared__ double2 sm[];
	const int a = blockIdx.x, fidx = blockIdx.y;
	const FFFace &F = P.face[fidx];
	const alisgpu_farfield_geom &g = P.g;
	const double2 *T = P.T + (size_t)a * 6 * P.nk;
	const unsigned char *pr = P.present + a * 6;
	const double kx = P.kx[a], ky = P.ky[a];
	// in-plane axes: x face (u=j, v=k), y face (u=i, v=k), z face (u=i, v=j)
	int u0, u1, v0, v1;
	if (F.axis == 0) u0 = F.j0, u1 = F.j1, v0 = F.k0, v1 = F.k1;
	else if (F.axis == 1) u0 = F.i0, u1 = F.i1, v0 = F.k0, v1 = F.k1;
	else u0 = F.i0, u1 = F.i1, v0 = F.j0, v1 = F.j1;
	const int nu = 1 + u1 - u0, nv = 1 + v1 - v0;
	double2 *al = sm;                       // [4][nu]
	double2 *be = sm + 4 * nu;              // [4][nv]
	// the four terms: (alpha, beta, accumulator component); see header
	for (int u = threadIdx.x; u < nu; u += blockDim.x) {
		int uu = u0 + u;
		double2 w0, w1;
		if (F.axis == 0) { w1 = lateral(g, 1, 1, uu, ky); w0 = lateral(g, 1, 0, uu, ky); }
		else { w1 = lateral(g, 0, 1, uu, kx); w0 = lateral(g, 0, 0, uu, kx); }
		double2 z = make_double2(0, 0);
		double2 A1 = uu > u0 ? w1 : z;               // range [u0+1, u1]
		double2 A0 = cscale(w0, trap(uu, u0, u1));   // trapezoid over [u0, u1]
		if (F.axis == 0) al[u] = A1, al[nu + u] = A1, al[2*nu + u] = A0, al[3*nu + u] = A0;
		else if (F.axis == 1) al[u] = A0, al[nu + u] = A0, al[2*nu + u] = A1, al[3*nu + u] = A1;
		else al[u] = A1, al[nu + u] = A1, al[2*nu + u] = A0, al[3*nu + u] = A0;
	}
	for (int v = threadIdx.x; v < nv; v += blockDim.x) {
		int vv = v0 + v;
		double2 z = make_double2(0, 0);
		if (F.axis == 0) {
			// EyHz: trap*Z(Hz); HzEy: trap*Z(Ey); EzHy: Z(Hy) on [v0+1,v1]; HyEz: Z(Ez) on [v0+1,v1]
			double t = trap(vv, v0, v1);
			be[v] = pr[5] ? cscale(zweight(g, T, P.nk, 5, vv), t) : z;
			be[nv + v] = pr[1] ? cscale(zweight(g, T, P.nk, 1, vv), t) : z;
			be[2*nv + v] = pr[4] && vv > v0 ? zweight(g, T, P.nk, 4, vv) : z;
			be[3*nv + v] = pr[2] && vv > v0 ? zweight(g, T, P.nk, 2, vv) : z;
		} else if (F.axis == 1) {
			// EzHx: Z(Hx) [v0+1,v1]; HxEz: Z(Ez) [v0+1,v1]; ExHz: trap*Z(Hz); HzEx: trap*Z(Ex)
			double t = trap(vv, v0, v1);
			be[v] = pr[3] && vv > v0 ? zweight(g, T, P.nk, 3, vv) : z;
			be[nv + v] = pr[2] && vv > v0 ? zweight(g, T, P.nk, 2, vv) : z;
			be[2*nv + v] = pr[5] ? cscale(zweight(g, T, P.nk, 5, vv), t) : z;
			be[3*nv + v] = pr[0] ? cscale(zweight(g, T, P.nk, 0, vv), t) : z;
		} else {
			// z face: beta over j -- ExHy, HyEx: trap*Y0; EyHx, HxEy: Y1 on [v0+1,v1]
			double2 y0 = cscale(lateral(g, 1, 0, vv, ky), trap(vv, v0, v1));
			double2 y1 = vv > v0 ? lateral(g, 1, 1, vv, ky) : z;
			be[v] = y0, be[nv + v] = y0, be[2*nv + v] = y1, be[3*nv + v] = y1;
		}
	}
	__syncthreads();
	// accumulator component of each term: x face (E1=Ey, H2=Hz, E2=Ez, H1=Hy);
	// y face (E1=Ez, H2=Hx, E2=Ex, H1=Hz); z face (E1=Ex, H2=Hy, E2=Ey, H1=Hx)
	const int q[4] = { 0, 3, 1, 2 };
	double2 s[4] = { {0,0}, {0,0}, {0,0}, {0,0} };
	const long long cells = (long long)nu * nv;
	for (long long t = threadIdx.x; t < cells; t += blockDim.x) {
		int u = (int)(t / nv), v = (int)(t % nv);
		const float2 *cell = F.acc + t * 4;
#pragma unroll
		for (int r = 0; r < 4; r++) {
			float2 x = cell[q[r]];
			double2 sv = make_double2(x.x, x.y);
			s[r] = cadd(s[r], cmul(cmul(al[r*nu + u], be[r*nv + v]), sv));
		}
	}
	// block reduction
	__shared__ double2 red[4][FF_THREADS / 32];
	for (int r = 0; r < 4; r++) {
		double2 v = s[r];
		for (int o = 16; o > 0; o >>= 1) {
			v.x += __shfl_down_sync(0xffffffffu, v.x, o);
			v.y += __shfl_down_sync(0xffffffffu, v.y, o);
		}
		if ((threadIdx.x & 31) == 0) red[r][threadIdx.x >> 5] = v;
	}
	__syncthreads();
	if (threadIdx.x) return;
	for (int r = 0; r < 4; r++) {
		double2 v = make_double2(0, 0);
		for (int w = 0; w < FF_THREADS / 32; w++) v = cadd(v, red[r][w]);
		s[r] = v;
	}
	double2 out;
	if (F.axis == 0) {
		// (EyHz - HzEy - EzHy + HyEz) e^{i kx x(i)} (+ mirror)
		double2 sum = cadd(csub(csub(s[0], s[1]), s[2]), s[3]);
		double xi = g.xE[F.i0 - g.iMin];
		out = cmul(sum, cexpi(kx * xi));
		if (g.sym[0]) out = cadd(out, cscale(cmul(csub(cadd(s[0], s[1]), cadd(s[2], s[3])), cexpi(-kx * xi)), g.cosk[0]));
	} else if (F.axis == 1) {
		// (EzHx - HxEz - ExHz + HzEx) e^{i ky y(j)} (+ mirror)
		double2 sum = cadd(csub(csub(s[0], s[1]), s[2]), s[3]);
		double yj = g.yE[F.j0 - g.jMin];
		out = cmul(sum, cexpi(ky * yj));
		if (g.sym[1]) out = cadd(out, cscale(cmul(csub(cadd(s[0], s[1]), cadd(s[2], s[3])), cexpi(-ky * yj)), g.cosk[1]));
	} else {
		int k = F.k0, kk = k - g.kMIN;
		const double2 *Ex = T, *Ey = T + P.nk, *Hx = T + 3 * P.nk, *Hy = T + 4 * P.nk;
		out = make_double2(0, 0);
		if (pr[4]) {
			double2 h = cscale(cadd(Hy[kk], Hy[kk + 1]), 0.5);
			out = cadd(out, cmul(s[0], h));
			if (g.sym[2]) out = cadd(out, cscale(cmul(s[0], cscale(cadd(Hy[1 - k - g.kMIN], Hy[-k - g.kMIN]), 0.5)), g.cosk[2]));
		}
		if (pr[0]) {
			out = csub(out, cmul(s[1], Ex[kk]));
			if (g.sym[2]) out = cadd(out, cscale(cmul(s[1], Ex[-k - g.kMIN]), g.cosk[2]));
		}
		if (pr[3]) {
			double2 h = cscale(cadd(Hx[kk], Hx[kk + 1]), 0.5);
			out = csub(out, cmul(s[2], h));
			if (g.sym[2]) out = csub(out, cscale(cmul(s[2], cscale(cadd(Hx[1 - k - g.kMIN], Hx[-k - g.kMIN]), 0.5)), g.cosk[2]));
		}
		if (pr[1]) {
			out = cadd(out, cmul(s[3], Ey[kk]));
			if (g.sym[2]) out = csub(out, cscale(cmul(s[3], Ey[-k - g.kMIN]), g.cosk[2]));
		}
	}
	P.part[a * 6 + fidx] = out;
}

// Faces of the phaser in the kernel's form, and the largest shared-memory
// weight table one of them needs.  Checks every index the kernel derives
// from the arguments: the frequency, and for every face its i, j and k
// ranges (k one beyond, for the half-cell H samples) against the lengths
// of the line tables and of the test fields, mirror images included.
static int ffFaces(alisgpu_phaser *p, int f, const alisgpu_farfield_geom *g, int nk, FFParams &P, size_t &smem,
                   const char *who)
{
	if (f < 0 || f >= alisgpu__phaser_nfreq(p))
		return alisgpu__fail(ALISGPU_EINVAL, "%s: frequency %d outside [0, %d)", who, f, alisgpu__phaser_nfreq(p));
	if (nk < 1 || g->zLen < 1 || g->xLen < 0 || g->yLen < 0)
		return alisgpu__fail(ALISGPU_EINVAL, "%s: bad table lengths (nk %d, z %d)", who, nk, g->zLen);
	const int kLen = nk < g->zLen ? nk : g->zLen;
	P.nface = alisgpu__phaser_nface(p);
	int maxn = 1;
	for (int q = 0; q < P.nface; q++) {
		const alisgpu_face *fc = alisgpu__phaser_face(p, q);
		FFFace &F = P.face[q];
		F.axis = fc->axis;
		F.i0 = fc->i0, F.i1 = fc->i1, F.j0 = fc->j0, F.j1 = fc->j1, F.k0 = fc->k0, F.k1 = fc->k1;
		bool ok = F.i0 >= g->iMin && F.i1 < g->iMin + g->xLen && F.j0 >= g->jMin && F.j1 < g->jMin + g->yLen &&
		          F.k0 >= g->kMIN && F.k1 + 1 < g->kMIN + kLen;
		if (g->sym[2]) ok = ok && -F.k1 >= g->kMIN && 1 - F.k0 < g->kMIN + kLen;
		if (!ok)
			return alisgpu__fail(ALISGPU_EINVAL, "%s: face %d [%d,%d]x[%d,%d]x[%d,%d] outside the tables", who, q,
			                     F.i0, F.i1, F.j0, F.j1, F.k0, F.k1);
		long long cells;
		F.acc = alisgpu__phaser_acc(p, f, q, &cells);
		int n1 = F.axis == 0 ? 1 + F.j1 - F.j0 : 1 + F.i1 - F.i0;
		int n2 = F.axis == 2 ? 1 + F.j1 - F.j0 : 1 + F.k1 - F.k0;
		maxn = n1 + n2 > maxn ? n1 + n2 : maxn;
	}
	smem = (size_t)4 * maxn * sizeof(double2);
	if (smem > 200 * 1024) return alisgpu__fail(ALISGPU_ERANGE, "%s: face of %d cells per side too large", who, maxn);
	return ALISGPU_OK;
}

extern "C" int alisgpu_farfield_sums(alisgpu_phaser *p, int f, const alisgpu_farfield_geom *g, int nA,
                                     const double *T, int nk, const unsigned char *present,
                                     const double *kx, const double *ky, double *out)
{
	ALIS_BATCH_GUARD();
	if (!p || !g || nA < 0 || nk < 0 || !T || !present || !kx || !ky || !out)
		return alisgpu__fail(ALISGPU_EINVAL, "farfield_sums: bad argument");
	if (!nA) return ALISGPU_OK;
	alisgpu__bind_phaser(p);
	FFParams P;
	memset(&P, 0, sizeof P);
	size_t smem = 0;
	int rc = ffFaces(p, f, g, nk, P, smem, "farfield_sums");
	if (rc) return rc;
	cudaStream_t st = alisgpu__stream();
	// Device copies of the geometry tables and the direction batch.  Every
	// allocation is made before anything is enqueued; any failure frees
	// what was taken and returns before a copy or a launch.
	std::vector<void *> tmp;
	bool failed = false;
	auto take = [&](size_t bytes) -> void * {
		void *d = 0;
		if (alisgpu__mallocAsync(&d, bytes ? bytes : 1) != cudaSuccess) d = 0, failed = true;
		tmp.push_back(d);
		return d;
	};
	auto release = [&]() { for (void *q : tmp) if (q) alisgpu__freeAsync(q); tmp.clear(); };
	const double *src[10] = { g->xE, g->xH, g->dxE, g->dxH, g->yE, g->yH, g->dyE, g->dyH, g->dzE, g->dzH };
	size_t bytes[10];
	for (int q = 0; q < 10; q++) bytes[q] = (size_t)(q < 4 ? g->xLen : q < 8 ? g->yLen : g->zLen) * sizeof(double);
	void *dTab[10];
	for (int q = 0; q < 10; q++) dTab[q] = take(bytes[q]);
	const size_t tBytes = (size_t)nA * 6 * nk * sizeof(double2);
	void *dT = take(tBytes), *dPr = take((size_t)nA * 6);
	void *dKx = take(nA * sizeof(double)), *dKy = take(nA * sizeof(double));
	double2 *part = (double2 *)take((size_t)nA * 6 * sizeof(double2));
	if (failed) {
		release();
		return alisgpu__fail(ALISGPU_ENOMEM, "farfield_sums: allocation failed");
	}
	cudaError_t e = cudaSuccess;
	for (int q = 0; q < 10 && e == cudaSuccess; q++)
		if (bytes[q]) e = cudaMemcpyAsync(dTab[q], src[q], bytes[q], cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dT, T, tBytes, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dPr, present, (size_t)nA * 6, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dKx, kx, nA * sizeof(double), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dKy, ky, nA * sizeof(double), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemsetAsync(part, 0, (size_t)nA * 6 * sizeof(double2), st);
	P.g = *g;
	P.g.xE = (const double *)dTab[0], P.g.xH = (const double *)dTab[1];
	P.g.dxE = (const double *)dTab[2], P.g.dxH = (const double *)dTab[3];
	P.g.yE = (const double *)dTab[4], P.g.yH = (const double *)dTab[5];
	P.g.dyE = (const double *)dTab[6], P.g.dyH = (const double *)dTab[7];
	P.g.dzE = (const double *)dTab[8], P.g.dzH = (const double *)dTab[9];
	P.nk = nk;
	P.T = (const double2 *)dT;
	P.present = (const unsigned char *)dPr;
	P.kx = (const double *)dKx, P.ky = (const double *)dKy;
	P.part = part;
	if (e == cudaSuccess) e = cudaFuncSetAttribute(k_farfield, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess && P.nface) {
		dim3 grid(nA, P.nface);
		int slot = alisgpu__prof_start();
		k_farfield<<<grid, FF_THREADS, smem, st>>>(P);
		alisgpu__prof_stop(slot, ALISGPU_K_FARFIELD);
		alisgpu__count_launch();
		e = cudaGetLastError();
	}
	std::vector<double2> h((size_t)nA * 6);
	if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, st);
	// whatever was enqueued finishes before the buffers go back to the pool
	cudaError_t es = cudaStreamSynchronize(st);
	release();
	if (e == cudaSuccess) e = es;
	if (e != cudaSuccess) return alisgpu__check(e, "farfield_sums");
	// faces in device order are min/max per axis as the host listed them;
	// the host gives the sign per face through out[] layout: out[a*12 + 2*face]
	for (int a = 0; a < nA; a++) for (int q = 0; q < 6; q++) {
		out[(a * 6 + q) * 2] = q < P.nface ? h[a * 6 + q].x : 0;
		out[(a * 6 + q) * 2 + 1] = q < P.nface ? h[a * 6 + q].y : 0;
	}
	return ALISGPU_OK;
}

// ---------------------------------------------------------------------
// Scratch-free variant: the same sums with every device buffer taken from
// one file-scope array instead of cudaMalloc.  The array is set up once
// per device (cudaGetSymbolAddress with that device current) by the first
// call made on it; make that first call before any stream capture starts.
// Calls share the array, so overlapping calls (several host threads, or
// a call issued while another is in flight) race; calls from one thread
// are serialised by the synchronisation at the end of each call, which
// also runs when a call fails after enqueueing work.
// ---------------------------------------------------------------------
static __device__ __align__(256) unsigned char ffStaticScratch[ALISGPU_FF_STATIC_BYTES];
#define FF_MAX_DEVICES 64
static unsigned char *ffStaticBase[FF_MAX_DEVICES];
static std::once_flag ffStaticOnce[FF_MAX_DEVICES];
static cudaError_t ffStaticErr[FF_MAX_DEVICES];

extern "C" int alisgpu_farfield_sums_static(alisgpu_phaser *p, int f, const alisgpu_farfield_geom *g, int nA,
                                            const double *T, int nk, const unsigned char *present,
                                            const double *kx, const double *ky, double *out)
{
	ALIS_BATCH_GUARD();
	if (!p || !g || nA < 0 || !T || !present || !kx || !ky || !out || nk < 0)
		return alisgpu__fail(ALISGPU_EINVAL, "farfield_sums_static: bad argument");
	if (!nA) return ALISGPU_OK;
	alisgpu__bind_phaser(p);
	FFParams P;
	memset(&P, 0, sizeof P);
	size_t smem = 0;
	int rc = ffFaces(p, f, g, nk, P, smem, "farfield_sums_static");
	if (rc) return rc;
	int dev = 0;
	ALIS_CUDA(cudaGetDevice(&dev));
	if (dev < 0 || dev >= FF_MAX_DEVICES) return alisgpu__fail(ALISGPU_ERANGE, "farfield_sums_static: device %d beyond %d", dev, FF_MAX_DEVICES);
	// the device address of the array, looked up once per device with that
	// device current (the host-side symbol is not a device address)
	std::call_once(ffStaticOnce[dev], [dev]() {
		void *base = 0;
		ffStaticErr[dev] = cudaGetSymbolAddress(&base, ffStaticScratch);
		if (ffStaticErr[dev] == cudaSuccess) ffStaticBase[dev] = (unsigned char *)base;
	});
	if (ffStaticErr[dev] != cudaSuccess) return alisgpu__check(ffStaticErr[dev], "farfield_sums_static: cudaGetSymbolAddress");
	// carve the scratch: tables, test fields, flags, wave numbers, partials
	size_t off = 0;
	auto take = [&](size_t bytes) -> size_t { size_t at = off; off += (bytes + 255) & ~(size_t)255; return at; };
	const size_t xb = (size_t)g->xLen * sizeof(double), yb = (size_t)g->yLen * sizeof(double), zb = (size_t)g->zLen * sizeof(double);
	size_t oTab[10];
	for (int q = 0; q < 4; q++) oTab[q] = take(xb);
	for (int q = 4; q < 8; q++) oTab[q] = take(yb);
	for (int q = 8; q < 10; q++) oTab[q] = take(zb);
	const size_t oT = take((size_t)nA * 6 * nk * sizeof(double2));
	const size_t oPr = take((size_t)nA * 6);
	const size_t oKx = take((size_t)nA * sizeof(double)), oKy = take((size_t)nA * sizeof(double));
	const size_t oPart = take((size_t)nA * 6 * sizeof(double2));
	if (off > (size_t)ALISGPU_FF_STATIC_BYTES)
		return alisgpu__fail(ALISGPU_ERANGE, "farfield_sums_static: %d directions need %zu bytes of scratch, the static buffer holds %u; "
		                     "split the batch", nA, off, (unsigned)ALISGPU_FF_STATIC_BYTES);
	cudaStream_t st = alisgpu__stream();
	unsigned char *base = ffStaticBase[dev];
	const double *src[10] = { g->xE, g->xH, g->dxE, g->dxH, g->yE, g->yH, g->dyE, g->dyH, g->dzE, g->dzH };
	const size_t len[10] = { xb, xb, xb, xb, yb, yb, yb, yb, zb, zb };
	const double *dev10[10];
	cudaError_t e = cudaSuccess;
	for (int q = 0; q < 10; q++) {
		dev10[q] = (const double *)(base + oTab[q]);
		if (len[q] && e == cudaSuccess) e = cudaMemcpyAsync(base + oTab[q], src[q], len[q], cudaMemcpyHostToDevice, st);
	}
	P.g = *g;
	P.g.xE = dev10[0], P.g.xH = dev10[1], P.g.dxE = dev10[2], P.g.dxH = dev10[3];
	P.g.yE = dev10[4], P.g.yH = dev10[5], P.g.dyE = dev10[6], P.g.dyH = dev10[7];
	P.g.dzE = dev10[8], P.g.dzH = dev10[9];
	P.nk = nk;
	if (e == cudaSuccess) e = cudaMemcpyAsync(base + oT, T, (size_t)nA * 6 * nk * sizeof(double2), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(base + oPr, present, (size_t)nA * 6, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(base + oKx, kx, (size_t)nA * sizeof(double), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(base + oKy, ky, (size_t)nA * sizeof(double), cudaMemcpyHostToDevice, st);
	// the partials of missing faces must read as zero
	if (e == cudaSuccess) e = cudaMemsetAsync(base + oPart, 0, (size_t)nA * 6 * sizeof(double2), st);
	P.T = (const double2 *)(base + oT);
	P.present = base + oPr;
	P.kx = (const double *)(base + oKx), P.ky = (const double *)(base + oKy);
	P.part = (double2 *)(base + oPart);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(k_farfield, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess && P.nface) {
		dim3 grid(nA, P.nface);
		int slot = alisgpu__prof_start();
		k_farfield<<<grid, FF_THREADS, smem, st>>>(P);
		alisgpu__prof_stop(slot, ALISGPU_K_FARFIELD);
		alisgpu__count_launch();
		e = cudaGetLastError();
	}
	// out[(a*6 + face)*2 + re/im] has the layout of the double2 partials
	if (e == cudaSuccess) e = cudaMemcpyAsync(out, base + oPart, (size_t)nA * 6 * sizeof(double2), cudaMemcpyDeviceToHost, st);
	// on success and on failure alike, nothing of this call is left in flight
	cudaError_t es = cudaStreamSynchronize(st);
	if (e == cudaSuccess) e = es;
	if (e != cudaSuccess) return alisgpu__check(e, "farfield_sums_static");
	return ALISGPU_OK;
}
