// voxel.cu -- voxelization of an object list on the GPU.
//
// The material maps of putObjectArray (reference src/object.c:70-121,
// 229-279, 339-405, shapes src/shapes.c:9-221) computed where the cells
// are: the index box of every object (first object owning each cell
// centre), the sub-pixel fill factors at the staggered Yee positions, and
// the harmonic eps^-1 accumulation in reverse list order.  Bit-identical
// to the host restatement: the shape predicates repeat its float and
// double arithmetic, the coordinates of every sample position come from
// host tables (the world's own itox, so graded grids and user grid
// functions are covered), and the trigonometric values of rotations and
// rotational lattices are host glibc results.  Built with FMA
// contraction off.
#include <cooperative_groups.h>
#include <cstring>
#include <vector>
#include <algorithm>
#include "common.cuh"

namespace cg = cooperative_groups;

typedef alisgpu_vox_node VoxNode;

struct VoxWorld {
	const VoxNode *node;
	const float *pool;                     // trigonometric values of rotational lattices
	const float *tab[3];                   // coordinates per axis: [(n - lo) * 3 + kind][slot]
	int lo[3], nslot, subN;
	int iMIN, iMAX, jMIN, jMAX, kMIN, kMAX;
	unsigned int *err;
};

#define VOX_DEPTH 12

// sample coordinate: base index n of kind (0: n - 1/2, 1: n, 2: n + 1/2)
// moved by the offset in slot s (0: none, 1: -1/2, 2: +1/2, 3: -h, 4: +h,
// 5 + q: the q-th sub-grid offset)
__device__ __forceinline__ float coord(const VoxWorld &V, int a, int n, int kind, int s)
{
	return V.tab[a][((n - V.lo[a]) * 3 + kind) * V.nslot + s];
}

struct Bx { float xMin, xMax, yMin, yMax, zMin, zMax; };

// bounding box of a basic shape, with the reference's precedence quirk
// in the centre form (see the host restatement)
__device__ __forceinline__ Bx boundsOf(const float f[3][3])
{
	Bx b;
	if (__fsub_rn(f[2][1], f[2][0]) != 0) {
		b.xMin = f[0][0], b.xMax = f[0][1], b.yMin = f[1][0], b.yMax = f[1][1], b.zMin = f[2][0], b.zMax = f[2][1];
	} else {
		b.xMin = __fsub_rn(f[0][0], f[1][0]);
		b.yMin = __fsub_rn(f[0][1], f[1][1]) != 0 ? f[1][1] : f[1][0];
		b.zMin = __fsub_rn(f[0][2], f[1][2]) != 0 ? f[1][2] : f[1][0];
		b.xMax = __fadd_rn(f[0][0], f[1][0]);
		b.yMax = __fadd_rn(f[0][1], f[1][1]) != 0 ? f[1][1] : f[1][0];
		b.zMax = __fadd_rn(f[0][2], f[1][2]) != 0 ? f[1][2] : f[1][0];
	}
	return b;
}

__device__ __forceinline__ float U(float v, float lo, float hi)
{
	return __fdiv_rn(__fsub_rn(__fsub_rn(__fmul_rn(2.0f, v), lo), hi), __fsub_rn(hi, lo));
}
__device__ __forceinline__ float sqf(float v) { return __fmul_rn(v, v); }
__device__ __forceinline__ bool IN(float v, float lo, float hi) { return lo <= v && v <= hi; }
__device__ __forceinline__ bool INOPEN(float v, float lo, float hi) { return lo < v && v < hi; }

// coordinate folded into a lattice's unit cell (double arithmetic as in the host)
__device__ __forceinline__ float foldAxis(float v, float a, float c, float lo, float hi)
{
	if (c != 0) v = __double2float_rn(__dadd_rn((double)v, __dmul_rn(__dmul_rn(0.5, (double)__fsub_rn(c, 1.0f)), (double)a)));
	const double t = __dadd_rn((double)v, __dmul_rn(0.5, (double)__fsub_rn(__fsub_rn(a, lo), hi)));
	const float q = (float)floor(__ddiv_rn(t, (double)a));
	// MAX(0, MIN(q, c - 1)) as the host macros compute it
	const float c1 = __fsub_rn(c, 1.0f), mn = q < c1 ? q : c1;
	const float m = c > 0 ? (0 > mn ? 0.0f : mn) : q;
	return __fsub_rn(v, __fmul_rn(a, m));
}

// membership in a basic shape (reference src/shapes.c:17-123)
__device__ __forceinline__ bool inBasic(const VoxNode &O, float x, float y, float z)
{
	switch (O.type) {
	case ALISGPU_SHAPE_BOX: { Bx b = boundsOf(O.f); return IN(x, b.xMin, b.xMax) && IN(y, b.yMin, b.yMax) && IN(z, b.zMin, b.zMax); }
	case ALISGPU_SHAPE_BALL: { Bx b = boundsOf(O.f);
		return __fadd_rn(__fadd_rn(sqf(U(x, b.xMin, b.xMax)), sqf(U(y, b.yMin, b.yMax))), sqf(U(z, b.zMin, b.zMax))) < 1; }
	case ALISGPU_SHAPE_DIAMOND: { Bx b = boundsOf(O.f);
		return __fadd_rn(__fadd_rn(fabsf(U(x, b.xMin, b.xMax)), fabsf(U(y, b.yMin, b.yMax))), fabsf(U(z, b.zMin, b.zMax))) <= 1; }
	case ALISGPU_SHAPE_BICONEX: { Bx b = boundsOf(O.f);
		return __dadd_rn((double)fabsf(U(x, b.xMin, b.xMax)), __dsqrt_rn((double)__fadd_rn(sqf(U(y, b.yMin, b.yMax)), sqf(U(z, b.zMin, b.zMax))))) < 1; }
	case ALISGPU_SHAPE_BICONEY: { Bx b = boundsOf(O.f);
		return __dadd_rn((double)fabsf(U(y, b.yMin, b.yMax)), __dsqrt_rn((double)__fadd_rn(sqf(U(z, b.zMin, b.zMax)), sqf(U(x, b.xMin, b.xMax))))) < 1; }
	case ALISGPU_SHAPE_BICONEZ: { Bx b = boundsOf(O.f);
		return __dadd_rn((double)fabsf(U(z, b.zMin, b.zMax)), __dsqrt_rn((double)__fadd_rn(sqf(U(x, b.xMin, b.xMax)), sqf(U(y, b.yMin, b.yMax))))) < 1; }
	case ALISGPU_SHAPE_RODX: { Bx b = boundsOf(O.f); return IN(x, b.xMin, b.xMax) && __fadd_rn(sqf(U(y, b.yMin, b.yMax)), sqf(U(z, b.zMin, b.zMax))) < 1; }
	case ALISGPU_SHAPE_RODY: { Bx b = boundsOf(O.f); return IN(y, b.yMin, b.yMax) && __fadd_rn(sqf(U(x, b.xMin, b.xMax)), sqf(U(z, b.zMin, b.zMax))) < 1; }
	case ALISGPU_SHAPE_RODZ: { Bx b = boundsOf(O.f); return IN(z, b.zMin, b.zMax) && __fadd_rn(sqf(U(x, b.xMin, b.xMax)), sqf(U(y, b.yMin, b.yMax))) < 1; }
	case ALISGPU_SHAPE_DRODX: { Bx b = boundsOf(O.f); return IN(x, b.xMin, b.xMax) && __fadd_rn(fabsf(U(y, b.yMin, b.yMax)), fabsf(U(z, b.zMin, b.zMax))) <= 1; }
	case ALISGPU_SHAPE_DRODY: { Bx b = boundsOf(O.f); return IN(y, b.yMin, b.yMax) && __fadd_rn(fabsf(U(z, b.zMin, b.zMax)), fabsf(U(x, b.xMin, b.xMax))) <= 1; }
	case ALISGPU_SHAPE_DRODZ: { Bx b = boundsOf(O.f); return IN(z, b.zMin, b.zMax) && __fadd_rn(fabsf(U(x, b.xMin, b.xMax)), fabsf(U(y, b.yMin, b.yMax))) <= 1; }
	case ALISGPU_SHAPE_HRODXY: { Bx b = boundsOf(O.f); return IN(x, b.xMin, b.xMax) && INOPEN(z, b.zMin, b.zMax) &&
		__fadd_rn(fabsf(U(z, b.zMin, b.zMax)), __fmul_rn(fabsf(U(y, b.yMin, b.yMax)), 2.0f)) < 2; }
	case ALISGPU_SHAPE_HRODYZ: { Bx b = boundsOf(O.f); return IN(y, b.yMin, b.yMax) && INOPEN(x, b.xMin, b.xMax) &&
		__fadd_rn(fabsf(U(x, b.xMin, b.xMax)), __fmul_rn(fabsf(U(z, b.zMin, b.zMax)), 2.0f)) < 2; }
	case ALISGPU_SHAPE_HRODZX: { Bx b = boundsOf(O.f); return IN(z, b.zMin, b.zMax) && INOPEN(y, b.yMin, b.yMax) &&
		__fadd_rn(fabsf(U(y, b.yMin, b.yMax)), __fmul_rn(fabsf(U(x, b.xMin, b.xMax)), 2.0f)) < 2; }
	case ALISGPU_SHAPE_HRODXZ: { Bx b = boundsOf(O.f); return IN(x, b.xMin, b.xMax) && INOPEN(y, b.yMin, b.yMax) &&
		__fadd_rn(fabsf(U(y, b.yMin, b.yMax)), __fmul_rn(fabsf(U(z, b.zMin, b.zMax)), 2.0f)) < 2; }
	case ALISGPU_SHAPE_HRODYX: { Bx b = boundsOf(O.f); return IN(y, b.yMin, b.yMax) && INOPEN(z, b.zMin, b.zMax) &&
		__fadd_rn(fabsf(U(z, b.zMin, b.zMax)), __fmul_rn(fabsf(U(x, b.xMin, b.xMax)), 2.0f)) < 2; }
	case ALISGPU_SHAPE_HRODZY: { Bx b = boundsOf(O.f); return IN(z, b.zMin, b.zMax) && INOPEN(x, b.xMin, b.xMax) &&
		__fadd_rn(fabsf(U(x, b.xMin, b.xMax)), __fmul_rn(fabsf(U(y, b.yMin, b.yMax)), 2.0f)) < 2; }
	}
	return false;
}

__device__ bool inCompound(const VoxWorld &V, const VoxNode &O, float x, float y, float z, int depth);

// membership in node id: basic shapes inline, compound shapes through the
// recursive evaluator
__device__ __forceinline__ bool inNode(const VoxWorld &V, int id, float x, float y, float z, int depth)
{
	const VoxNode &O = V.node[id];
	return O.type < ALISGPU_SHAPE_TRANSLATION ? inBasic(O, x, y, z) : inCompound(V, O, x, y, z, depth);
}

__device__ __noinline__ bool inLattice(const VoxWorld &V, const VoxNode &O, const float f[3][3], float x, float y, float z, int depth)
{
	const VoxNode &o = V.node[O.child];
	if (f[0][0] != 0) x = foldAxis(x, f[0][0], f[0][1], o.f[0][0], o.f[0][1]);
	if (f[1][0] != 0) y = foldAxis(y, f[1][0], f[1][1], o.f[1][0], o.f[1][1]);
	if (f[2][0] != 0) z = foldAxis(z, f[2][0], f[2][1], o.f[2][0], o.f[2][1]);
	return inNode(V, O.child, x, y, z, depth + 1);
}

// compound shapes (reference src/shapes.c:128-221): members evaluated at
// moved, rotated or folded coordinates
__device__ __noinline__ bool inCompound(const VoxWorld &V, const VoxNode &O, float x, float y, float z, int depth)
{
	if (depth >= VOX_DEPTH) { atomicOr(V.err, 16u); return false; }
	switch (O.type) {
	case ALISGPU_SHAPE_TRANSLATION:
		return inNode(V, O.child, __fsub_rn(x, O.f[0][0]), __fsub_rn(y, O.f[0][1]), __fsub_rn(z, O.f[0][2]), depth + 1);
	case ALISGPU_SHAPE_ROTATION: {
		x = __fsub_rn(x, O.f[1][0]), y = __fsub_rn(y, O.f[1][1]), z = __fsub_rn(z, O.f[1][2]);
		const float cx = O.rot[0], sx = O.rot[1], cy = O.rot[2], sy = O.rot[3], cz = O.rot[4], sz = O.rot[5];
		const float u = __fadd_rn(__fmul_rn(cz, x), __fmul_rn(sz, y)), v = __fsub_rn(__fmul_rn(cz, y), __fmul_rn(sz, x));
		const float w = __fadd_rn(__fmul_rn(cy, z), __fmul_rn(sy, u));
		return inNode(V, O.child, __fsub_rn(__fmul_rn(cy, u), __fmul_rn(sy, z)), __fadd_rn(__fmul_rn(cx, v), __fmul_rn(sx, w)),
		              __fsub_rn(__fmul_rn(cx, w), __fmul_rn(sx, v)), depth + 1);
	}
	case ALISGPU_SHAPE_COMBINATION:
		for (int n = 0; n < O.nchild; n++) if (inNode(V, O.child + n, x, y, z, depth + 1)) return true;
		return false;
	case ALISGPU_SHAPE_INTERSECTION:
		for (int n = 0; n < O.nchild; n++) if (!inNode(V, O.child + n, x, y, z, depth + 1)) return false;
		return true;
	case ALISGPU_SHAPE_DIFFERENCE:
		if (!inNode(V, O.child, x, y, z, depth + 1)) return false;
		for (int n = 1; n < O.nchild; n++) if (inNode(V, O.child + n, x, y, z, depth + 1)) return false;
		return true;
	case ALISGPU_SHAPE_LATTICE:
		return inLattice(V, O, O.f, x, y, z, depth);
	case ALISGPU_SHAPE_DLATTICE: {
		if (inLattice(V, O, O.f, x, y, z, depth)) return true;
		float f[3][3];
		memcpy(f, O.f, sizeof f);
		for (int d = 0; d < 3; d++) if (f[d][0] != 0) f[d][1] = __fsub_rn(f[d][1], f[d][1] != 0 ? 1.0f : 2.0f);
		return inLattice(V, O, f, x, y, z, depth);
	}
	case ALISGPU_SHAPE_CLATTICEX: case ALISGPU_SHAPE_CLATTICEY: case ALISGPU_SHAPE_CLATTICEZ: {
		const int N = (int)O.f[0][0];
		const float a0 = O.f[1][0], b0 = O.f[1][1];
		for (int n = 0; n < N; n++) {
			const float c = V.pool[O.trig + n], s = V.pool[O.trig + N + n];
			if (O.type == ALISGPU_SHAPE_CLATTICEX) {
				const float dy = __fsub_rn(y, a0), dz = __fsub_rn(z, b0);
				if (inNode(V, O.child, x, __fadd_rn(__fadd_rn(__fmul_rn(dy, c), __fmul_rn(dz, s)), a0),
				           __fadd_rn(__fsub_rn(__fmul_rn(dz, c), __fmul_rn(dy, s)), b0), depth + 1)) return true;
			} else if (O.type == ALISGPU_SHAPE_CLATTICEY) {
				const float dx = __fsub_rn(x, a0), dz = __fsub_rn(z, b0);
				if (inNode(V, O.child, __fadd_rn(__fadd_rn(__fmul_rn(dx, c), __fmul_rn(dz, s)), a0), y,
				           __fadd_rn(__fsub_rn(__fmul_rn(dz, c), __fmul_rn(dx, s)), b0), depth + 1)) return true;
			} else {
				const float dx = __fsub_rn(x, a0), dy = __fsub_rn(y, b0);
				if (inNode(V, O.child, __fadd_rn(__fadd_rn(__fmul_rn(dx, c), __fmul_rn(dy, s)), a0),
				           __fadd_rn(__fsub_rn(__fmul_rn(dy, c), __fmul_rn(dx, s)), b0), z, depth + 1)) return true;
			}
		}
		return false;
	}
	}
	return false;
}

// 1 if the sample belongs to object o and to none listed before it
__device__ __forceinline__ float owned(const VoxWorld &V, int o, float x, float y, float z)
{
	if (!inNode(V, o, x, y, z, 0)) return 0;
	while (o--) if (inNode(V, o, x, y, z, 0)) return 0;
	return 1;
}

// sample position of one axis: base (n, kind) plus the slot's offset
struct Pos { int n, kind; };

__device__ __forceinline__ float ownedAt(const VoxWorld &V, int o, Pos p[3], const int s[3])
{
	return owned(V, o, coord(V, 0, p[0].n, p[0].kind, s[0]), coord(V, 1, p[1].n, p[1].kind, s[1]), coord(V, 2, p[2].n, p[2].kind, s[2]));
}

// Sub-pixel fill factor at a (possibly staggered) position (reference
// src/object.c:70-121): binary, the edge rule for subN < 0, or the corner
// test.  A position whose corners disagree with its centre needs the
// subN^3 supersampling: it returns false, and the warp-wide pass computes
// the value.
__device__ bool fillFirst(const VoxWorld &V, int o, Pos p[3], float &out)
{
	const int s0[3] = { 0, 0, 0 };
	const float n = ownedAt(V, o, p, s0);
	const int subN = V.subN;
	out = n;
	if (subN < 2) {
		if (n != 0 || subN >= 0) return true;
		// the staggered axis: pairs of samples half a cell to either side
		const bool si = p[0].kind != 1, sj = p[1].kind != 1, sk = p[2].kind != 1;
		// slots: 1 = -1/2, 2 = +1/2
		#define OWN(a, b, c) ([&] { const int s_[3] = { a, b, c }; return ownedAt(V, o, p, s_) != 0; }())
		bool one = false;
		if (si) {
			one = (OWN(1, 1, 0) && OWN(2, 1, 0)) || (OWN(1, 2, 0) && OWN(2, 2, 0)) ||
			      (OWN(1, 0, 1) && OWN(2, 0, 1)) || (OWN(1, 0, 2) && OWN(2, 0, 2));
		} else if (sj) {
			one = (OWN(1, 1, 0) && OWN(1, 2, 0)) || (OWN(2, 1, 0) && OWN(2, 2, 0)) ||
			      (OWN(0, 1, 1) && OWN(0, 2, 1)) || (OWN(0, 1, 2) && OWN(0, 2, 2));
		} else if (sk) {
			one = (OWN(1, 0, 1) && OWN(1, 0, 2)) || (OWN(2, 0, 1) && OWN(2, 0, 2)) ||
			      (OWN(0, 1, 1) && OWN(0, 1, 2)) || (OWN(0, 2, 1) && OWN(0, 2, 2));
		}
		#undef OWN
		out = one ? 1.0f : 0.0f;
		return true;
	}
	// corners: slots 3 (-h) and 4 (+h)
	for (int a = 0; a < 2; a++) for (int b = 0; b < 2; b++) for (int d = 0; d < 2; d++) {
		const int s[3] = { 3 + a, 3 + b, 3 + d };
		if (ownedAt(V, o, p, s) != n) return false;
	}
	return true;
}

// --- kernels ---

// first object owning each cell centre -> per-object index box
__global__ void k_vox_bounds(const VoxWorld V, int nobj, int *box)
{
	const int nj = 1 + V.jMAX - V.jMIN, nk = 1 + V.kMAX - V.kMIN;
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long long)(1 + V.iMAX - V.iMIN) * nj * nk) return;
	const int i = V.iMIN + (int)(t / ((long long)nj * nk)), j = V.jMIN + (int)((t / nk) % nj), k = V.kMIN + (int)(t % nk);
	const float x = coord(V, 0, i, 1, 0), y = coord(V, 1, j, 1, 0), z = coord(V, 2, k, 1, 0);
	int o = 0;
	while (o < nobj && !inNode(V, o, x, y, z, 0)) o++;
	if (o < nobj) {
		int *b = box + 6 * o;
		atomicMin(b + 0, i), atomicMax(b + 1, i), atomicMin(b + 2, j), atomicMax(b + 3, j), atomicMin(b + 4, k), atomicMax(b + 5, k);
	}
}

// The positions of one fill request.  Box: the three staggered samples
// (i - 1/2, j, k), (i, j - 1/2, k), (i, j, k - 1/2) of every cell of
// [i0,i1] x [j0,j1] x [k0,k1] into out[0..2].  Edge plane (edge = axis):
// the sample at index i0 + 1/2 of that axis over [j0,j1] x [k0,k1] of the
// other two axes in increasing order, into out[0].
struct FillJob {
	int i0, i1, j0, j1, k0, k1, edge;
	float *out[3];
	unsigned long long *list;              // positions left for supersampling: t * 4 + component
	unsigned int *count;
};

__device__ __forceinline__ void jobPos(const FillJob &J, long long t, int c, Pos p[3])
{
	const int nk = 1 + J.k1 - J.k0;
	if (J.edge < 0) {
		const long long nj = 1 + J.j1 - J.j0;
		const int i = J.i0 + (int)(t / (nj * nk)), j = J.j0 + (int)((t / nk) % nj), k = J.k0 + (int)(t % nk);
		p[0] = { i, c == 0 ? 0 : 1 }, p[1] = { j, c == 1 ? 0 : 1 }, p[2] = { k, c == 2 ? 0 : 1 };
	} else {
		const int u = J.j0 + (int)(t / nk), v = J.k0 + (int)(t % nk);
		if (J.edge == 0) p[0] = { J.i0, 2 }, p[1] = { u, 1 }, p[2] = { v, 1 };
		else if (J.edge == 1) p[0] = { u, 1 }, p[1] = { J.i0, 2 }, p[2] = { v, 1 };
		else p[0] = { u, 1 }, p[1] = { v, 1 }, p[2] = { J.i0, 2 };
	}
}

// first pass: one thread per position; the positions whose corners
// disagree go to the list (warp-aggregated append)
__global__ void k_vox_fill(const VoxWorld V, const FillJob J, int o, long long total)
{
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= total) return;
	const int comps = J.edge < 0 ? 3 : 1;
	for (int c = 0; c < comps; c++) {
		Pos p[3];
		jobPos(J, t, c, p);
		float f;
		const bool done = fillFirst(V, o, p, f);
		J.out[c][t] = f;
		if (!done) {
			cg::coalesced_group g = cg::coalesced_threads();
			unsigned int base = 0;
			if (g.thread_rank() == 0) base = atomicAdd(J.count, g.size());
			base = g.shfl(base, 0);
			J.list[base + g.thread_rank()] = (unsigned long long)t * 4 + c;
		}
	}
}

// second pass: one warp per listed position, the subN^3 samples spread
// over the lanes.  The reference sums 0/1 samples in float, exact below
// 2^24 samples, so the integer count is the same value in any order.
__global__ void k_vox_refine(const VoxWorld V, const FillJob J, int o)
{
	const unsigned int n = *J.count;
	const int lane = threadIdx.x & 31, subN = V.subN, s3 = subN * subN * subN;
	for (unsigned int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += (gridDim.x * blockDim.x) >> 5) {
		const unsigned long long item = J.list[w];
		const int c = (int)(item & 3);
		const long long t = (long long)(item >> 2);
		Pos p[3];
		jobPos(J, t, c, p);
		int cnt = 0;
		for (int q = lane; q < s3; q += 32) {
			const int s[3] = { 5 + q / (subN * subN), 5 + (q / subN) % subN, 5 + q % subN };
			cnt += ownedAt(V, o, p, s) != 0;
		}
		cnt = __reduce_add_sync(0xffffffffu, cnt);
		if (lane == 0) J.out[c][t] = __fdiv_rn((float)cnt, (float)s3);
	}
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
struct alisgpu_voxelizer {
	VoxWorld V;
	VoxNode *dNode;
	float *dPool, *dTab[3];
	unsigned int *dErr;
	float *dOut;                           // fill scratch: 3 floats, 3 list entries per cell
	unsigned long long *dList;
	unsigned int *dCount;
	size_t cap;                            // cells the scratch holds
	int refineBlocks;
};

// per-thread stack for the recursion through compound shapes: the
// kernel's own frame and one frame of the compound evaluator and of the
// lattice fold per level of nesting (raised once, never lowered: a change
// of the limit waits for the whole device)
#define VOX_STACK_BASE 1024
#define VOX_STACK_LEVEL 384

static void vfree(void *p)
{
	if (p) cudaFreeAsync(p, 0);
}
// cells per fill launch (three floats and three list entries each)
#define VOX_CHUNK (1 << 23)

static int voxUpload(alisgpu_voxelizer *v, const alisgpu_vox_node *nodes, int nnode, const float *pool, int npool,
                     const float *const tab[3], const int lo[3], const int hi[3], int nslot)
{
	ALIS_CUDA(cudaMallocAsync((void **)&v->dNode, nnode * sizeof(VoxNode), 0));
	ALIS_CUDA(cudaMemcpy(v->dNode, nodes, nnode * sizeof(VoxNode), cudaMemcpyHostToDevice));
	ALIS_CUDA(cudaMallocAsync((void **)&v->dPool, (npool > 0 ? npool : 1) * sizeof(float), 0));
	if (npool > 0) ALIS_CUDA(cudaMemcpy(v->dPool, pool, npool * sizeof(float), cudaMemcpyHostToDevice));
	for (int a = 0; a < 3; a++) {
		const size_t n = (size_t)(1 + hi[a] - lo[a]) * 3 * nslot;
		ALIS_CUDA(cudaMallocAsync((void **)&v->dTab[a], n * sizeof(float), 0));
		ALIS_CUDA(cudaMemcpy(v->dTab[a], tab[a], n * sizeof(float), cudaMemcpyHostToDevice));
	}
	ALIS_CUDA(cudaMallocAsync((void **)&v->dErr, sizeof(unsigned int), 0));
	ALIS_CUDA(cudaMemset(v->dErr, 0, sizeof(unsigned int)));
	int dev = 0, sms = 0;
	ALIS_CUDA(cudaGetDevice(&dev));
	ALIS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	v->refineBlocks = 4 * sms;
	// nesting depth of the compound shapes (members come after their owner)
	std::vector<int> depth(nnode, 0);
	int deepest = 0;
	for (int n = 0; n < nnode; n++)
		for (int c = 0; c < nodes[n].nchild; c++) {
			depth[nodes[n].child + c] = depth[n] + 1;
			deepest = std::max(deepest, depth[n] + 1);
		}
	const size_t need = VOX_STACK_BASE + (size_t)VOX_STACK_LEVEL * deepest;
	size_t stack = 0;
	ALIS_CUDA(cudaDeviceGetLimit(&stack, cudaLimitStackSize));
	if (stack < need) ALIS_CUDA(cudaDeviceSetLimit(cudaLimitStackSize, need));
	return ALISGPU_OK;
}

extern "C" int alisgpu_voxelizer_create(const alisgpu_vox_node *nodes, int nnode, const float *pool, int npool,
                                        const float *const tab[3], const int lo[3], const int hi[3], int nslot, int subN,
                                        const int MIN[3], const int MAX[3], alisgpu_voxelizer **out)
{
	if (!nodes || nnode <= 0 || !tab || !lo || !hi || nslot <= 0 || !MIN || !MAX || !out || (npool > 0 && !pool))
		return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_create: bad argument");
	for (int a = 0; a < 3; a++)
		if (!tab[a] || lo[a] > MIN[a] - 1 || hi[a] < MAX[a] + 2 || MAX[a] < MIN[a])
			return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_create: coordinate table of axis %d does not cover the grid", a);
	for (int n = 0; n < nnode; n++) {
		const VoxNode &o = nodes[n];
		if (o.type < 0 || o.type >= ALISGPU_SHAPE_COUNT || (o.nchild > 0 && (o.child <= n || o.child + o.nchild > nnode)))
			return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_create: node %d malformed", n);
		if (o.type >= ALISGPU_SHAPE_CLATTICEX && o.type <= ALISGPU_SHAPE_CLATTICEZ && (int)o.f[0][0] > 0 &&
		    (o.trig < 0 || o.trig + 2 * (int)o.f[0][0] > npool))
			return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_create: node %d trigonometric values out of the pool", n);
		const bool list = o.type == ALISGPU_SHAPE_COMBINATION || o.type == ALISGPU_SHAPE_INTERSECTION;
		if (o.type == ALISGPU_SHAPE_DIFFERENCE ? o.nchild < 1 : o.type >= ALISGPU_SHAPE_TRANSLATION && !list && o.nchild != 1)
			return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_create: node %d lacks its members", n);
	}
	alisgpu_voxelizer *v = new alisgpu_voxelizer();
	const int rc = voxUpload(v, nodes, nnode, pool, npool, tab, lo, hi, nslot);
	if (rc) {
		alisgpu_voxelizer_destroy(v);
		return rc;
	}
	for (int a = 0; a < 3; a++) v->V.tab[a] = v->dTab[a], v->V.lo[a] = lo[a];
	v->V.node = v->dNode, v->V.pool = v->dPool, v->V.nslot = nslot, v->V.subN = subN, v->V.err = v->dErr;
	v->V.iMIN = MIN[0], v->V.jMIN = MIN[1], v->V.kMIN = MIN[2], v->V.iMAX = MAX[0], v->V.jMAX = MAX[1], v->V.kMAX = MAX[2];
	*out = v;
	return ALISGPU_OK;
}

extern "C" int alisgpu_voxelizer_destroy(alisgpu_voxelizer *v)
{
	if (!v) return ALISGPU_OK;
	vfree(v->dNode), vfree(v->dPool), vfree(v->dErr);
	vfree(v->dOut), vfree(v->dList), vfree(v->dCount);
	for (int a = 0; a < 3; a++) vfree(v->dTab[a]);
	delete v;
	return ALISGPU_OK;
}

static int voxCheck(alisgpu_voxelizer *v)
{
	unsigned int e = 0;
	ALIS_CUDA(cudaMemcpy(&e, v->dErr, sizeof e, cudaMemcpyDeviceToHost));
	if (e) return alisgpu__fail(ALISGPU_ERANGE, "voxelizer: %s", "shapes nested too deeply");
	return ALISGPU_OK;
}

extern "C" int alisgpu_voxelizer_bounds(alisgpu_voxelizer *v, int nobj, int *box)
{
	if (!v || nobj <= 0 || !box) return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_bounds: bad argument");
	const VoxWorld &V = v->V;
	std::vector<int> init(6 * nobj);
	for (int o = 0; o < nobj; o++) {
		int *b = &init[6 * o];
		b[0] = V.iMAX, b[1] = V.iMIN, b[2] = V.jMAX, b[3] = V.jMIN, b[4] = V.kMAX, b[5] = V.kMIN;
	}
	int *d = 0;
	ALIS_CUDA(cudaMallocAsync((void **)&d, init.size() * sizeof(int), 0));
	ALIS_CUDA(cudaMemcpy(d, init.data(), init.size() * sizeof(int), cudaMemcpyHostToDevice));
	const long long cells = (long long)(1 + V.iMAX - V.iMIN) * (1 + V.jMAX - V.jMIN) * (1 + V.kMAX - V.kMIN);
	k_vox_bounds<<<(unsigned)((cells + 127) / 128), 128>>>(V, nobj, d);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	ALIS_CUDA(cudaMemcpy(box, d, init.size() * sizeof(int), cudaMemcpyDeviceToHost));
	vfree(d);
	return voxCheck(v);
}

// one fill request: first pass, supersampling of the listed positions,
// results to the host arrays
static int voxRun(alisgpu_voxelizer *v, int o, FillJob J, long long total, float *const host[3])
{
	const int comps = J.edge < 0 ? 3 : 1;
	if ((size_t)total > v->cap) {
		vfree(v->dOut), vfree(v->dList), vfree(v->dCount);
		v->dOut = 0, v->dList = 0, v->dCount = 0, v->cap = 0;
		ALIS_CUDA(cudaMallocAsync((void **)&v->dOut, 3 * (size_t)total * sizeof(float), 0));
		ALIS_CUDA(cudaMallocAsync((void **)&v->dList, 3 * (size_t)total * sizeof(unsigned long long), 0));
		ALIS_CUDA(cudaMallocAsync((void **)&v->dCount, sizeof(unsigned int), 0));
		v->cap = (size_t)total;
	}
	for (int c = 0; c < 3; c++) J.out[c] = v->dOut + (size_t)c * total;
	J.list = v->dList, J.count = v->dCount;
	ALIS_CUDA(cudaMemsetAsync(v->dCount, 0, sizeof(unsigned int)));
	k_vox_fill<<<(unsigned)((total + 127) / 128), 128>>>(v->V, J, o, total);
	alisgpu__count_launch();
	ALIS_CUDA(cudaGetLastError());
	if (v->V.subN >= 2) {
		k_vox_refine<<<v->refineBlocks, 256>>>(v->V, J, o);
		alisgpu__count_launch();
		ALIS_CUDA(cudaGetLastError());
	}
	for (int c = 0; c < comps; c++)
		ALIS_CUDA(cudaMemcpy(host[c], J.out[c], (size_t)total * sizeof(float), cudaMemcpyDeviceToHost));
	return ALISGPU_OK;
}

extern "C" int alisgpu_voxelizer_fill(alisgpu_voxelizer *v, int o, int i0, int i1, int j0, int j1, int k0, int k1,
                                      float *fx, float *fy, float *fz)
{
	if (!v || o < 0 || !fx || !fy || !fz || i1 < i0 || j1 < j0 || k1 < k0) return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_fill: bad argument");
	// slabs of whole i planes, each written where it lies in the box arrays
	const size_t plane = (size_t)(1 + j1 - j0) * (1 + k1 - k0);
	const int slab = (int)(plane >= VOX_CHUNK ? 1 : VOX_CHUNK / plane);
	for (int a = i0; a <= i1; a += slab) {
		const int b = a + slab - 1 < i1 ? a + slab - 1 : i1;
		const size_t at = plane * (a - i0);
		FillJob J = { a, b, j0, j1, k0, k1, -1 };
		float *const host[3] = { fx + at, fy + at, fz + at };
		const int rc = voxRun(v, o, J, (long long)(plane * (1 + b - a)), host);
		if (rc) return rc;
	}
	return voxCheck(v);
}

extern "C" int alisgpu_voxelizer_fill_edge(alisgpu_voxelizer *v, int o, int axis, int n, int u0, int u1, int v0, int v1, float *out)
{
	if (!v || o < 0 || axis < 0 || axis > 2 || !out || u1 < u0 || v1 < v0) return alisgpu__fail(ALISGPU_EINVAL, "voxelizer_fill_edge: bad argument");
	FillJob J = { n, n, u0, u1, v0, v1, axis };
	float *const host[3] = { out, out, out };
	const int rc = voxRun(v, o, J, (long long)(1 + u1 - u0) * (1 + v1 - v0), host);
	return rc ? rc : voxCheck(v);
}
