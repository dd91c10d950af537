// common.cuh -- shared device-side definitions of the GB300 ALiS engine.
//
// Storage of one world on the device: every field component (E, H, the
// eps^-1 maps) uses the same halo'd layout over
// [iMIN-1, iMAX+1] x [jMIN-1, jMAX+1] x [kMIN-1, kMAX+1]; k is fastest and
// each (i, j) row starts kOff = 31 floats before a 128-byte boundary so
// that k = kMIN is 128-byte aligned (row pitch is a multiple of 32
// floats).  Smaller arrays (CPML psi slabs, ADE maps and currents) are
// compact box arrays with their own strides.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include "alisgpu.h"

#define ALIS_KOFF 31
#define ALIS_MAXPOLES 6
#define ALIS_MAXTFSF 4

struct Layout {
	int i0, j0, k0;          // first stored index (MIN - 1)
	int ni, nj, nk;          // stored extents
	long long sj, si;        // row pitch and plane pitch (floats)
	__host__ __device__ long long at(int i, int j, int k) const {
		return (long long)(i - i0) * si + (long long)(j - j0) * sj + (k - k0) + ALIS_KOFF;
	}
	size_t elems() const { return (size_t)ni * (size_t)si; }
};

// compact box array: element (i,j,k) at p[(i-i0)*si + (j-j0)*sj + (k-k0)]
struct BoxArr {
	float *p;
	int i0, i1, j0, j1, k0, k1;
	long long sj, si;
	__host__ __device__ long long at(int i, int j, int k) const {
		return (long long)(i - i0) * si + (long long)(j - j0) * sj + (k - k0);
	}
	__host__ __device__ bool has(int i, int j, int k) const {
		return i >= i0 && i <= i1 && j >= j0 && j <= j1 && k >= k0 && k <= k1;
	}
	size_t elems() const { return (size_t)(1 + i1 - i0) * (size_t)si; }
};

// one dispersive object as the kernels see it
struct DevObj {
	int i0, i1, j0, j1, k0, k1;          // box of maps and currents
	int NJ, NK;
	float a[3];
	int cond;                             // 0: no conductivity; 1: the reference's factor; 2: its compensated form
	float JJ[ALIS_MAXPOLES][3], JK[ALIS_MAXPOLES][3], JE[ALIS_MAXPOLES][3];
	float KJ[ALIS_MAXPOLES][3], KK[ALIS_MAXPOLES][3], KE[ALIS_MAXPOLES][3];
	float *fill[3];                       // compact over the box
	float *J[2][ALIS_MAXPOLES][3];        // [m][pole][axis]
	float *K[2][ALIS_MAXPOLES][3];
	long long sj, si;                     // strides of the box arrays
};

// TFSF box as the main-world kernels see it
struct DevTfsf {
	int iMin, iMax, jMin, jMax, kMin, kMax;
	int iMIN, iMAX, jMIN, jMAX, kMIN, kMAX;
	int auxIMAX, auxJMAX, aliasX, aliasY;
	Layout L;                             // layout of the auxiliary world
	const float *G[2][3];                 // aux H (E step) or aux E (H step), [m][comp]
	float dtdMin[3], dtdMax[3];           // dt/ds at the min face and max face
};

// FP16 field storage of a world (alisgpu_world_set_storage): each E and H
// component holds IEEE half values times 2^e, one exponent per component
// and plane of the layout.  Per field and step parity the world keeps the
// exponents readers use (ex; ghost copies that move whole planes point a
// plane at another's), the exponents the step computed (exK) and 2^ex as
// floats (sc), all indexed [comp * L.ni + (i - L.i0)]; the inverse scales
// 2^-e of the field's next step (inv); the step's largest magnitudes,
// spread over HALF_SLOTS words per (component, plane) so that the plane's
// warps update different ones, at [(comp * L.ni + plane) * HALF_SLOTS +
// slot]; and the table a half step of the field reads its scales from,
// HALF_TAB floats per plane: the other field's scales at the plane and at
// the plane + ALT, its own scales as stored, its inverse scales.  After
// each half step a small kernel (k_half_next) turns the maxima into the
// field's next exponents and makes the other field's table.
#define HALF_SLOTS 32
#define HALF_TAB 12
#define HALF_E0 (-11)
#define HALF_EMIN (-100)
#define HALF_EMAX 100
struct HalfPlanes {
	const float *tab;                     // the step's scale table
	unsigned *mCur;                       // the step's maxima
};

// the exponent a half step stores with, from the float bits m of the
// largest magnitude of the previous step: M = f 2^x, f in [0.5, 1), gives
// x - 11 (M 2^-e in [2^10, 2^11)); subnormal M gives the minimum
__host__ __device__ __forceinline__ int halfExponent(unsigned m)
{
	if (m == 0) return HALF_E0;
	if (m >= 0x7f800000u) return HALF_EMAX;
	if (m < 0x00800000u) return HALF_EMIN;
	const int e = (int)(m >> 23) - 126 - 11;
	return e < HALF_EMIN ? HALF_EMIN : e > HALF_EMAX ? HALF_EMAX : e;
}

// 2^e as a float, e in [-126, 127]
__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((unsigned)(127 + e) << 23); }

// a half value of p times s (s a power of two: exact)
__device__ __forceinline__ float halfAt(const void *p, long long c, float s)
{
	return __half2float(__ushort_as_half(((const unsigned short *)p)[c])) * s;
}

// v 2^-e (inv = 2^-e) rounded to the nearest half, values beyond the half
// range saturated at +-65504 (cvt .satfinite)
__device__ __forceinline__ unsigned short halfOf(float v, float inv)
{
	unsigned short h;
	asm("cvt.rn.satfinite.f16.f32 %0, %1;" : "=h"(h) : "f"(v * inv));
	return h;
}

struct HalfStepParams {
	int iMIN, iMAX, jMIN, jMAX, kMIN, kMAX;
	int iMin, iMax, jMin, jMax, kMin, kMax;
	Layout L;
	int m;
	float *F[3];
	const float *G[3];
	const float *C[3];                    // eps^-1 maps (E half step) or null
	const void *matIdx;                   // per cell index into matTab (or null): the
	const float4 *matTab;                 // distinct (C[0], C[1], C[2]) triples
	int matWide;                          // index of 16 bits (else 8)
	const float *dtd[3];                  // dt/ds tables indexed from MIN
	const float *cp[9];                   // CPML b/c tables (xP,xPy,xPz,yP,yPz,yPx,zP,zPx,zPy)
	int slabOn[6];                        // xMin,yMin,zMin,xMax,yMax,zMax
	int slabLo[6], slabHi[6];             // slab range along the face axis
	BoxArr psi[6][2];                     // (Py,Pz) (Pz,Px) (Px,Py) per face
	int nobj;
	const DevObj *obj;
	int ntfsf;
	DevTfsf tf[ALIS_MAXTFSF];
	float *Fother[3];                     // E of set m during the H step (ADE drive)
	unsigned int *err;                    // device error word
	// per-axis classification of cells (indexed from MIN): bits 0-7 object
	// n's range, bit 8 any object n >= 8, bit 12 within a TFSF box's index
	// range (one cell of margin), bit 13/14 CPML slab of the min/max face,
	// bit 15 TFSF face plane.  A cell takes TFSF corrections only where all
	// three axes have bit 12 and one has bit 15 (tfsfBits).
	const unsigned short *cls[3];
	// worlds with more than 8 objects: per tile of ALIS_TILE_K cells along
	// k x ALIS_TILE_J rows x 1 plane, the objects whose box meets it, in
	// list order (tileObj[tileStart[t] .. tileStart[t + 1]]); tiles
	// numbered (plane * tjn + j tile) * tkn + k tile, from MIN
	const int *tileStart, *tileObj;
	int tjn, tkn;
	HalfPlanes h;                         // FP16 storage (the HALF instances)
};
#define ALIS_TILE_K 32
#define ALIS_TILE_J 8
#define CLS_OBJ8 0x100u
#define CLS_TFSF_IN 0x1000u
#define CLS_PML_LO 0x2000u
#define CLS_PML_HI 0x4000u
#define CLS_TFSF 0x8000u

// CLS_TFSF where the cell may lie on a TFSF box face (a face plane in
// one axis, the box's range in the others), else 0
__device__ __forceinline__ unsigned tfsfBits(unsigned bi, unsigned bj, unsigned bk)
{
	return (bi & bj & bk & CLS_TFSF_IN) ? (bi | bj | bk) & CLS_TFSF : 0u;
}

// the eps^-1 triple of cell c from the material index
__device__ __forceinline__ float4 matTriple(const HalfStepParams &P, int c)
{
	const unsigned q = P.matWide ? (unsigned)__ldg((const unsigned short *)P.matIdx + c)
	                             : (unsigned)__ldg((const unsigned char *)P.matIdx + c);
	return __ldg(P.matTab + q);
}

// ---- launch bookkeeping ----
extern "C" void alisgpu__count_launch(void);
// event pair around a launch when profiling is on: slot = prof_start(); launch; prof_stop(slot, kind)
extern "C" int alisgpu__prof_start(void);
extern "C" void alisgpu__prof_stop(int slot, int kind);
extern "C" cudaStream_t alisgpu__stream(void);
extern "C" int alisgpu__fail(int code, const char *fmt, ...);
extern "C" int alisgpu__check(cudaError_t e, const char *what);
#define ALIS_CUDA(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return alisgpu__check(e_, #call); } while (0)

// Device memory of worlds, phasers and their scratch comes from the
// stream-ordered pool on the main stream of the world's group: freeing a
// world that finished does not wait for the work of every other world.
// An injected allocation failure (alisgpu_inject_alloc_failures) is taken here.
extern "C" int alisgpu__alloc_denied(void);
template <class T>
static inline cudaError_t alisgpu__mallocAsync(T **p, size_t bytes)
{
	if (alisgpu__alloc_denied()) { *p = 0; return cudaErrorMemoryAllocation; }
	return cudaMallocAsync((void **)p, bytes, alisgpu__stream());
}
static inline cudaError_t alisgpu__freeAsync(void *p)
{
	return p ? cudaFreeAsync(p, alisgpu__stream()) : cudaSuccess;
}
