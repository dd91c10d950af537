/*
 * engine.h -- internal contract between the host layer (world, objects,
 * sources, phasers, observers: files in this directory) and a stepping
 * backend.
 *
 * The host layer owns the ALiS data model exactly as the public structs
 * describe it (geometry, 1-D coefficient tables, material maps, source
 * descriptors, phaser descriptors) and keeps host mirrors of every field.
 * A backend owns the time stepping: updateE, updateH, updatePhaser and the
 * near-to-far sums.  The product backend (../gpu) keeps the live state in
 * HBM and runs CUDA kernels; the hooks below tell it when host-side setup
 * changed and when host mirrors must be refreshed.
 */
#ifndef ALIS_ENGINE_H
#define ALIS_ENGINE_H

#include "alis_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Single precision, always: the type of the setup quantities that the
 * reference computes in float and that decide integers (a waveform's peak
 * step and length, the phaser frequency grid).  The FP64 build of the oracle reads `float` as double
 * but defines this type as float beforehand, so both runs make the same
 * decisions and differ only in the rounding of their arithmetic. */
#ifndef ALIS_FP64
typedef float alis_f32;
#endif

/* ---- hooks the host layer calls; every backend implements them ---- */

/* W (a user world or a TFSF auxiliary world) was created; host arrays exist. */
void alis_be_world_created(world W);
/* W is about to be freed. */
void alis_be_world_deleted(world W);
/* Materials, ADE maps/coefficients or the eps^-1 maps of W changed. */
void alis_be_objects_changed(world W);
/* Sources or TFSF boxes of W changed (also scalars such as coskx). */
void alis_be_sources_changed(world W);
/* rebootWorld: fields, psi, J/K and time were reset on the host. */
void alis_be_world_reset(world W);
/* Bring host mirrors of W's fields (and J/K) up to date. */
void alis_be_sync_world(world W);
/* A phaser set (array ending with f == 0) was created / is deleted. */
void alis_be_phaser_created(phaser P);
void alis_be_phaser_deleted(phaser P);
/* Bring host mirrors of a phaser set's accumulators up to date.
 * P may point at any element of the set. */
void alis_be_sync_phaser(phaser P);
/* Poynting flux of each face of phaser P (xMin, xMax, yMin, yMax, zMin,
 * zMax; 0 for a missing face) as fluxX/fluxY/fluxZ compute it.  Returns 0
 * when the backend leaves the reduction to the host mirrors. */
int alis_be_phaser_flux(phaser P, float face[6]);
/* bring the host mirrors of every phaser set on W up to date */
void alis_be_sync_phasers_of(world W);
/* The plane sum of poyntingX/Y/Z (before their scale factors) at plane
 * index pos of axis, over in-plane index ranges [uLo, uHi] x [vLo, vHi]
 * of the two other axes in increasing order.  Returns 0 when the backend
 * leaves it to the host mirrors. */
int alis_be_plane_flux(world W, int axis, int pos, int uLo, int uHi, int vLo, int vHi, float *out);
/* Bring the host mirrors of E and H (and the currents of dispersive
 * objects nearby) up to date around cell (i, j, k) -- the cells a field
 * function evaluated there reads; alis_be_hold_sync(W) then makes further
 * syncs of W no-ops until alis_be_hold_sync(0).  Returns 0 when only a
 * full sync will do. */
int alis_be_sync_near(world W, int i, int j, int k);
/* the same for field functions evaluated over an index box (slices) */
int alis_be_sync_box(world W, int i0, int i1, int j0, int j1, int k0, int k1);
void alis_be_hold_sync(world W);
/* The sum objectAbsorption forms for dispersive object n before its scale
 * factors; 0 when the backend leaves it to the host mirrors. */
int alis_be_object_absorption(world W, int n, float *out);
/* second-order coupling of WS to the pumps WP1, WP2 (reference
 * src/update.c:343-411) */
void alis_be_nonlinear(world WS, world WP1, world WP2, float Alt);
/* The running DFT of sliceFreqDom over the index box b[6] kept by the
 * backend (reference src/slices.c:326-356): a handle or NULL.  add: one
 * call's F += f * re, G += f * im; 0 when the backend does not evaluate
 * field function f (the host loop then takes over after read).  read:
 * the sums as box arrays (k fastest); 0 when there are none. */
void *alis_be_slice_dft_begin(world W, const int b[6]);
int alis_be_slice_dft_add(void *h, world W, field *f, float re, float im);
int alis_be_slice_dft_read(void *h, float *F, float *G);
void alis_be_slice_dft_end(void *h);
/* Voxelization of the object list O[0..N-1] on the backend (reference
 * src/object.c:70-121, 229-279): a handle, or NULL when the host loops do
 * it (a shape the backend does not evaluate).  With a handle: box[6 o..]
 * = iMin, iMax, jMin, jMax, kMin, kMax of the cell centres object o owns
 * first; the fill factors of object o at (i - 1/2, j, k), (i, j - 1/2, k),
 * (i, j, k - 1/2) over the index box b[6], as box arrays (k fastest); and
 * those at index n + 1/2 of axis over the plane [u0,u1] x [v0,v1] of the
 * other two axes.  Each returns 0 when the host is to do the work. */
void *alis_be_vox_begin(world W, object *O, int N);
int alis_be_vox_bounds(void *v, int N, int *box);
int alis_be_vox_fill(void *v, int o, const int *b, float *fx, float *fy, float *fz);
int alis_be_vox_fill_edge(void *v, int o, int axis, int n, int u0, int u1, int v0, int v1, float *out);
void alis_be_vox_end(void *v);
/* Streams of W's own for W and its TFSF auxiliary worlds (a backend
 * without streams does nothing). */
void alis_be_world_streams(world W);
/* Flush and sync everything the backend holds (end of a timed loop). */
void alis_be_sync_all(void);
/* begin (1) or end (0) recording the steps of many worlds into batched
 * launches (a backend without batching does nothing) */
void alis_be_batch(int begin);

/*
 * Near-to-far-field face sums for one phaser and a batch of nA directions.
 * T[a] are the test fields (host, indexed [kMIN..kMax+1]); kx[a], ky[a] the
 * lateral wave numbers.  out[a] receives the sum over all PML-side faces of
 * the farFieldX/Y/Z bilinear forms (reference src/farfld.c:248-459,
 * 488-493), before the lattice factor and normalisation.
 */
void alis_be_farfield_sums(phaser P, int nA, const tfield *T, const float *kx,
                           const float *ky, double complex *out);

/* ---- helpers the host layer provides to backends ---- */

/* Per-source value for the current half step, following the reference
 * updateS (src/update.c:161-179): f = waveForm(t, phase) unless the source
 * carries a Phase map.  Returns 0 if the source is inactive this step. */
int alis_source_active(world W, source S);

/* Index helpers for the lazy-sync check used by field functions. */
#define ALIS_SYNC(W) alis_be_sync_world(W)

#ifdef __cplusplus
}
#endif
#endif
