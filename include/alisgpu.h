/*
 * alisgpu.h -- device C-ABI of the GB300 ALiS engine (sm_103a).
 *
 * The ALiS public API (alis_c.h) is the drop-in boundary a user program
 * links against.  Underneath it, the host layer drives the GPU only
 * through the entry points below: plain C structs, host pointers and
 * sizes, status codes.  Each entry point names the reference loops it
 * replaces.  All work is ordered on one CUDA stream per process
 * (alisgpu_stream); calls return before the GPU finishes unless they
 * return data to the host.
 *
 * Array conventions.  A host "box array" is one contiguous float block
 * covering an index box [i0,i1] x [j0,j1] x [k0,k1] with k fastest, which
 * is exactly the data block behind ALiS's float*** arrays
 * (&F[i0][j0][k0]).  On the device every field of a world is stored with
 * a one-cell halo and a row pitch padded to 32 floats, so that the first
 * interior cell of each row is 128-byte aligned.
 *
 * Status: ALISGPU_OK (0) or a negative ALISGPU_E* code;
 * alisgpu_last_error() returns a message for the last failure.
 */
#ifndef ALISGPU_H
#define ALISGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
	ALISGPU_OK = 0,
	ALISGPU_EINVAL = -1,    /* bad argument */
	ALISGPU_ENOMEM = -2,    /* device allocation failed */
	ALISGPU_ECUDA = -3,     /* CUDA runtime error */
	ALISGPU_ENODEV = -4,    /* no usable GPU */
	ALISGPU_ERANGE = -5,    /* request beyond a fixed capacity */
	ALISGPU_ENOTSUP = -6    /* not available for the world's storage form */
};

const char *alisgpu_last_error(void);
/* Initialise the device (first call selects GPU 0 or $ALISGPU_DEVICE). */
int alisgpu_init(void);
/* Wait for all queued work. */
int alisgpu_synchronize(void);
/* The CUDA stream (cudaStream_t) every kernel of the engine runs on. */
void *alisgpu_stream(void);
/* Kernel launches issued so far by this library (for launch accounting). */
unsigned long long alisgpu_launch_count(void);
/* Fault injection for the error paths, on the host: the next n
 * stream-ordered allocations of the engine (world, phaser and far-field
 * buffers) report an out-of-memory failure without allocating (n = 0
 * clears it).  Returns the previous count. */
int alisgpu_inject_alloc_failures(int n);

/* Per-kernel timing with CUDA events recorded around each launch on the
 * engine stream (off by default; adds two event records per launch).
 * alisgpu_profile_read synchronises, returns the summed device time and
 * launch count of one kernel kind since the last read, and resets it. */
enum {
	ALISGPU_K_STEP_E = 0,      /* fused E half step, worlds of >= 65536 cells */
	ALISGPU_K_STEP_H = 1,      /* fused H half step (with ADE update) */
	ALISGPU_K_GHOST = 2,       /* boundary ghost copies */
	ALISGPU_K_SOURCE = 3,      /* soft sources */
	ALISGPU_K_GATHER = 4,      /* phaser face gather */
	ALISGPU_K_FLUSH = 5,       /* phaser DFT flush */
	ALISGPU_K_FARFIELD = 6,    /* FP64 far-field sums */
	ALISGPU_K_STEP_AUX = 7,    /* half steps of small (TFSF auxiliary) worlds */
	ALISGPU_K_FLUX = 8,        /* phaser face fluxes */
	ALISGPU_K_KINDS = 9
};
int alisgpu_profile(int enable);
int alisgpu_profile_read(int kind, double *ms, unsigned long long *launches);

/* ---- worlds (reference src/world.c:164-280) ---- */

typedef struct alisgpu_geometry {
	int iMIN, iMAX, jMIN, jMAX, kMIN, kMAX;   /* grid including CPML cells */
	int iMin, iMax, jMin, jMax, kMin, kMax;   /* physical domain */
	int complexField;                          /* 1: second (imaginary) field set */
	int pml[6];                                /* CPML on xMin,yMin,zMin,xMax,yMax,zMax */
} alisgpu_geometry;

typedef struct alisgpu_world alisgpu_world;

/* Allocate zeroed E, H and CPML psi storage. */
int alisgpu_world_create(const alisgpu_geometry *g, alisgpu_world **w);
int alisgpu_world_destroy(alisgpu_world *w);
/* Zero fields, psi and ADE currents (reference src/world.c:334-380). */
int alisgpu_world_reset(alisgpu_world *w);
/* Device bytes held by the world (fields, psi, maps, currents). */
size_t alisgpu_world_bytes(const alisgpu_world *w);
/* Storage form of the E and H components (no counterpart in the
 * reference, which stores float).  ALISGPU_STORAGE_HALF holds each
 * component as IEEE half values times 2^e, one exponent e per component
 * and x plane: half the field bytes, with the update arithmetic in float.
 * A half step takes e from the largest magnitude M the plane's cells of
 * the component reached in the field's previous half step, before
 * rounding (e = x - 11 for M = f 2^x, f in [0.5, 1); -11 while M = 0;
 * clamped to [-100, 100]), rounds each updated cell to nearest even
 * (saturating at +-65504 2^e), and the source patches then add to the
 * rounded values and round again.  Ghost copies move values unchanged.
 * ADE currents, CPML psi and TFSF auxiliary worlds stay float.  Only
 * before the first half step and for real fields (else ALISGPU_EINVAL /
 * ALISGPU_ENOTSUP).  The observers (field downloads, plane fluxes, slice
 * DFTs, object absorption, the phaser gather) read the half values.  A
 * half world refuses with ALISGPU_ENOTSUP: field uploads, batched
 * recording, ghost lists other than copies, negations and zeros that move
 * whole planes, source patches outside the updated cells, and nonlinear
 * coupling. */
enum { ALISGPU_STORAGE_FLOAT = 0, ALISGPU_STORAGE_HALF = 1 };
int alisgpu_world_set_storage(alisgpu_world *w, int storage);
/* Stream groups (no counterpart in the reference, which runs one world at
 * a time on the host cores).  Every world starts in the default group,
 * whose main stream alisgpu_stream() returns.  own_streams moves w to a
 * group of its own after its queued work, so its steps overlap on the
 * device with those of worlds in other groups; share_streams puts w into
 * parent's group (a TFSF auxiliary world with the world it feeds).
 * alisgpu_synchronize() waits for every group. */
int alisgpu_world_own_streams(alisgpu_world *w);
int alisgpu_world_share_streams(alisgpu_world *w, alisgpu_world *parent);
void *alisgpu_world_stream(const alisgpu_world *w);

/* 1-D tables of the E (grid 0) or H (grid 1) lattice: dtd[3] = dt/dx,
 * dt/dy, dt/dz indexed from iMIN/jMIN/kMIN; cpml[9] = xP, xPy, xPz, yP,
 * yPz, yPx, zP, zPx, zPy (NULL where an axis has no CPML)
 * (reference src/world.c:98-161). */
int alisgpu_set_line_tables(alisgpu_world *w, int grid, const float *const dtd[3], const float *const cpml[9]);

/* Inverse-permittivity maps of the E lattice as host box arrays over
 * [iMIN,iMAX+1]x[jMIN,jMAX]x[kMIN,kMAX], [iMIN,iMAX]x[jMIN,jMAX+1]x..,
 * [..]x[kMIN,kMAX+1]; all NULL removes them (vacuum branch)
 * (reference src/object.c:168-175, 374-399). */
int alisgpu_set_eps(alisgpu_world *w, const float *cx, const float *cy, const float *cz);

/* One dispersive object: fill maps and ADE recursion coefficients
 * (reference src/object.c:178-226, 290-336). */
typedef struct alisgpu_dispersive {
	int iMin, iMax, jMin, jMax, kMin, kMax;    /* box of maps and currents */
	int NJ, NK;                                /* Drude-type poles, all poles */
	const float *fill[3];                      /* host box arrays (x, y, z) */
	float a[3];                                /* conductivity factors ax, ay, az */
	const float *JJ[3], *JK[3], *JE[3];        /* [NK] per axis */
	const float *KJ[3], *KK[3], *KE[3];        /* [NK] per axis, entries >= NJ used */
} alisgpu_dispersive;

/* Replace the dispersive objects of a world (n may be 0). */
int alisgpu_set_dispersive(alisgpu_world *w, int n, const alisgpu_dispersive *objs);

/* Copy one field component between device and a host box array over the
 * halo'd grid [iMIN-1,iMAX+1]x[jMIN-1,jMAX+1]x[kMIN-1,kMAX+1].
 * field 0 = E, 1 = H; m = 0 real / 1 imaginary set; comp 0..2. */
int alisgpu_field_download(alisgpu_world *w, int field, int m, int comp, float *host);
int alisgpu_field_upload(alisgpu_world *w, int field, int m, int comp, const float *host);
/* E and H over the index box [i0,i1]x[j0,j1]x[k0,k1] (inside the halo'd
 * grid) into host[field][m][comp][i][j][k], field 0 E / 1 H, m up to the
 * complex set: the cells an observer probe reads, without whole arrays. */
int alisgpu_field_box_download(alisgpu_world *w, int i0, int i1, int j0, int j1, int k0, int k1, float *host);
/* ADE current J (isK 0) or K (isK 1) of object n, pole p, axis comp,
 * set m, as a host box array over the object's box. */
int alisgpu_current_download(alisgpu_world *w, int n, int m, int p, int comp, int isK, float *host);
/* Every current of object n in one transfer: for m (up to the complex
 * set), pole p, axis comp: J, then K for pair poles; each a box array over
 * the object's box, back to back in host. */
int alisgpu_object_currents_download(alisgpu_world *w, int n, float *host);

/* ---- half steps (reference src/update.c:87-341) ---- */

/* TFSF box of a world and its auxiliary incident-field world
 * (reference src/source.c:269-334, src/update.c:205-272).  Aux field
 * rows are aliased as in the reference: i > auxIMAX reads row
 * auxIMAX+Alt of the component, same for j. */
typedef struct alisgpu_tfsf {
	alisgpu_world *aux;
	int iMin, iMax, jMin, jMax, kMin, kMax;
	int iMIN, iMAX, jMIN, jMAX, kMIN, kMAX;
	int auxIMAX, auxJMAX;
	int aliasX, aliasY;                         /* aux rows aliased along x / y */
} alisgpu_tfsf;

/* Soft-source increments for this half step, added in list order
 * (reference src/update.c:161-179): F[field,m,comp] over the box +=
 * values[voff + cell] (box order, k fastest). */
typedef struct alisgpu_source_patch {
	int m, comp;
	int i0, i1, j0, j1, k0, k1;
	int voff;
} alisgpu_source_patch;

/* Ghost-cell copy F = cos F' + sin G', G = cos G' - sin F' from
 * (i+di, j+dj, k+dk) over a box (reference src/update.c:182-191). */
typedef struct alisgpu_ghost_copy {
	int comp;
	int i0, i1, j0, j1, k0, k1;
	int di, dj, dk;
	float cosk, sink;
} alisgpu_ghost_copy;

typedef struct alisgpu_half_step {
	int field;                                  /* 0: E half step, 1: H */
	int ntfsf;
	const alisgpu_tfsf *tfsf;
	int nsrc;
	const alisgpu_source_patch *src;
	const float *values;                        /* host source increments */
	int nvalues;
	int nghost;
	const alisgpu_ghost_copy *ghost;
	int concurrent;                             /* 1: a TFSF auxiliary world, read only by its
	                                               parent's half steps; it may run concurrently
	                                               with the parent's step of the same field */
	int attach;                                 /* with concurrent: run this step inside the
	                                               parent's next half step of the same field
	                                               (one launch) when both forms allow it */
} alisgpu_half_step;

/* Batched launches (no counterpart in the reference): between these two
 * calls the calling thread's alisgpu_half_step_run and
 * alisgpu_phaser_record calls on worlds of the shared streams are
 * recorded; consecutive calls of one kind (E half steps, H half steps,
 * phaser samples) on distinct worlds run as a few launches over all of
 * them.  Any other call on a world launches what was recorded first. */
int alisgpu_batch_begin(void);
int alisgpu_batch_end(void);

/* One half step of a world: conductivity, ADE subtraction, curl with
 * eps^-1, CPML psi (and, for H, the ADE current update driven by E),
 * TFSF face corrections, sources, ghost copies -- bit-identical to the
 * reference order.  Replaces reference src/update.c:275-341. */
int alisgpu_half_step_run(alisgpu_world *w, const alisgpu_half_step *s);

/* Cell spacings of the E and H grids (CE->dx, CE->dy, CE->dz and CH->...)
 * per axis over [MIN, MAX], for the observer reductions below. */
int alisgpu_set_spacing(alisgpu_world *w, const float *const dE[3], const float *const dH[3]);

/* Instantaneous Poynting flux through the plane index pos of axis (0 x,
 * 1 y, 2 z) over the in-plane index box [lo[q], hi[q]] of its two other
 * axes in increasing order: the sum poyntingX/Y/Z form before their
 * scale factors, with their float and double arithmetic in their order as
 * one OpenMP thread runs it (reference src/output.c:233-356). */
int alisgpu_plane_flux(alisgpu_world *w, int axis, int pos, const int lo[2], const int hi[2], float *out);

/* Power absorbed by dispersive object n before its scale factors (the
 * sum objectAbsorption forms before dividing by the 2-D widths, doubling
 * at symmetry planes and dividing by dt), with its arithmetic in its order
 * as one OpenMP thread runs it (reference src/output.c:359-435). */
int alisgpu_object_absorption(alisgpu_world *w, int n, float *out);

/* Second-order coupling of field set m of the signal world ws to the pump
 * fields of wp1 and wp2 (the same grid; wp1 == wp2 for second-harmonic
 * generation, ws itself allowed) over the box of dispersive object n, with
 * the tensor d and sign Alt (reference src/update.c:343-411). */
int alisgpu_nonlinear_twm(alisgpu_world *ws, const alisgpu_world *wp1, const alisgpu_world *wp2, int n, int m,
                          const float d[3][6], float Alt);

/* ---- frequency-domain slices (reference src/slices.c:326-356) ----
 * The running DFT sliceFreqDom keeps over a slice box: per call
 * F += f * re, G += f * im for every cell, f the sample of a field
 * function of src/fields.c:130-291 -- component comp of E (field 0) or H
 * (field 1), real (m 0) or imaginary (m 1) set, raw (avg 0) or averaged
 * (avg 1: E over its two samples along its axis, H over its four around
 * the cell's centre line) -- mirrored on the symmetry planes of the axes
 * with sym[a] != 0 with parity par[a] (the reference's sign times the
 * Bloch cosine).  The sums stay on the device until downloaded as box
 * arrays (k fastest), F then G. */
typedef struct alisgpu_slice_dft alisgpu_slice_dft;
int alisgpu_slice_dft_create(alisgpu_world *w, const int box[6], alisgpu_slice_dft **d);
int alisgpu_slice_dft_add(alisgpu_slice_dft *d, int field, int m, int comp, int avg, const int sym[3], const float par[3],
                          float re, float im);
int alisgpu_slice_dft_download(alisgpu_slice_dft *d, float *F, float *G);
int alisgpu_slice_dft_destroy(alisgpu_slice_dft *d);

/* ---- voxelization (reference src/object.c:70-121, 229-279; src/shapes.c:9-221) ----
 * An object list as a node array: nodes 0..N-1 are the list's objects in
 * order, compound shapes point at their members further on.  Sample
 * coordinates come from host tables tab[a][((n - lo[a]) * 3 + kind) *
 * nslot + slot]: index n of axis a at n - 1/2, n, n + 1/2 (kind 0, 1, 2)
 * moved by slot 0: none, 1: -1/2, 2: +1/2, 3: -h, 4: +h, 5 + q: the q-th
 * sub-grid offset of the fill factor (subN >= 2). */
enum {
	ALISGPU_SHAPE_BOX, ALISGPU_SHAPE_BALL, ALISGPU_SHAPE_DIAMOND, ALISGPU_SHAPE_BICONEX, ALISGPU_SHAPE_BICONEY,
	ALISGPU_SHAPE_BICONEZ, ALISGPU_SHAPE_RODX, ALISGPU_SHAPE_RODY, ALISGPU_SHAPE_RODZ, ALISGPU_SHAPE_DRODX,
	ALISGPU_SHAPE_DRODY, ALISGPU_SHAPE_DRODZ, ALISGPU_SHAPE_HRODXY, ALISGPU_SHAPE_HRODYZ, ALISGPU_SHAPE_HRODZX,
	ALISGPU_SHAPE_HRODXZ, ALISGPU_SHAPE_HRODYX, ALISGPU_SHAPE_HRODZY, ALISGPU_SHAPE_TRANSLATION, ALISGPU_SHAPE_ROTATION,
	ALISGPU_SHAPE_COMBINATION, ALISGPU_SHAPE_INTERSECTION, ALISGPU_SHAPE_DIFFERENCE, ALISGPU_SHAPE_LATTICE,
	ALISGPU_SHAPE_DLATTICE, ALISGPU_SHAPE_CLATTICEX, ALISGPU_SHAPE_CLATTICEY, ALISGPU_SHAPE_CLATTICEZ,
	ALISGPU_SHAPE_COUNT
};

typedef struct alisgpu_vox_node {
	int type;                                   /* ALISGPU_SHAPE_* */
	float f[3][3];                              /* the object's parameters */
	int child, nchild;                          /* first member node and count */
	float rot[6];                               /* rotation: cos, sin about x, y, z */
	int trig;                                   /* rotational lattice: N cos then N sin in pool */
} alisgpu_vox_node;

typedef struct alisgpu_voxelizer alisgpu_voxelizer;

int alisgpu_voxelizer_create(const alisgpu_vox_node *nodes, int nnode, const float *pool, int npool,
                             const float *const tab[3], const int lo[3], const int hi[3], int nslot, int subN,
                             const int MIN[3], const int MAX[3], alisgpu_voxelizer **v);
int alisgpu_voxelizer_destroy(alisgpu_voxelizer *v);
/* per object the index box of the cell centres it owns first:
 * box[6 o] = iMin, iMax, jMin, jMax, kMin, kMax (min > max: none) */
int alisgpu_voxelizer_bounds(alisgpu_voxelizer *v, int nobj, int *box);
/* fill factors of object o at (i - 1/2, j, k), (i, j - 1/2, k), (i, j, k - 1/2)
 * over a box, as box arrays */
int alisgpu_voxelizer_fill(alisgpu_voxelizer *v, int o, int i0, int i1, int j0, int j1, int k0, int k1,
                           float *fx, float *fy, float *fz);
/* fill factors at index n + 1/2 of axis over the plane [u0,u1] x [v0,v1] of
 * the other two axes in increasing order */
int alisgpu_voxelizer_fill_edge(alisgpu_voxelizer *v, int o, int axis, int n, int u0, int u1, int v0, int v1, float *out);

/* ---- phasers (reference src/phaser.c:21-110) ---- */

typedef struct alisgpu_phaser alisgpu_phaser;

/* One face of a phaser box: axis 0/1/2 (x/y/z normal) and its planar
 * index box; components (E1, E2, H1, H2) are (Ey, Ez, Hy, Hz) for x
 * faces, (Ez, Ex, Hz, Hx) for y, (Ex, Ey, Hx, Hy) for z. */
typedef struct alisgpu_face {
	int axis;
	int i0, i1, j0, j1, k0, k1;
} alisgpu_face;

/* Accumulators for nfreq frequencies over nface faces of world w.
 * ring: time steps buffered on the device between DFT flushes.
 * kahan: 1 adds compensated summation (not bit-identical to the
 * reference's plain float sums; more accurate). */
int alisgpu_phaser_create(alisgpu_world *w, int nfreq, int nface, const alisgpu_face *faces, int ring, int kahan, alisgpu_phaser **p);
int alisgpu_phaser_destroy(alisgpu_phaser *p);
/* Record the face fields of the current time step with its phase
 * factors exp(2 pi i f t_E) and exp(2 pi i f t_H) (interleaved re, im;
 * [nfreq] each).  Flushes automatically when the ring is full. */
int alisgpu_phaser_record(alisgpu_phaser *p, const float *phaseE, const float *phaseH);
/* Accumulate every buffered step into the DFT sums. */
int alisgpu_phaser_flush(alisgpu_phaser *p);
/* Copy accumulator (frequency f, face, component q = E1,E2,H1,H2) as
 * interleaved complex host box array over the face box. */
int alisgpu_phaser_download(alisgpu_phaser *p, int f, int face, int q, float *host);
int alisgpu_phaser_zero(alisgpu_phaser *p);
/* Poynting flux of every face at every frequency, out[f * nface + face]:
 * the value the reference's fluxX/fluxY/fluxZ return for that face, with
 * their float and double arithmetic in their order as one OpenMP thread
 * runs it (reference src/phaser.c:142-219).  wE[a] / wH[a]: the E-grid and
 * H-grid spacings (CE->dx, CH->dx, ...) of axis a over [lo[a], hi[a]], a
 * box that holds every face.  Flushes the ring first. */
int alisgpu_phaser_face_flux(alisgpu_phaser *p, const float *const wE[3], const float *const wH[3],
                             const int lo[3], const int hi[3], float *out);

/* ---- near-to-far-field sums in FP64 (reference src/farfld.c:248-459) ---- */

/* For each direction a: sum over the phaser's faces (sign -1 for min
 * faces) of the face bilinear forms with test fields T (interleaved
 * complex, indexed k - kMIN, length nk per component; 6 components
 * Ex..Hz, missing ones flagged by present[a*6+c] = 0), lateral wave
 * numbers kx, ky and the world line tables.  See alisgpu_farfield_geom. */
typedef struct alisgpu_farfield_geom {
	int iMin, iMax, jMin, jMax, kMin, kMax, kMIN;
	int faceOn[6];                              /* xMin,xMax,yMin,yMax,zMin,zMax */
	int sym[3];                                 /* symmetry planes x,y,z */
	double cosk[3];                             /* coskx, cosky, coskz */
	const double *xE, *xH, *yE, *yH;            /* coordinates itox(i), itox(i-0.5), ... */
	const double *dxE, *dxH, *dyE, *dyH, *dzE, *dzH; /* CE/CH spacings */
	int xLen, yLen, zLen;                       /* table lengths, indexed from iMin, jMin, kMIN */
} alisgpu_farfield_geom;

int alisgpu_farfield_sums(alisgpu_phaser *p, int f, const alisgpu_farfield_geom *g, int nA,
                          const double *T, int nk, const unsigned char *present,
                          const double *kx, const double *ky, double *out);

/* Scratch-free variant of alisgpu_farfield_sums (no counterpart in the
 * reference): same arguments and results, but it allocates no device
 * memory -- its device buffers (tables, test fields, partial sums) live in
 * one static device array of ALISGPU_FF_STATIC_BYTES that every GPU
 * loading the library holds until exit.  For callers that cannot allocate:
 * a serving loop whose device memory is fully admitted to resident jobs
 * (a cudaMalloc there fails, or takes memory promised to a job), and hosts
 * whose allocator policy forbids device allocation after start-up.  The
 * call is synchronous: it returns after its own copies and kernel have
 * finished, also when it fails.  A batch whose buffers exceed the array
 * is refused with ALISGPU_ERANGE (about 650 directions of a 256-cell-high
 * phaser box fit); a frequency or table length the phaser's faces do not
 * fit is refused with ALISGPU_EINVAL.  The first call on a device looks up
 * the array's device address; make that first call before any stream
 * capture.  Calls share the array, which keeps the last call's contents:
 * calls that overlap on the GPU (several host threads) race. */
#define ALISGPU_FF_STATIC_BYTES (16u << 20)
int alisgpu_farfield_sums_static(alisgpu_phaser *p, int f, const alisgpu_farfield_geom *g, int nA,
                                 const double *T, int nk, const unsigned char *present,
                                 const double *kx, const double *ky, double *out);

#ifdef __cplusplus
}
#endif
#endif /* ALISGPU_H */
