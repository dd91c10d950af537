/* Stand-in for <hdf5.h> used only to compile the reference sources into
 * the oracle/_ref checker (libhdf5 is not installed).  Every call fails;
 * none is reached by the hot path or by the test drivers. */
#ifndef ORACLE_STUB_HDF5_H
#define ORACLE_STUB_HDF5_H
typedef long hid_t;
typedef unsigned long long hsize_t;
#define H5F_ACC_RDONLY 0
#define H5F_ACC_TRUNC 0
#define H5P_DEFAULT 0
#define H5S_ALL 0
#define H5T_NATIVE_FLOAT 0
static inline hid_t H5Fopen(const char *n, int f, int p) { (void)n; (void)f; (void)p; return -1; }
static inline hid_t H5Fcreate(const char *n, int f, int a, int b) { (void)n; (void)f; (void)a; (void)b; return -1; }
static inline long H5Gget_objname_by_idx(hid_t f, int i, char *n, int s) { (void)f; (void)i; (void)n; (void)s; return -1; }
static inline hid_t H5Dopen(hid_t f, const char *n, int p) { (void)f; (void)n; (void)p; return -1; }
static inline hid_t H5Dcreate(hid_t f, const char *n, int t, hid_t s, int a, int b, int c) { (void)f; (void)n; (void)t; (void)s; (void)a; (void)b; (void)c; return -1; }
static inline hid_t H5Dget_space(hid_t d) { (void)d; return -1; }
static inline int H5Sget_simple_extent_ndims(hid_t s) { (void)s; return 0; }
static inline int H5Sget_simple_extent_dims(hid_t s, hsize_t *d, hsize_t *m) { (void)s; (void)d; (void)m; return 0; }
static inline hid_t H5Screate_simple(int r, const hsize_t *d, const hsize_t *m) { (void)r; (void)d; (void)m; return -1; }
static inline int H5Dread(hid_t d, int t, int a, int b, int p, void *buf) { (void)d; (void)t; (void)a; (void)b; (void)p; (void)buf; return -1; }
static inline int H5Dwrite(hid_t d, int t, int a, int b, int p, const void *buf) { (void)d; (void)t; (void)a; (void)b; (void)p; (void)buf; return -1; }
static inline int H5Dclose(hid_t d) { (void)d; return 0; }
static inline int H5Sclose(hid_t s) { (void)s; return 0; }
static inline int H5Fclose(hid_t f) { (void)f; return 0; }
#endif
