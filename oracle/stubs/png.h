/* Stand-in for <png.h> used only to compile the reference sources into
 * the oracle/_ref checker (libpng is not installed).  PNG writing becomes
 * a no-op; the test drivers never request images. */
#ifndef ORACLE_STUB_PNG_H
#define ORACLE_STUB_PNG_H
#include <stdio.h>
typedef void *png_structp;
typedef void *png_infop;
typedef unsigned char png_byte;
#define PNG_LIBPNG_VER_STRING "stub"
#define PNG_Z_DEFAULT_COMPRESSION 0
#define PNG_COLOR_TYPE_RGB 0
#define PNG_INTERLACE_NONE 0
#define PNG_COMPRESSION_TYPE_DEFAULT 0
#define PNG_FILTER_TYPE_DEFAULT 0
static inline png_structp png_create_write_struct(const char *v, void *a, void *b, void *c) { (void)v; (void)a; (void)b; (void)c; return 0; }
static inline png_infop png_create_info_struct(png_structp p) { (void)p; return 0; }
static inline void png_init_io(png_structp p, FILE *f) { (void)p; (void)f; }
static inline void png_set_compression_level(png_structp p, int l) { (void)p; (void)l; }
static inline void png_set_IHDR(png_structp p, png_infop i, int w, int h, int b, int c, int il, int cm, int fm) { (void)p; (void)i; (void)w; (void)h; (void)b; (void)c; (void)il; (void)cm; (void)fm; }
static inline void png_write_info(png_structp p, png_infop i) { (void)p; (void)i; }
static inline void png_write_row(png_structp p, png_byte *r) { (void)p; (void)r; }
static inline void png_write_end(png_structp p, png_infop i) { (void)p; (void)i; }
static inline void png_destroy_write_struct(png_structp *p, void *i) { (void)p; (void)i; }
#endif
