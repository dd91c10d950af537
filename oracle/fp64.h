/*
 * fp64.h -- forced first include (gcc -include) of the FP64 build of the
 * oracle.  Test infrastructure only: it makes the FP64 reference run
 * against which the error of the FP32 path (the reference's arithmetic,
 * which the engine reproduces byte for byte) is stated.
 *
 * The host setup layer, the restated stepper (cpu_step.c) and the scene
 * drivers are compiled a second time with every `float` read as `double`
 * and every single-precision libm call read as its double-precision
 * counterpart.  The discretisation is the same: grid, CPML grading, ADE
 * poles, sources, TFSF plane waves, phaser frequencies and far-field
 * recursions are the reference's formulas (src/update.c, src/world.c,
 * src/object.c, src/source.c, src/phaser.c, src/farfld.c), evaluated in
 * FP64.  Float literals (`0.5f`, the `PI` constant) keep their float
 * values, and the setup quantities that decide integers (a waveform's
 * peak step and length, the phaser frequency grid) stay single precision
 * through `alis_f32`, so both runs solve the same discrete problem and
 * differ only in the rounding of their arithmetic.  (A Pulse of 600 nm
 * and supplement 150 at dt = 5 puts pi*deviation/dt at 959.9999 in float
 * and 960.0 in double, which would move its peak by one step; phasers
 * over 400-800 nm in steps of 400/63 number 64 in float and 65 in
 * double.)
 *
 * The system headers come first, so that their own float declarations
 * keep their types; everything included after this file sees the macros.
 */
#ifndef ALIS_ORACLE_FP64_H
#define ALIS_ORACLE_FP64_H

#include <complex.h>
#include <float.h>
#include <ieee754.h>
#include <limits.h>
#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <time.h>
#include <unistd.h>
#include <values.h>
#include <omp.h>

#define ALIS_FP64 1

/* the setup type that stays single precision (engine.h) */
typedef float alis_f32;

#define float double

#define sinf sin
#define cosf cos
#define tanf tan
#define asinf asin
#define acosf acos
#define atanf atan
#define atan2f atan2
#define sqrtf sqrt
#define expf exp
#define logf log
#define log10f log10
#define powf pow
#define fabsf fabs
#define floorf floor
#define ceilf ceil
#define roundf round
#define truncf trunc
#define fmodf fmod
#define fminf fmin
#define fmaxf fmax
#define hypotf hypot
#define fmaf fma

#define cexpf cexp
#define cabsf cabs
#define cargf carg
#define conjf conj
#define crealf creal
#define cimagf cimag
#define csqrtf csqrt
#define casinf casin
#define cacosf cacos
#define cpowf cpow
#define clogf clog

#endif
