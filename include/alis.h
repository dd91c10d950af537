/*
 * alis.h -- umbrella header of the GB300 ALiS engine (reference src/alis.h:7-8):
 * the C interface plus the material and colormap tables.
 */
#include "alis_c.h"
#include "alis_m.h"
