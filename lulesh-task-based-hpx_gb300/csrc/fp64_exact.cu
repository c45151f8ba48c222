// Double-precision step kernels with every operation rounded separately
// (LULESH_FP64_EXACT). The build compiles this file with --fmad=false.
#define LULESH_VARIANT fp64x
#define LULESH_EXACT 1
#include "fp64_kernels.cuh"
