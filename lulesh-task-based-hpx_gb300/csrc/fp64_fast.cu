// Double-precision step kernels, FMA contraction allowed (LULESH_FP64).
#define LULESH_VARIANT fp64
#define LULESH_EXACT 0
#include "fp64_kernels.cuh"
