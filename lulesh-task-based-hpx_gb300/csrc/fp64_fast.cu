// Double-precision step kernels, FMA contraction allowed (LULESH_FP64).
#define LULESH_VARIANT fp64
#define LULESH_EXACT 0
#include "fp64_kernels.cuh"

namespace lulesh {
namespace fp64 {

// The fast variants' arithmetic helpers evaluated on given inputs, for
// accuracy tests against correctly rounded host results. fn: 0 rcp,
// 1 rcbrt_pos, 2 sqrt_fast, 3 recip_sqrt, 4 the reciprocal seed
// (rcp.approx.ftz.f64).
__global__ void k_math_probe(int fn, const double* __restrict__ in, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = in[i];
    double r;
    if (fn == 0) r = rcp(x);
    else if (fn == 1) r = rcbrt_pos(x);
    else if (fn == 2) r = sqrt_fast(x);
    else if (fn == 3) r = recip_sqrt(x);
    else asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    out[i] = r;
}

int launch_math_probe(int fn, const double* in, double* out, int n, cudaStream_t s) {
    k_math_probe<<<blocks_for(n, 256), 256, 0, s>>>(fn, in, out, n);
    return 1;
}

}  // namespace fp64
}  // namespace lulesh
