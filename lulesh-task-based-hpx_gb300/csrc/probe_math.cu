// The fast variants' arithmetic helpers evaluated on given inputs, for the
// accuracy tests (lulesh_probe_math in liblulesh_probe.so). The helpers are
// the forceinline device functions of step_math.cuh and float_pair.cuh,
// compiled here with the same flags as the step's fast translation units,
// so they round as they do inside the kernels.
#define LULESH_VARIANT probe
#define LULESH_EXACT 0
#include "step_math.cuh"
#include "float_pair.cuh"
#include "lulesh_probe.h"
#include "fp64_emu.cuh"
#include "fp64_emu_add.cuh"

namespace lulesh {
namespace probe {

// fn: 0 rcp, 1 rcbrt_pos, 2 sqrt_fast, 3 recip_sqrt, 4 the reciprocal seed
// (rcp.approx.ftz.f64), 5 narrow, 6 and 7 the high and low float of split.
__global__ void k_math_probe(int fn, const double* __restrict__ in, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = in[i];
    double r;
    if (fn == 0) r = rcp(x);
    else if (fn == 1) r = rcbrt_pos(x);
    else if (fn == 2) r = sqrt_fast(x);
    else if (fn == 3) r = recip_sqrt(x);
    else if (fn == 4) asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    else if (fn == 5) r = double(narrow(x));
    else if (fn == 6) r = double(split(x).x);
    else r = double(split(x).y);
    out[i] = r;
}

__device__ __noinline__ double dmul_fp64_pipe(double a, double b) { return a * b; }
__device__ __noinline__ double dadd_fp64_pipe(double a, double b) { return a + b; }

// The FP64 pipe's product and the integer pipes' product of the same operands.
__global__ void k_dmul_probe(const double* __restrict__ a, const double* __restrict__ b,
                             double* __restrict__ native, double* __restrict__ ipipe, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    native[i] = dmul_fp64_pipe(a[i], b[i]);
    ipipe[i] = dmul_ipipe(a[i], b[i]);
}

// The FP64 pipe's sum and the integer pipes' sum of the same operands.
__global__ void k_dadd_probe(const double* __restrict__ a, const double* __restrict__ b,
                             double* __restrict__ native, double* __restrict__ ipipe, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    native[i] = dadd_fp64_pipe(a[i], b[i]);
    ipipe[i] = dadd_ipipe(a[i], b[i]);
}

}  // namespace probe
}  // namespace lulesh

extern "C" int lulesh_probe_math(int32_t fn, const double* in, double* out, int64_t n) {
    if (!in || !out || fn < 0 || fn > 7 || n < 1 || n > (int64_t(1) << 26)) return LULESH_EINVAL;
    const size_t bytes = sizeof(double) * size_t(n);
    double *d_in = nullptr, *d_out = nullptr;
    if (cudaMalloc(&d_in, bytes) != cudaSuccess) return LULESH_ENOMEM;
    if (cudaMalloc(&d_out, bytes) != cudaSuccess) {
        cudaFree(d_in);
        return LULESH_ENOMEM;
    }
    int st = LULESH_OK;
    if (cudaMemcpy(d_in, in, bytes, cudaMemcpyHostToDevice) != cudaSuccess) st = LULESH_ECUDA;
    if (st == LULESH_OK) {
        const int count = int(n);
        lulesh::probe::k_math_probe<<<(count + 255) / 256, 256>>>(fn, d_in, d_out, count);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(out, d_out, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = LULESH_ECUDA;
    }
    cudaFree(d_in);
    cudaFree(d_out);
    return st;
}

// The pairs (a, b) on the device through probe kernel k (k_dmul_probe or
// k_dadd_probe): native and integer-pipe results.
template <class Kernel>
static int pair_probe(Kernel k, const double* a, const double* b, double* native, double* ipipe, int64_t n) {
    if (!a || !b || !native || !ipipe || n < 1 || n > (int64_t(1) << 26)) return LULESH_EINVAL;
    const size_t bytes = sizeof(double) * size_t(n);
    double* d = nullptr;
    if (cudaMalloc(&d, 4 * bytes) != cudaSuccess) return LULESH_ENOMEM;
    int st = LULESH_OK;
    if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        st = LULESH_ECUDA;
    if (st == LULESH_OK) {
        const int count = int(n);
        k<<<(count + 255) / 256, 256>>>(d, d + n, d + 2 * n, d + 3 * n, count);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(native, d + 2 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(ipipe, d + 3 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = LULESH_ECUDA;
    }
    cudaFree(d);
    return st;
}

extern "C" int lulesh_probe_dadd(const double* a, const double* b, double* native, double* ipipe, int64_t n) {
    return pair_probe(lulesh::probe::k_dadd_probe, a, b, native, ipipe, n);
}

extern "C" int lulesh_probe_dmul(const double* a, const double* b, double* native, double* ipipe, int64_t n) {
    return pair_probe(lulesh::probe::k_dmul_probe, a, b, native, ipipe, n);
}
