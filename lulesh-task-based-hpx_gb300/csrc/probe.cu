// Pipe-rate probe (liblulesh_probe.so, not the product library): the double
// FMA, add, divide and square-root throughput and the float FMA throughput of
// the current GPU, for the FP64 roof that bounds the double-precision step
// (the benchmark reports kernel rates against it), and the rates of the
// integer-pipe multiply and add the fast kernels use beside the FP64 pipe.
//
// Each thread runs 8 independent dependency chains of one operation in a
// loop; the grid is 8 blocks of 256 threads per SM. Rates are operations per
// second counted per thread (an FMA counts once).
#include <cuda_runtime.h>

#include "lulesh_gb300.h"
#include "lulesh_probe.h"
#include "fp64_emu.cuh"
#include "fp64_emu_add.cuh"

namespace {

template <int OP>
__global__ void k_probe(double* out, int iters, double a, double b) {
    double r[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = 1.0 + 0.1 * k + 1e-3 * threadIdx.x;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (OP == 0) r[k] = fma(r[k], a, b);
            if (OP == 1) r[k] = r[k] + b;
            if (OP == 2) r[k] = a / r[k];
            if (OP == 3) r[k] = sqrt(r[k] + b);
            if (OP == 4) r[k] = r[k] * a;                                   // FP64 pipe multiply
            if (OP == 5) r[k] = lulesh::dmul_ipipe(r[k], a);                // integer-pipe multiply
            if (OP == 6) r[k] = (k & 1) ? lulesh::dmul_ipipe(r[k], a) : r[k] * a;  // half each
            if (OP == 7) r[k] = lulesh::dadd_ipipe(r[k], b);                // integer-pipe add
            if (OP == 8) r[k] = (k & 1) ? lulesh::dadd_ipipe(r[k], b) : r[k] + b;  // half each
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += r[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_probe_f32(float* out, int iters, float a, float b) {
    float r[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = 1.0f + 0.1f * k + 1e-3f * threadIdx.x;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = fmaf(r[k], a, b);
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += r[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int lulesh_probe_pipe_rates(double out[10]) {
    if (!out) return LULESH_EINVAL;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LULESH_ENODEV;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return LULESH_ECUDA;
    const int blocks = sms * 8, threads = 256;
    void* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return LULESH_ENOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters[10] = {2000, 2000, 200, 200, 20000, 2000, 2000, 2000, 2000, 2000};
    int st = LULESH_OK;
    for (int op = 0; op < 10 && st == LULESH_OK; ++op) {
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {  // first pass warms up
            cudaEventRecord(e0);
            double* d = static_cast<double*>(buf);
            switch (op) {
                case 0: k_probe<0><<<blocks, threads>>>(d, iters[op], 0.999999, 1e-6); break;
                case 1: k_probe<1><<<blocks, threads>>>(d, iters[op], 0.999999, 1e-6); break;
                case 2: k_probe<2><<<blocks, threads>>>(d, iters[op], 1.000001, 1e-6); break;
                case 3: k_probe<3><<<blocks, threads>>>(d, iters[op], 1.000001, 1e-6); break;
                case 4: k_probe_f32<<<blocks, threads>>>(static_cast<float*>(buf), iters[op], 0.999999f, 1e-6f); break;
                case 5: k_probe<4><<<blocks, threads>>>(d, iters[op], 0.999999, 0.0); break;
                case 6: k_probe<5><<<blocks, threads>>>(d, iters[op], 0.999999, 0.0); break;
                case 7: k_probe<6><<<blocks, threads>>>(d, iters[op], 0.999999, 0.0); break;
                case 8: k_probe<7><<<blocks, threads>>>(d, iters[op], 0.999999, 1e-6); break;
                default: k_probe<8><<<blocks, threads>>>(d, iters[op], 0.999999, 1e-6);
            }
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess) st = LULESH_ECUDA;
            cudaEventElapsedTime(&ms, e0, e1);
        }
        out[op] = double(blocks) * threads * iters[op] * 8 / (double(ms) * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (cudaGetLastError() != cudaSuccess) st = LULESH_ECUDA;
    return st;
}
