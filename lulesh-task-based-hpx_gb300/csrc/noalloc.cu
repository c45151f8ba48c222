// Allocation-free Courant/hydro time-step constraints.
//
// lulesh_dt_constraints_noalloc computes the same two minima as the dt part of
// the material kernel (the reference's CalcConstraintForElemsTask), from
// caller-owned device arrays, for callers that cannot allocate device memory:
// a host framework that owns every device allocation through its own pool or
// budget, or a loop that cannot afford cudaMalloc/cudaFree, which may
// synchronize the whole device. Its only working memory is the file-scope
// array below, which every GPU that loads this library holds until exit.
//
// The reduction needs one partial minimum per thread block plus an arrival
// counter, so the array holds kNoAllocMaxBlocks partials (256 KiB) and the
// counter: at 256 threads per block that bounds numElem to
// LULESH_NOALLOC_MAX_ELEMS = 4,194,304 (an s = 161 cube); larger sizes are
// rejected with LULESH_EINVAL.
//
// All calls share that one array. Each call clears the counter on its stream
// before its kernel, and the kernel leaves the partials of the last call
// behind; two calls whose kernels overlap on the GPU (different streams, or
// different host threads on one device) race on the array and give wrong
// minima, so serialize them.
#define LULESH_VARIANT noalloc
#define LULESH_EXACT 0
#include <mutex>

#include "step_math.cuh"

namespace lulesh {
namespace noalloc {

constexpr int kBlock = 256;
constexpr int kNoAllocMaxBlocks = 16384;
static_assert(size_t(kNoAllocMaxBlocks) * kBlock == LULESH_NOALLOC_MAX_ELEMS, "limit mismatch");

// partials [0, kNoAllocMaxBlocks) then the arrival counter
constexpr size_t kCounterOffset = sizeof(DtPartial) * kNoAllocMaxBlocks;
constexpr size_t kScratchBytes = kCounterOffset + 256;

static __device__ __align__(256) unsigned char g_dt_scratch[kScratchBytes];

__global__ void __launch_bounds__(kBlock)
    k_dt_constraints(const double* __restrict__ ss, const double* __restrict__ vdov,
                     const double* __restrict__ arealg, int n, lulesh_params prm,
                     unsigned char* scratch, double* out) {
    DtPartial* partials = reinterpret_cast<DtPartial*>(scratch);
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + kCounterOffset);
    // fmin folds (not the step's bit-pattern minimum, which assumes the
    // non-negative candidates of its own state): caller arrays may hold any
    // value, and a NaN candidate is then ignored as fmin ignores it
    double dtc = 1.0e+20, dth = 1.0e+20;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double courant, hydro;
    if (i < n && dt_candidates(prm, __ldg(ss + i), __ldg(vdov + i), __ldg(arealg + i), courant, hydro)) {
        dtc = fmin(dtc, courant);
        dth = fmin(dth, hydro);
    }
    block_min2(dtc, dth);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x].dtc = dtc;
        partials[blockIdx.x].dth = dth;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 1.0e+20, b = 1.0e+20;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
        a = fmin(a, __ldcg(&partials[k].dtc));
        b = fmin(b, __ldcg(&partials[k].dth));
    }
    __syncthreads();
    block_min2(a, b);
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = b;
    }
}

// Device address of g_dt_scratch for each device (looked up with that device
// current). Host code cannot pass g_dt_scratch itself: its name there is a
// host-side stand-in, not a device address. The address is looked up again
// on every call whose stream is not capturing, so it follows a device reset
// (which may reload the module elsewhere); a call made while its stream
// captures a graph uses the address of the last call on that device, so the
// first call on a device must come before any capture.
static std::mutex g_mutex;
static void* g_addr[64] = {};

static int scratch_address(int device, cudaStream_t stream, void** out) {
    if (device < 0 || device >= 64) return LULESH_EINVAL;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) return LULESH_ECUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_dt_scratch) != cudaSuccess || !p) return LULESH_ECUDA;
        g_addr[device] = p;
    }
    if (!g_addr[device]) return LULESH_EINVAL;  // first call on this device inside a capture
    *out = g_addr[device];
    return LULESH_OK;
}

}  // namespace noalloc
}  // namespace lulesh

extern "C" int lulesh_dt_constraints_noalloc(const double* ss, const double* vdov,
                                             const double* arealg, int32_t numElem, double qqc,
                                             double dvovmax, double* out_dt, void* stream) {
    using namespace lulesh::noalloc;
    if (!ss || !vdov || !arealg || !out_dt || numElem < 1) return LULESH_EINVAL;
    if (numElem > LULESH_NOALLOC_MAX_ELEMS) return LULESH_EINVAL;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return LULESH_ECUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* base = nullptr;
    const int st = scratch_address(device, s, &base);
    if (st != LULESH_OK) return st;
    unsigned char* scratch = static_cast<unsigned char*>(base);
    if (cudaMemsetAsync(scratch + kCounterOffset, 0, sizeof(unsigned), s) != cudaSuccess)
        return LULESH_ECUDA;
    lulesh_params prm{};
    prm.qqc = qqc;
    prm.dvovmax = dvovmax;
    const int blocks = (numElem + kBlock - 1) / kBlock;
    k_dt_constraints<<<blocks, kBlock, 0, s>>>(ss, vdov, arealg, numElem, prm, scratch, out_dt);
    return cudaGetLastError() == cudaSuccess ? LULESH_OK : LULESH_ECUDA;
}
