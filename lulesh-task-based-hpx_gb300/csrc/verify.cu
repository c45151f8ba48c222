// Final report of a run, computed on the device: the origin energy and the
// plane-0 symmetry diffs of the energy field (VerifyAndWriteFinalOutput,
// lulesh-util.cc:60-115), so a run can be checked without downloading its
// fields.
//
// Built with --fmad=false. One block walks the rows j of the (j, k > j)
// pairs in the reference's order: each row (in chunks of the block size) is
// evaluated in parallel into shared memory, and thread 0 folds it into the
// running values in pair order. TotalAbsDiff is therefore the reference's
// sequential sum bit for bit; the maxima are exact whatever the order.
#include <cuda_runtime.h>

#include "lulesh_dev.h"

namespace lulesh {
namespace {

constexpr int kVerifyBlock = 256;

__global__ void __launch_bounds__(kVerifyBlock) k_verify(const double* __restrict__ e, int nx,
                                                          double* __restrict__ out) {
    __shared__ double s_abs[kVerifyBlock], s_rel[kVerifyBlock];
    double maxAbs = 0.0, totAbs = 0.0, maxRel = 0.0;  // meaningful in thread 0
    for (int j = 0; j < nx; ++j) {
        for (int k0 = j + 1; k0 < nx; k0 += kVerifyBlock) {
            const int k = k0 + int(threadIdx.x);
            if (k < nx) {
                const double ekj = e[size_t(k) * nx + j];
                const double a = fabs(e[size_t(j) * nx + k] - ekj);
                s_abs[threadIdx.x] = a;
                s_rel[threadIdx.x] = fabs(ekj) > 1e-8 ? a / ekj : 0.0;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                const int n = min(kVerifyBlock, nx - k0);
                for (int t = 0; t < n; ++t) {
                    const double a = s_abs[t], r = s_rel[t];
                    totAbs += a;
                    if (maxAbs < a) maxAbs = a;
                    if (maxRel < r) maxRel = r;
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        out[0] = e[0];
        out[1] = maxAbs;
        out[2] = totAbs;
        out[3] = maxRel;
    }
}

}  // namespace

int launch_verify(const double* e, int nx, double* out, cudaStream_t s) {
    k_verify<<<1, kVerifyBlock, 0, s>>>(e, nx, out);
    return 1;
}

}  // namespace lulesh
