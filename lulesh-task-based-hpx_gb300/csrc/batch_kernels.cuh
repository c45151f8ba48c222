// Batched persistent phase kernels, shared by every arithmetic variant.
//
// Included at the end of a variant's translation unit (after its
// forces_elem / nodes_node / kinematics_elem / material_elem). One launch
// per phase covers every active instance of a batch: a fixed grid of blocks
// pulls (instance, tile) items from a per-phase queue counter until the
// queue is empty, so large and small instances, and material tiles with 1 or
// 20 EOS passes, share the SMs without a launch per instance. Material tiles
// are queued most expensive first.
//
// A block takes `grab` consecutive tiles per queue access, copies a tile's
// Mesh (device pointers of that instance) into shared memory when the
// instance changes, and runs the variant's per-element function over the
// tile. The force, node and kinematics phases fetch their next queue position
// while the current tiles run (their tiles cost alike, so the reservation
// costs no balance); the material phase takes its next position only when
// its tiles are done, so that its cost-sorted queue stays dynamically
// balanced (reserving ahead cost 4-6 % of a serving run).
//
// The bound asks ptxas for at least one resident block per SM: without the
// minimum, its heuristic held the material phase to 64 registers with
// spills inside the EOS loop (6 % slower batched cycles).
// Each instance keeps its own dt (DevTime), and the material phase lowers
// the instance's Courant/hydro minima with atomic minima on the doubles' bit
// patterns (exact for positive values, so the order does not matter).

namespace lulesh {
namespace LULESH_VARIANT {

// Atomic min of a positive double, through its bit pattern (positive IEEE
// doubles order like their unsigned 64-bit patterns).
__device__ __forceinline__ void atomic_min_pos(double* addr, double v) {
    atomicMin(reinterpret_cast<unsigned long long*>(addr),
              static_cast<unsigned long long>(__double_as_longlong(v)));
}

template <int PHASE>
__global__ void __launch_bounds__(kBatchMaxBlock, 1) kb_phase(BatchCtl c, int grab) {
    constexpr int kind = (PHASE == 1) ? TILES_NODE : (PHASE == 3) ? TILES_MAT : TILES_ELEM;
    constexpr bool kPrefetch = PHASE != 3;
    __shared__ __align__(16) unsigned long long s_mesh[(sizeof(Mesh) + 7) / 8];
    __shared__ int s_tile;
    __shared__ int s_active;
    __shared__ double s_dt;
    const Mesh& m = *reinterpret_cast<const Mesh*>(s_mesh);
    const int ntiles = __ldg(c.ntiles + kind);
    const BatchTile* tiles = c.tiles[kind];
    int cur_inst = -1;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(&c.queue[PHASE], (unsigned)grab);
    __syncthreads();
    int t0 = s_tile;
    while (t0 < ntiles) {
        const int t1 = min(t0 + grab, ntiles);
        __syncthreads();  // every thread has read s_tile
        // the next queue position, fetched while this grab's tiles run
        if (kPrefetch && threadIdx.x == 0) s_tile = (int)atomicAdd(&c.queue[PHASE], (unsigned)grab);
        for (int t = t0; t < t1; ++t) {
            const BatchTile tile = tiles[t];
            if (tile.inst != cur_inst) {  // the same for every thread of the block
                __syncthreads();          // the previous instance's Mesh is no longer read
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(c.meshes + tile.inst);
                for (int k = threadIdx.x; k < (int)((sizeof(Mesh) + 7) / 8); k += blockDim.x) s_mesh[k] = src[k];
                if (threadIdx.x == 0) {
                    s_active = c.times[tile.inst].active;
                    s_dt = c.times[tile.inst].deltatime;
                }
                __syncthreads();
                cur_inst = tile.inst;
            }
            if (!s_active) continue;
            if (PHASE == 3) {
                double dtc = 1.0e+20, dth = 1.0e+20;
                for (int k = threadIdx.x; k < tile.count; k += blockDim.x)
                    material_elem(m, tile.first + k, dtc, dth);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    dtc = fmin(dtc, __shfl_down_sync(0xffffffffu, dtc, o));
                    dth = fmin(dth, __shfl_down_sync(0xffffffffu, dth, o));
                }
                if ((threadIdx.x & 31) == 0) {
                    atomic_min_pos(&m.result->dtcourant, dtc);
                    atomic_min_pos(&m.result->dthydro, dth);
                }
            } else {
                for (int k = threadIdx.x; k < tile.count; k += blockDim.x) {
#if LULESH_GEO_FORM
                    // the fast double variant's geometry form (each instance's
                    // geometry formed at admission, kept by its kinematics)
                    if (PHASE == 0) forces_geo_elem(m, tile.first + k);
                    if (PHASE == 2) kinematics_fast<true>(m, tile.first + k, s_dt);
#else
                    if (PHASE == 0) forces_elem(m, tile.first + k);
                    if (PHASE == 2) kinematics_elem(m, tile.first + k, s_dt);
#endif
                    if (PHASE == 1) nodes_node(m, tile.first + k, s_dt);
                }
            }
        }
        if (!kPrefetch && threadIdx.x == 0) s_tile = (int)atomicAdd(&c.queue[PHASE], (unsigned)grab);
        __syncthreads();  // thread 0's next queue position is visible
        t0 = s_tile;
    }
}

int launch_batch_phase(int phase, const BatchCtl& c, const BatchLaunch& l, cudaStream_t s) {
    switch (phase) {
        case 0: kb_phase<0><<<l.grid, l.block, 0, s>>>(c, l.grab); break;
        case 1: kb_phase<1><<<l.grid, l.block, 0, s>>>(c, l.grab); break;
        case 2: kb_phase<2><<<l.grid, l.block, 0, s>>>(c, l.grab); break;
        default: kb_phase<3><<<l.grid, l.block, 0, s>>>(c, l.grab); break;
    }
    return 1;
}

int batch_occupancy(int phase, int block) {
    int n = 0;
    cudaError_t e;
    switch (phase) {
        case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_phase<0>, block, 0); break;
        case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_phase<1>, block, 0); break;
        case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_phase<2>, block, 0); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_phase<3>, block, 0); break;
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace LULESH_VARIANT
}  // namespace lulesh
