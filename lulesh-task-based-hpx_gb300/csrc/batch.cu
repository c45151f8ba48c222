// Batched ensembles: many independent Sedov problems resident in one device
// pool, every cycle of all of them replayed from one CUDA graph.
//
// Pool. One cudaMalloc of the requested size; each admitted problem takes a
// contiguous first-fit block for its mesh arrays (mesh_bytes) and is freed on
// retire (neighbouring free blocks coalesce). Per-slot Mesh descriptors,
// DevTime and StepResult live in small fixed arrays.
//
// Work queue. The host keeps three tile tables (elements, nodes, material
// positions) covering every slot in use; material tiles are cut at
// repeat-count boundaries and queued most expensive first. Tables live in
// fixed device arrays and their lengths in device memory, so admitting or
// retiring a problem changes them between graph replays without
// re-capturing the graph (the graph is re-captured only when a table
// outgrows its capacity or the launch shapes change).
//
// Graph of one cycle: kb_time_increment (per-slot TimeIncrement, dt minima
// re-armed, queues cleared) -> forces -> nodes -> kinematics -> material
// (persistent kernels over the queue) -> kb_time_finish.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "lulesh_dev.h"

namespace {

using lulesh::BatchCtl;
using lulesh::BatchLaunch;
using lulesh::BatchTile;
using lulesh::DevTime;
using lulesh::Mesh;
using lulesh::StepResult;

#define BCK(call)                                    \
    do {                                             \
        if ((call) != cudaSuccess) return LULESH_ECUDA; \
    } while (0)

// First-fit allocator over [0, size) with coalescing free blocks.
class Pool {
   public:
    void reset(size_t size) {
        free_.clear();
        if (size) free_[0] = size;
    }
    // Returns the offset or SIZE_MAX.
    size_t alloc(size_t n) {
        n = (n + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const size_t off = it->first, rest = it->second - n;
            free_.erase(it);
            if (rest) free_[off + n] = rest;
            return off;
        }
        return SIZE_MAX;
    }
    void release(size_t off, size_t n) {
        n = (n + 255) & ~size_t(255);
        auto it = free_.emplace(off, n).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t largest_free() const {
        size_t m = 0;
        for (const auto& kv : free_) m = std::max(m, kv.second);
        return m;
    }

   private:
    std::map<size_t, size_t> free_;
};

struct Slot {
    bool in_use = false;
    size_t off = 0, bytes = 0;
    int s = 0, numElem = 0, numNode = 0;
    std::vector<int32_t> repCount;  // elements per EOS repeat class, classes in matOrder order
    std::vector<int32_t> repValue;
    bool finished = false;  // reached its stoptime, cycle limit or an error (seen by lulesh_batch_run)
};

struct Launch3 {
    int (*phase)(int, const BatchCtl&, const BatchLaunch&, cudaStream_t);
    int (*occupancy)(int, int);
};

Launch3 batch_launchers(int precision) {
    switch (precision) {
        case LULESH_FP64: return {lulesh::fp64::launch_batch_phase, lulesh::fp64::batch_occupancy};
        case LULESH_FP64_EXACT: return {lulesh::fp64x::launch_batch_phase, lulesh::fp64x::batch_occupancy};
        default: return {lulesh::mixed::launch_batch_phase, lulesh::mixed::batch_occupancy};
    }
}

}  // namespace

struct lulesh_batch {
    int precision = LULESH_FP64;
    int sms = 0;
    cudaStream_t stream = nullptr;
    char* pool_base = nullptr;
    size_t pool_bytes = 0;
    Pool pool;
    std::vector<Slot> slots;
    // device arrays
    Mesh* d_meshes = nullptr;
    DevTime* d_times = nullptr;
    StepResult* d_results = nullptr;
    BatchTile* d_tiles[3] = {nullptr, nullptr, nullptr};
    size_t tile_cap[3] = {0, 0, 0};
    int32_t* d_ntiles = nullptr;
    unsigned* d_queue = nullptr;
    double* d_verify = nullptr;  // [4] lulesh_batch_verify output
    // pinned host mirrors
    Mesh* h_meshes = nullptr;
    DevTime* h_times = nullptr;
    StepResult* h_results = nullptr;
    int32_t* h_ntiles = nullptr;
    double* h_verify = nullptr;
    std::vector<BatchTile> h_tiles[3];
    // launch shapes and graph
    Launch3 L{};
    lulesh_batch_tuning tuning{};
    cudaGraphExec_t graph = nullptr;
    int graph_kernels = 0;
    bool tiles_dirty = true;
    int64_t launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

int free_slot(const lulesh_batch* b) {
    for (int i = 0; i < int(b->slots.size()); ++i)
        if (!b->slots[i].in_use) return i;
    return -1;
}

// Completes an admission: the slot's mesh descriptor, time state (with its
// own stoptime and cycle limit) and result word go to the device, and the
// slot records its pool block and repeat classes (repeat count, elements).
int finish_admit(lulesh_batch* b, int slot, size_t off, size_t bytes, Mesh m, const lulesh_time_state& ts,
                 double stoptime, int32_t max_cycles, const std::vector<int2>& classes, int s,
                 int32_t* slot_out) {
    m.result = b->d_results + slot;
    m.dtime = b->d_times + slot;
    m.partials = nullptr;
    m.matGrid = 0;
    DevTime t{};
    t.time = ts.time;
    t.deltatime = ts.deltatime;
    t.dtcourant = ts.dtcourant;
    t.dthydro = ts.dthydro;
    t.dtfixed = ts.dtfixed;
    t.deltatimemultlb = ts.deltatimemultlb;
    t.deltatimemultub = ts.deltatimemultub;
    t.dtmax = ts.dtmax;
    t.stoptime = stoptime > 0.0 ? stoptime : ts.stoptime;
    t.cycle = ts.cycle;
    t.max_cycles = max_cycles > 0 ? max_cycles : INT32_MAX;
    t.active = 1;
    StepResult r{};
    r.dtcourant = r.dthydro = 1.0e+20;
    Slot& sl = b->slots[slot];
    sl.repCount.clear();
    sl.repValue.clear();
    for (const int2& c : classes) {
        sl.repValue.push_back(c.x);
        sl.repCount.push_back(c.y);
    }
    b->h_meshes[slot] = m;
    b->h_times[slot] = t;
    b->h_results[slot] = r;
    auto release = [&](int code) {
        b->pool.release(off, bytes);
        return code;
    };
    if (m.geo) {  // the fast double variant's element geometry, before the first force phase
        b->launches += lulesh::fp64::launch_geometry(m, b->stream);
        if (cudaGetLastError() != cudaSuccess) return release(LULESH_ECUDA);
    }
    if (cudaMemcpyAsync(b->d_meshes + slot, b->h_meshes + slot, sizeof(Mesh), cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(b->d_times + slot, b->h_times + slot, sizeof(DevTime), cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(b->d_results + slot, b->h_results + slot, sizeof(StepResult), cudaMemcpyHostToDevice,
                        b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return release(LULESH_ECUDA);
    sl.in_use = true;
    sl.off = off;
    sl.bytes = bytes;
    sl.s = s;
    sl.numElem = m.numElem;
    sl.numNode = m.numNode;
    b->tiles_dirty = true;
    if (slot_out) *slot_out = slot;
    return LULESH_OK;
}

BatchCtl make_ctl(const lulesh_batch* b) {
    BatchCtl c{};
    c.meshes = b->d_meshes;
    c.times = b->d_times;
    c.results = b->d_results;
    for (int k = 0; k < 3; ++k) c.tiles[k] = b->d_tiles[k];
    c.ntiles = b->d_ntiles;
    c.queue = b->d_queue;
    c.slots = int32_t(b->slots.size());
    return c;
}

BatchLaunch shape(const lulesh_batch* b, int phase) {
    const int block = b->tuning.block[phase];
    const int occ = std::max(1, b->L.occupancy(phase, block));
    const int per_sm = std::max(1, std::min(b->tuning.blocks_per_sm[phase], occ));
    return {block, b->sms * per_sm, std::max(1, b->tuning.grab[phase])};
}

// Tile size for the problems still running: the tuned size, halved (down to
// 64) while the running problems' elements would give each resident block
// of the widest phase fewer than 4 tiles. When the first problems of an
// ensemble finish, the rest then still spread over every SM instead of a few
// long tiles.
int effective_tile(const lulesh_batch* b) {
    int64_t elems = 0;
    for (const Slot& sl : b->slots)
        if (sl.in_use && !sl.finished) elems += sl.numElem;
    int blocks = 1;
    for (int p = 0; p < 4; ++p) blocks = std::max(blocks, shape(b, p).grid);
    int T = std::max(32, b->tuning.tile);
    while (T > 64 && elems < int64_t(4) * blocks * T) T /= 2;
    return T;
}

// Rebuilds the three tile tables from the slots in use, leaving out problems
// already finished (their tiles would only be fetched and skipped). Returns
// true when a table outgrew its device capacity (the caller reallocates and
// re-captures).
bool rebuild_tiles(lulesh_batch* b) {
    const int T = effective_tile(b);
    for (auto& t : b->h_tiles) t.clear();
    for (int s = 0; s < int(b->slots.size()); ++s) {
        const Slot& sl = b->slots[s];
        if (!sl.in_use || sl.finished) continue;
        for (int e = 0; e < sl.numElem; e += T)
            b->h_tiles[lulesh::TILES_ELEM].push_back({s, e, std::min(T, sl.numElem - e), std::min(T, sl.numElem - e)});
        for (int n = 0; n < sl.numNode; n += T)
            b->h_tiles[lulesh::TILES_NODE].push_back({s, n, std::min(T, sl.numNode - n), std::min(T, sl.numNode - n)});
        int pos = 0;
        for (size_t c = 0; c < sl.repCount.size(); ++c) {
            const int end = pos + sl.repCount[c];
            for (int t = pos; t < end; t += T) {
                const int cnt = std::min(T, end - t);
                b->h_tiles[lulesh::TILES_MAT].push_back({s, t, cnt, cnt * sl.repValue[c]});
            }
            pos = end;
        }
    }
    // most expensive material tiles first, so long tiles start early
    std::stable_sort(b->h_tiles[lulesh::TILES_MAT].begin(), b->h_tiles[lulesh::TILES_MAT].end(),
                     [](const BatchTile& x, const BatchTile& y) { return x.cost > y.cost; });
    bool grew = false;
    for (int k = 0; k < 3; ++k) {
        b->h_ntiles[k] = int32_t(b->h_tiles[k].size());
        if (b->h_tiles[k].size() > b->tile_cap[k]) grew = true;
    }
    return grew;
}

int upload_tiles(lulesh_batch* b) {
    if (rebuild_tiles(b)) {
        // grow the tables (with head-room) and re-capture the graph
        BCK(cudaStreamSynchronize(b->stream));
        for (int k = 0; k < 3; ++k) {
            if (b->h_tiles[k].size() <= b->tile_cap[k]) continue;
            if (b->d_tiles[k]) cudaFree(b->d_tiles[k]);
            b->tile_cap[k] = b->h_tiles[k].size() * 2 + 64;
            if (cudaMalloc(&b->d_tiles[k], b->tile_cap[k] * sizeof(BatchTile)) != cudaSuccess) {
                b->d_tiles[k] = nullptr;
                b->tile_cap[k] = 0;
                return LULESH_ENOMEM;
            }
        }
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
    }
    for (int k = 0; k < 3; ++k)
        if (!b->h_tiles[k].empty())
            BCK(cudaMemcpyAsync(b->d_tiles[k], b->h_tiles[k].data(), b->h_tiles[k].size() * sizeof(BatchTile),
                                cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_ntiles, b->h_ntiles, 3 * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));  // the host tables are reused
    b->tiles_dirty = false;
    return LULESH_OK;
}

int build_graph(lulesh_batch* b) {
    if (b->graph) return LULESH_OK;
    const BatchCtl c = make_ctl(b);
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int k = lulesh::launch_batch_time_increment(c, b->stream);
    for (int p = 0; p < 4; ++p) k += b->L.phase(p, c, shape(b, p), b->stream);
    k += lulesh::launch_batch_time_finish(c, b->stream);
    if (cudaStreamEndCapture(b->stream, &g) != cudaSuccess) return LULESH_ECUDA;
    const cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return LULESH_ECUDA;
    }
    b->graph_kernels = k;
    return LULESH_OK;
}

int prepare(lulesh_batch* b) {
    if (b->tiles_dirty) {
        const int st = upload_tiles(b);
        if (st != LULESH_OK) return st;
    }
    return build_graph(b);
}

int refresh_status(lulesh_batch* b) {
    const size_t n = b->slots.size();
    BCK(cudaMemcpyAsync(b->h_times, b->d_times, n * sizeof(DevTime), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaMemcpyAsync(b->h_results, b->d_results, n * sizeof(StepResult), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return LULESH_OK;
}

int replay(lulesh_batch* b, int cycles, double* device_ms) {
    int st = prepare(b);
    if (st != LULESH_OK) return st;
    BCK(cudaEventRecord(b->ev0, b->stream));
    for (int k = 0; k < cycles; ++k) {
        BCK(cudaGraphLaunch(b->graph, b->stream));
        b->launches += b->graph_kernels;
    }
    BCK(cudaEventRecord(b->ev1, b->stream));
    BCK(cudaEventSynchronize(b->ev1));
    if (device_ms) {
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        *device_ms = ms;
    }
    return LULESH_OK;
}

}  // namespace

extern "C" {

int lulesh_batch_footprint(int32_t precision, int32_t s, uint64_t* bytes) {
    if (!bytes || s < 1 || s > 640) return LULESH_EINVAL;
    if (precision != LULESH_FP64 && precision != LULESH_FP64_EXACT && precision != LULESH_MIXED)
        return LULESH_EINVAL;
    const int ne = s * s * s, nn = (s + 1) * (s + 1) * (s + 1);
    *bytes = lulesh::mesh_bytes(precision, ne, nn);
    return LULESH_OK;
}

void lulesh_batch_destroy(lulesh_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    for (void* p : {(void*)b->pool_base, (void*)b->d_meshes, (void*)b->d_times, (void*)b->d_results,
                    (void*)b->d_tiles[0], (void*)b->d_tiles[1], (void*)b->d_tiles[2],
                    (void*)b->d_ntiles, (void*)b->d_queue, (void*)b->d_verify})
        if (p) cudaFree(p);
    for (void* p : {(void*)b->h_meshes, (void*)b->h_times, (void*)b->h_results, (void*)b->h_ntiles,
                    (void*)b->h_verify})
        if (p) cudaFreeHost(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int lulesh_batch_create(int32_t precision, uint64_t pool_bytes, int32_t max_slots, lulesh_batch** out) {
    if (!out) return LULESH_EINVAL;
    *out = nullptr;
    if (precision != LULESH_FP64 && precision != LULESH_FP64_EXACT && precision != LULESH_MIXED)
        return LULESH_EINVAL;
    if (max_slots < 1 || max_slots > 65536 || pool_bytes < 4096) return LULESH_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return LULESH_ENODEV;
    lulesh_batch* b = new (std::nothrow) lulesh_batch;
    if (!b) return LULESH_ENOMEM;
    auto fail = [&](int code) {
        lulesh_batch_destroy(b);
        return code;
    };
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(LULESH_ECUDA);
    b->precision = precision;
    b->L = batch_launchers(precision);
    b->slots.resize(max_slots);
    b->pool_bytes = (pool_bytes + 255) & ~uint64_t(255);
    const size_t n = size_t(max_slots);
    if (cudaMalloc(&b->pool_base, b->pool_bytes) != cudaSuccess) return fail(LULESH_ENOMEM);
    b->pool.reset(b->pool_bytes);
    if (cudaMalloc(&b->d_meshes, n * sizeof(Mesh)) != cudaSuccess ||
        cudaMalloc(&b->d_times, n * sizeof(DevTime)) != cudaSuccess ||
        cudaMalloc(&b->d_results, n * sizeof(StepResult)) != cudaSuccess ||
        cudaMalloc(&b->d_ntiles, 3 * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&b->d_queue, 4 * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&b->d_verify, 4 * sizeof(double)) != cudaSuccess)
        return fail(LULESH_ENOMEM);
    if (cudaMallocHost(&b->h_meshes, n * sizeof(Mesh)) != cudaSuccess ||
        cudaMallocHost(&b->h_times, n * sizeof(DevTime)) != cudaSuccess ||
        cudaMallocHost(&b->h_results, n * sizeof(StepResult)) != cudaSuccess ||
        cudaMallocHost(&b->h_ntiles, 3 * sizeof(int32_t)) != cudaSuccess ||
        cudaMallocHost(&b->h_verify, 4 * sizeof(double)) != cudaSuccess)
        return fail(LULESH_ENOMEM);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
        return fail(LULESH_ECUDA);
    std::memset(b->h_meshes, 0, n * sizeof(Mesh));
    for (size_t i = 0; i < n; ++i) {
        b->h_times[i] = DevTime{};
        b->h_times[i].max_cycles = -1;  // empty slot
        b->h_results[i] = StepResult{};
    }
    b->h_ntiles[0] = b->h_ntiles[1] = b->h_ntiles[2] = 0;
    if (cudaMemcpyAsync(b->d_meshes, b->h_meshes, n * sizeof(Mesh), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaMemcpyAsync(b->d_times, b->h_times, n * sizeof(DevTime), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaMemcpyAsync(b->d_results, b->h_results, n * sizeof(StepResult), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaMemcpyAsync(b->d_ntiles, b->h_ntiles, 3 * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->d_queue, 0, 4 * sizeof(unsigned), b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return fail(LULESH_ECUDA);
    // defaults until lulesh_batch_autotune: the single-problem kernels' shapes
    const int blocks[4] = {128, 256, 128, 128};
    for (int p = 0; p < 4; ++p) {
        b->tuning.block[p] = blocks[p];
        b->tuning.blocks_per_sm[p] = 8;
        b->tuning.grab[p] = 1;
    }
    b->tuning.tile = 1024;
    *out = b;
    return LULESH_OK;
}

int lulesh_batch_admit(lulesh_batch* b, const lulesh_problem* p, int32_t* slot_out) {
    if (!b) return LULESH_EINVAL;
    int st = lulesh::check_problem(p);
    if (st != LULESH_OK) return st;
    const int slot = free_slot(b);
    if (slot < 0) return LULESH_ENOMEM;
    const int ne = p->s * p->s * p->s, nn = (p->s + 1) * (p->s + 1) * (p->s + 1);
    const size_t bytes = lulesh::mesh_bytes(b->precision, ne, nn);
    const size_t off = b->pool.alloc(bytes);
    if (off == SIZE_MAX) return LULESH_ENOMEM;
    // built on the device: no host Domain, nothing uploaded but the region runs
    Mesh m{};
    lulesh_time_state ts{};
    std::vector<int2> classes;
    st = lulesh::mesh_init_problem(m, b->pool_base + off, p, b->precision, b->stream, &ts, &classes);
    if (st != LULESH_OK) {
        b->pool.release(off, bytes);
        return st;
    }
    b->launches += b->precision == LULESH_MIXED ? 6 : 5;  // the build kernels, the order (and the mirror)
    return finish_admit(b, slot, off, bytes, m, ts, p->stoptime, p->max_cycles, classes, p->s, slot_out);
}

int lulesh_batch_admit_view(lulesh_batch* b, const lulesh_domain_view* v, double stoptime,
                            int32_t max_cycles, int32_t* slot_out) {
    if (!b || !v || !v->time) return LULESH_EINVAL;
    int st = lulesh::validate_view(v);
    if (st != LULESH_OK) return st;
    const int slot = free_slot(b);
    if (slot < 0) return LULESH_ENOMEM;
    const int ne = v->numElem, nn = v->numNode;
    const size_t bytes = lulesh::mesh_bytes(b->precision, ne, nn);
    const size_t off = b->pool.alloc(bytes);
    if (off == SIZE_MAX) return LULESH_ENOMEM;
    Mesh m{};
    st = lulesh::mesh_init(m, b->pool_base + off, v, b->precision, b->stream);
    if (st != LULESH_OK) {
        b->pool.release(off, bytes);
        return st;
    }
    // repeat classes in matOrder order (largest repeat count first)
    std::map<int, int, std::greater<int>> count;
    for (int i = 0; i < ne; ++i) ++count[lulesh::region_rep(v->regNumList[i] - 1, v->numReg, v->cost)];
    std::vector<int2> classes;
    for (const auto& kv : count) classes.push_back(make_int2(kv.first, kv.second));
    return finish_admit(b, slot, off, bytes, m, *v->time, stoptime, max_cycles, classes, v->sizeX, slot_out);
}

int lulesh_batch_origin_energy(lulesh_batch* b, int32_t slot, double* e0) {
    if (!b || !e0 || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].in_use) return LULESH_EINVAL;
    BCK(cudaMemcpyAsync(e0, b->h_meshes[slot].e, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return LULESH_OK;
}

int lulesh_batch_verify(lulesh_batch* b, int32_t slot, lulesh_verify_result* out) {
    if (!b || !out || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].in_use) return LULESH_EINVAL;
    const Slot& sl = b->slots[slot];
    if (sl.s < 1 || int64_t(sl.s) * sl.s * sl.s != int64_t(sl.numElem)) return LULESH_EINVAL;
    b->launches += lulesh::launch_verify(b->h_meshes[slot].e, sl.s, b->d_verify, b->stream);
    BCK(cudaGetLastError());
    BCK(cudaMemcpyAsync(b->h_verify, b->d_verify, 4 * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    out->e0 = b->h_verify[0];
    out->maxabs = b->h_verify[1];
    out->totabs = b->h_verify[2];
    out->maxrel = b->h_verify[3];
    out->cycle = b->h_times[slot].cycle;
    out->nx = sl.s;
    return LULESH_OK;
}

int lulesh_batch_retire(lulesh_batch* b, int32_t slot) {
    if (!b || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].in_use) return LULESH_EINVAL;
    BCK(cudaStreamSynchronize(b->stream));
    Slot& sl = b->slots[slot];
    b->pool.release(sl.off, sl.bytes);
    sl = Slot{};
    b->h_times[slot] = DevTime{};
    b->h_times[slot].max_cycles = -1;
    b->h_results[slot] = StepResult{};
    BCK(cudaMemcpyAsync(b->d_times + slot, b->h_times + slot, sizeof(DevTime), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_results + slot, b->h_results + slot, sizeof(StepResult), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->tiles_dirty = true;
    return LULESH_OK;
}

int lulesh_batch_run(lulesh_batch* b, int32_t cycles, int32_t* active_slots, double* device_ms) {
    if (!b || cycles < 0) return LULESH_EINVAL;
    int st = replay(b, cycles, device_ms);
    if (st != LULESH_OK) return st;
    st = refresh_status(b);
    if (st != LULESH_OK) return st;
    // problems that finished in these cycles leave the tile tables
    for (size_t i = 0; i < b->slots.size(); ++i) {
        Slot& sl = b->slots[i];
        if (sl.in_use && !sl.finished && !b->h_times[i].active) {
            sl.finished = true;
            b->tiles_dirty = true;
        }
    }
    if (active_slots) {
        int n = 0;
        for (size_t i = 0; i < b->slots.size(); ++i) n += (b->slots[i].in_use && b->h_times[i].active);
        *active_slots = n;
    }
    return LULESH_OK;
}

int lulesh_batch_status(const lulesh_batch* b, lulesh_slot_status* out, int32_t n) {
    if (!b || !out || n < 0) return LULESH_EINVAL;
    const int m = std::min<int>(n, int(b->slots.size()));
    for (int i = 0; i < m; ++i) {
        lulesh_slot_status& o = out[i];
        o = lulesh_slot_status{};
        const Slot& sl = b->slots[i];
        o.in_use = sl.in_use;
        if (!sl.in_use) continue;
        const DevTime& t = b->h_times[i];
        const StepResult& r = b->h_results[i];
        o.active = t.active;
        o.cycle = t.cycle;
        o.err = r.err;
        o.err_elem = r.err_elem;
        o.numElem = sl.numElem;
        o.s = sl.s;
        o.time = t.time;
        o.deltatime = t.deltatime;
        o.dtcourant = t.dtcourant;
        o.dthydro = t.dthydro;
    }
    return LULESH_OK;
}

int lulesh_batch_download(lulesh_batch* b, int32_t slot, lulesh_domain_view* host, uint32_t mask) {
    if (!b || !host || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].in_use) return LULESH_EINVAL;
    const Mesh& m = b->h_meshes[slot];
    if (host->numElem != m.numElem || host->numNode != m.numNode) return LULESH_EINVAL;
    BCK(cudaStreamSynchronize(b->stream));
    return lulesh::copy_fields(m, host, mask, false, b->stream);
}

int lulesh_batch_get_tuning(const lulesh_batch* b, lulesh_batch_tuning* out) {
    if (!b || !out) return LULESH_EINVAL;
    *out = b->tuning;
    return LULESH_OK;
}

int lulesh_batch_set_tuning(lulesh_batch* b, const lulesh_batch_tuning* t) {
    if (!b || !t || t->tile < 32) return LULESH_EINVAL;
    for (int p = 0; p < 4; ++p)
        if (t->block[p] < 32 || t->block[p] > lulesh::kBatchMaxBlock || t->block[p] % 32 || t->blocks_per_sm[p] < 1 ||
            t->grab[p] < 1 || t->grab[p] > 64)
            return LULESH_EINVAL;
    BCK(cudaStreamSynchronize(b->stream));
    b->tuning = *t;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->tiles_dirty = true;
    return LULESH_OK;
}

int64_t lulesh_batch_launch_count(const lulesh_batch* b) { return b ? b->launches : 0; }

}  // extern "C"

extern "C" int lulesh_batch_autotune(lulesh_batch* b, int32_t cycles, lulesh_batch_tuning* chosen) {
    if (!b || cycles < 1) return LULESH_EINVAL;
    const size_t n = b->slots.size();
    size_t total = 0;
    for (const Slot& sl : b->slots)
        if (sl.in_use) total += sl.bytes;
    if (total == 0) {
        if (chosen) *chosen = b->tuning;
        return LULESH_OK;
    }
    const size_t tb = n * sizeof(DevTime), rb = n * sizeof(StepResult);
    char* snap = nullptr;
    if (cudaMalloc(&snap, total + tb + rb) != cudaSuccess) return LULESH_ENOMEM;
    auto copy_state = [&](bool save) -> int {
        size_t o = 0;
        for (const Slot& sl : b->slots) {
            if (!sl.in_use) continue;
            char* live = b->pool_base + sl.off;
            BCK(cudaMemcpyAsync(save ? snap + o : live, save ? live : snap + o, sl.bytes,
                                cudaMemcpyDeviceToDevice, b->stream));
            o += sl.bytes;
        }
        BCK(cudaMemcpyAsync(save ? (void*)(snap + o) : (void*)b->d_times, save ? (void*)b->d_times : (void*)(snap + o),
                            tb, cudaMemcpyDeviceToDevice, b->stream));
        BCK(cudaMemcpyAsync(save ? (void*)(snap + o + tb) : (void*)b->d_results,
                            save ? (void*)b->d_results : (void*)(snap + o + tb), rb, cudaMemcpyDeviceToDevice,
                            b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        return LULESH_OK;
    };
    // time `cycles` replays of tuning t from the saved state (one untimed
    // replay first: a freshly instantiated graph's first launch is slower)
    auto measure = [&](const lulesh_batch_tuning& t, double* ms) -> int {
        int st = lulesh_batch_set_tuning(b, &t);
        if (st == LULESH_OK) st = copy_state(false);
        if (st == LULESH_OK) st = replay(b, 1, nullptr);
        if (st == LULESH_OK) st = copy_state(false);
        if (st == LULESH_OK) st = replay(b, cycles, ms);
        return st;
    };
    int st = copy_state(true);
    lulesh_batch_tuning best = b->tuning;
    double best_ms = 1e300;
    if (st == LULESH_OK) st = measure(best, &best_ms);
    const int blocks[3] = {64, 128, 256}, per_sm[4] = {1, 2, 4, 8}, tiles[3] = {256, 1024, 4096};
    for (int bi = 0; bi < 3 && st == LULESH_OK; ++bi)
        for (int pi = 0; pi < 4 && st == LULESH_OK; ++pi)
            for (int ti = 0; ti < 3 && st == LULESH_OK; ++ti) {
                lulesh_batch_tuning t = best;
                for (int p = 0; p < 4; ++p) {
                    t.block[p] = blocks[bi];
                    t.blocks_per_sm[p] = per_sm[pi];
                }
                t.tile = tiles[ti];
                double ms = 0;
                st = measure(t, &ms);
                if (st == LULESH_OK && ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
    // per-phase refinement of block size and blocks per SM
    for (int p = 0; p < 4 && st == LULESH_OK; ++p)
        for (int bi = 0; bi < 3 && st == LULESH_OK; ++bi)
            for (int pi = 0; pi < 4 && st == LULESH_OK; ++pi) {
                lulesh_batch_tuning t = best;
                t.block[p] = blocks[bi];
                t.blocks_per_sm[p] = per_sm[pi];
                double ms = 0;
                st = measure(t, &ms);
                if (st == LULESH_OK && ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
    // per-phase tiles per queue access (fewer queue round trips for cheap tiles)
    const int grabs[4] = {1, 2, 4, 8};
    for (int p = 0; p < 4 && st == LULESH_OK; ++p)
        for (int gi = 0; gi < 4 && st == LULESH_OK; ++gi) {
            lulesh_batch_tuning t = best;
            t.grab[p] = grabs[gi];
            if (t.grab[p] == best.grab[p]) continue;
            double ms = 0;
            st = measure(t, &ms);
            if (st == LULESH_OK && ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
    best.ms_per_cycle = best_ms / cycles;
    const int st2 = copy_state(false);
    cudaFree(snap);
    if (st == LULESH_OK) st = st2;
    if (st == LULESH_OK) st = lulesh_batch_set_tuning(b, &best);
    if (st == LULESH_OK) b->tuning.ms_per_cycle = best.ms_per_cycle;
    if (chosen) *chosen = b->tuning;
    return st;
}
