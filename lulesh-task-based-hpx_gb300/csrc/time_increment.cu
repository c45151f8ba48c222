// Device-side time control for the CUDA-graph forms of the time loop.
// Built with --fmad=false: every operation is rounded as the host
// TimeIncrement rounds it, so the graph forms and the host loop pick
// identical time steps.
#include "lulesh_dev.h"

namespace lulesh {

// Loop condition of hpx_main (lulesh.cc:2374-2375) followed by
// TimeIncrement (lulesh.cc:182-229). Returns false when the loop has ended
// (or an error stopped it) and marks the state inactive.
__device__ __forceinline__ bool advance_time(DevTime* t, const StepResult* r) {
    if (t->max_cycles < 0 || r->err != 0 || !(t->time < t->stoptime && t->cycle < t->max_cycles)) {
        t->active = 0;
        return false;
    }
    t->active = 1;
    double targetdt = t->stoptime - t->time;
    if ((t->dtfixed <= 0.0) && (t->cycle != 0)) {
        const double olddt = t->deltatime;
        double gnewdt = 1.0e+20;
        if (t->dtcourant < gnewdt) gnewdt = t->dtcourant / 2.0;
        if (t->dthydro < gnewdt) gnewdt = t->dthydro * 2.0 / 3.0;
        double newdt = gnewdt;
        const double ratio = newdt / olddt;
        if (ratio >= 1.0) {
            if (ratio < t->deltatimemultlb) newdt = olddt;
            else if (ratio > t->deltatimemultub) newdt = olddt * t->deltatimemultub;
        }
        if (newdt > t->dtmax) newdt = t->dtmax;
        t->deltatime = newdt;
    }
    if ((targetdt > t->deltatime) && (targetdt < (4.0 * t->deltatime / 3.0)))
        targetdt = 2.0 * t->deltatime / 3.0;
    if (targetdt < t->deltatime) t->deltatime = targetdt;
    t->time += t->deltatime;
    ++t->cycle;
    return true;
}

// Single problem: one thread.
__global__ void k_time_increment(DevTime* t, const StepResult* r) { advance_time(t, r); }

// Stores the cycle's dt minima (lulesh.cc:2229-2236) and stops the loop on a
// device error.
__global__ void k_time_finish(DevTime* t, const StepResult* r) {
    if (!t->active) return;
    t->dtcourant = r->dtcourant;
    t->dthydro = r->dthydro;
    if (r->err != 0) t->active = 0;
}

// Batch: one thread per slot; re-arms the slot's dt minima (1e20, as
// lulesh.cc:2214-2215) and clears the per-phase tile queues.
__global__ void kb_time_increment(BatchCtl c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
        for (int k = 0; k < 4; ++k) c.queue[k] = 0u;
    if (i >= c.slots) return;
    if (advance_time(c.times + i, c.results + i)) {
        c.results[i].dtcourant = 1.0e+20;
        c.results[i].dthydro = 1.0e+20;
    }
}

__global__ void kb_time_finish(BatchCtl c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.slots) return;
    DevTime* t = c.times + i;
    const StepResult* r = c.results + i;
    if (!t->active) return;
    t->dtcourant = r->dtcourant;
    t->dthydro = r->dthydro;
    if (r->err != 0) t->active = 0;
}

int launch_time_increment(DevTime* t, StepResult* r, cudaStream_t s) {
    k_time_increment<<<1, 1, 0, s>>>(t, r);
    return 1;
}

int launch_time_finish(DevTime* t, StepResult* r, cudaStream_t s) {
    k_time_finish<<<1, 1, 0, s>>>(t, r);
    return 1;
}

int launch_batch_time_increment(const BatchCtl& c, cudaStream_t s) {
    kb_time_increment<<<blocks_for(c.slots, 128), 128, 0, s>>>(c);
    return 1;
}

int launch_batch_time_finish(const BatchCtl& c, cudaStream_t s) {
    kb_time_finish<<<blocks_for(c.slots, 128), 128, 0, s>>>(c);
    return 1;
}

}  // namespace lulesh
