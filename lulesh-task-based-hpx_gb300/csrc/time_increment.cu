// Device-side time control for the CUDA-graph form of the time loop.
// Built with --fmad=false: every operation is rounded as the host
// TimeIncrement rounds it, so the graph form and the host loop pick
// identical time steps.
#include "lulesh_dev.h"

namespace lulesh {

// Loop condition of hpx_main (lulesh.cc:2374-2375) followed by
// TimeIncrement (lulesh.cc:182-229); a single thread.
__global__ void k_time_increment(DevTime* t, const StepResult* r) {
    if (r->err != 0 || !(t->time < t->stoptime && t->cycle < t->max_cycles)) {
        t->active = 0;
        return;
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
}

// Stores the cycle's dt minima (lulesh.cc:2229-2236) and stops the loop on a
// device error.
__global__ void k_time_finish(DevTime* t, const StepResult* r) {
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

}  // namespace lulesh
