// Serving loop with continuous batching on top of the batch pool.
//
// One host thread. Requests whose arrival time has passed queue up in
// arrival order; the loop admits them into the resident batch as slots and
// pool memory free up (each problem built directly in its pool block by the
// device build, so admission costs milliseconds and no host Domain), replays
// cycles of every resident problem from the batch's CUDA graph in chunks of
// about sync_ms of device time (the chunk adapts to the measured cycle time),
// and retires finished problems with their final report computed on the
// device. Requests that arrive while others run join the next chunk, so
// their work overlaps on the device with the problems already resident.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <numeric>
#include <thread>
#include <vector>

#include "lulesh_dev.h"

namespace {

// Quantile q of v with linear interpolation between order statistics (the
// sample quantile of Hyndman and Fan's definition 7): for fewer than 100
// samples p99 lies between the two largest instead of being the largest.
double quantile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double h = q * double(v.size() - 1);
    const size_t lo = size_t(std::floor(h));
    const size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (h - double(lo)) * (v[hi] - v[lo]);
}

}  // namespace

extern "C" int lulesh_serve(int32_t precision, uint64_t hbm_budget, int32_t max_slots,
                            const lulesh_request* reqs, int32_t n, double sync_ms,
                            lulesh_request_result* results, lulesh_serve_stats* stats) {
    if (!reqs || !results || n < 1 || max_slots < 1 || !(sync_ms > 0.0)) return LULESH_EINVAL;
    for (int i = 0; i < n; ++i) {
        uint64_t need = 0;
        const int st = lulesh_batch_footprint(precision, reqs[i].problem.s, &need);
        if (st != LULESH_OK) return st;
        if (need > hbm_budget) return LULESH_EINVAL;  // could never be admitted
        if (!(reqs[i].arrival_s >= 0.0)) return LULESH_EINVAL;
    }
    lulesh_batch* b = nullptr;
    int st = lulesh_batch_create(precision, hbm_budget, max_slots, &b);
    if (st != LULESH_OK) return st;

    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return reqs[a].arrival_s < reqs[c].arrival_s; });
    for (int i = 0; i < n; ++i) {
        results[i] = lulesh_request_result{};
        results[i].arrival_s = reqs[i].arrival_s;
        results[i].s = reqs[i].problem.s;
    }

    using clock = std::chrono::steady_clock;
    const auto t0 = clock::now();
    auto now_s = [&] { return std::chrono::duration<double>(clock::now() - t0).count(); };

    size_t next = 0;              // next request (arrival order) not yet queued
    std::deque<int> pending;      // arrived, waiting for a slot and pool memory
    std::map<int, int> inflight;  // slot -> request
    std::vector<lulesh_slot_status> status(max_slots);
    std::map<int, uint64_t> slot_bytes;  // slot -> pool bytes of its problem
    int done = 0, chunk = 8, max_resident = 0;
    uint64_t resident_bytes = 0, peak_bytes = 0;
    double device_ms = 0.0;
    while (st == LULESH_OK && done < n) {
        const double t = now_s();
        while (next < order.size() && reqs[order[next]].arrival_s <= t) pending.push_back(order[next++]);
        // admit in arrival order; one that does not fit yet waits while later,
        // smaller ones may go first
        for (auto it = pending.begin(); it != pending.end();) {
            int32_t slot = -1;
            const int a = lulesh_batch_admit(b, &reqs[*it].problem, &slot);
            if (a == LULESH_ENOMEM) {
                ++it;
                continue;
            }
            if (a != LULESH_OK) {
                st = a;
                break;
            }
            results[*it].admitted_s = now_s();
            inflight[slot] = *it;
            uint64_t need = 0;
            lulesh_batch_footprint(precision, reqs[*it].problem.s, &need);
            slot_bytes[slot] = need;
            resident_bytes += need;
            it = pending.erase(it);
        }
        if (st != LULESH_OK) break;
        max_resident = std::max(max_resident, int(inflight.size()));
        peak_bytes = std::max(peak_bytes, resident_bytes);
        if (inflight.empty()) {
            // nothing resident (every request fits the empty pool, so none is
            // pending): sleep until the next arrival, in short steps
            if (next < order.size()) {
                const double wait = reqs[order[next]].arrival_s - now_s();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
            }
            continue;
        }
        int32_t active = 0;
        double ms = 0.0;
        st = lulesh_batch_run(b, chunk, &active, &ms);
        if (st != LULESH_OK) break;
        device_ms += ms;
        const double per_cycle = ms / chunk;
        if (per_cycle > 0) chunk = std::max(1, std::min(512, int(sync_ms / per_cycle)));
        st = lulesh_batch_status(b, status.data(), max_slots);
        if (st != LULESH_OK) break;
        for (auto it = inflight.begin(); it != inflight.end();) {
            const lulesh_slot_status& ss = status[it->first];
            if (ss.active) {
                ++it;
                continue;
            }
            lulesh_request_result& r = results[it->second];
            r.finished_s = now_s();
            r.time_to_solution_s = r.finished_s - r.arrival_s;
            r.cycles = ss.cycle;
            r.err = ss.err;
            r.zone_cycles = int64_t(ss.numElem) * ss.cycle;
            // the final report on the device: no field leaves the GPU
            lulesh_verify_result vr{};
            st = lulesh_batch_verify(b, it->first, &vr);
            r.e0 = vr.e0;
            r.maxabs = vr.maxabs;
            r.totabs = vr.totabs;
            r.maxrel = vr.maxrel;
            if (st == LULESH_OK) st = lulesh_batch_retire(b, it->first);
            if (st != LULESH_OK) break;
            resident_bytes -= slot_bytes[it->first];
            slot_bytes.erase(it->first);
            it = inflight.erase(it);
            ++done;
        }
    }
    const int64_t launches = lulesh_batch_launch_count(b);
    lulesh_batch_destroy(b);
    if (st != LULESH_OK) return st;

    if (stats) {
        std::vector<double> tts(n), queued(n);
        double last = 0.0;
        int64_t zc = 0;
        for (int i = 0; i < n; ++i) {
            tts[i] = results[i].time_to_solution_s;
            queued[i] = results[i].admitted_s - results[i].arrival_s;
            last = std::max(last, results[i].finished_s);
            zc += results[i].zone_cycles;
        }
        *stats = lulesh_serve_stats{};
        stats->wall_s = last;
        stats->device_s = device_ms / 1e3;
        stats->zone_cycles = zc;
        stats->zone_cycles_per_s = last > 0 ? double(zc) / last : 0.0;
        stats->p50_s = quantile(tts, 0.50);
        stats->p99_s = quantile(tts, 0.99);
        stats->mean_s = std::accumulate(tts.begin(), tts.end(), 0.0) / n;
        stats->launches = launches;
        stats->served = done;
        stats->max_resident = max_resident;
        stats->peak_resident_bytes = int64_t(peak_bytes);
        stats->p50_queue_s = quantile(queued, 0.50);
        stats->p99_queue_s = quantile(queued, 0.99);
    }
    return LULESH_OK;
}
