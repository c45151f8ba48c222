// Serving loop with continuous batching on top of the batch pool.
//
// Two host threads. The preparation thread waits for each request's arrival
// time and builds its Domain on the host (the reference's set-up, which is
// the slow part of admission for large s). The serving thread admits built
// requests into the resident batch as slots and pool memory free up, replays
// cycles of every resident problem from the batch's CUDA graph in chunks of
// about sync_ms of device time (the chunk adapts to the measured cycle time),
// and retires finished problems. Requests that arrive while others run join
// the next chunk, so their work overlaps on the device with the problems
// already resident.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "lulesh_dev.h"

namespace {

struct Built {
    int idx;
    lulesh_domain* dom;
};

double quantile(std::vector<double> v, double q) {  // nearest rank
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    size_t k = size_t(std::ceil(q * double(v.size())));
    k = std::min(std::max<size_t>(k, 1), v.size());
    return v[k - 1];
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

    std::mutex mu;
    std::condition_variable cv;
    std::deque<Built> ready;
    bool stop = false;
    int prep_error = LULESH_OK;
    std::thread prep([&] {
        for (int idx : order) {
            for (;;) {
                std::unique_lock<std::mutex> lk(mu);
                if (stop) return;
                const double wait = reqs[idx].arrival_s - now_s();
                if (wait <= 0) break;
                cv.wait_for(lk, std::chrono::duration<double>(std::min(wait, 0.05)));
            }
            const lulesh_problem& p = reqs[idx].problem;
            lulesh_domain* dom = nullptr;
            const int e = lulesh_domain_create(p.s, p.nr, p.balance, p.cost, p.energy_scale, &dom);
            std::lock_guard<std::mutex> lk(mu);
            if (e != LULESH_OK) {
                prep_error = e;
                cv.notify_all();
                return;
            }
            ready.push_back({idx, dom});
            cv.notify_all();
        }
    });

    std::map<int, int> inflight;  // slot -> request
    std::vector<lulesh_slot_status> status(max_slots);
    int done = 0, chunk = 8, max_resident = 0;
    double device_ms = 0.0;
    while (st == LULESH_OK && done < n) {
        {
            std::unique_lock<std::mutex> lk(mu);
            if (prep_error != LULESH_OK) {
                st = prep_error;
                break;
            }
            for (auto it = ready.begin(); it != ready.end();) {
                const lulesh_problem& p = reqs[it->idx].problem;
                int32_t slot = -1;
                const int a = lulesh_batch_admit_view(b, lulesh_domain_get_view(it->dom), p.stoptime,
                                                      p.max_cycles, &slot);
                if (a == LULESH_ENOMEM) {  // not yet: a later, smaller request may fit
                    ++it;
                    continue;
                }
                if (a != LULESH_OK) {
                    st = a;
                    break;
                }
                results[it->idx].admitted_s = now_s();
                inflight[slot] = it->idx;
                lulesh_domain_destroy(it->dom);
                it = ready.erase(it);
            }
            if (st != LULESH_OK) break;
            max_resident = std::max(max_resident, int(inflight.size()));
            if (inflight.empty()) {
                cv.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
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
            st = lulesh_batch_origin_energy(b, it->first, &r.e0);
            if (st == LULESH_OK) st = lulesh_batch_retire(b, it->first);
            if (st != LULESH_OK) break;
            it = inflight.erase(it);
            ++done;
        }
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
        cv.notify_all();
    }
    prep.join();
    for (Built& x : ready) lulesh_domain_destroy(x.dom);
    const int64_t launches = lulesh_batch_launch_count(b);
    lulesh_batch_destroy(b);
    if (st != LULESH_OK) return st;

    if (stats) {
        std::vector<double> tts(n);
        double last = 0.0;
        int64_t zc = 0;
        for (int i = 0; i < n; ++i) {
            tts[i] = results[i].time_to_solution_s;
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
    }
    return LULESH_OK;
}
