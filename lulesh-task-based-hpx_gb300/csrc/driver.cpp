// lulesh-gb300: the reference program's command line and output on top of
// the GB300 C ABI.
//
// Flags as the reference registers them (lulesh.cc:2421-2432): --s --r --i
// --b --c --q --p, --f (accepted and ignored: it only sets the number of viz
// files) and --v, refused as the reference refuses it when built without viz
// output (lulesh-util.cc:48-54: message and exit(-1)); Silo viz output is not
// built here. --hpx:threads=N is accepted for drop-in command lines. Added:
// --precision fp64|fp64_exact|mixed and --graph (device TimeIncrement with
// the cycle replayed from a CUDA graph).
//
// Output: with --q the reference's CSV line "s,regions,cycles,threads,elapsed,e0"
// (lulesh.cc:2405-2407; threads = 1, the single GPU); otherwise the report of
// VerifyAndWriteFinalOutput (lulesh-util.cc:60-115).
#include <sys/time.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "lulesh_gb300.h"

namespace {

double now_s() {
    timeval t;
    gettimeofday(&t, nullptr);
    return double(t.tv_sec) + double(t.tv_usec) / 1e6;
}

int die(const char* what, int st) {
    std::fprintf(stderr, "%s: %s\n", what, lulesh_strerror(st));
    return st == LULESH_EVOLUME ? -1 : 2;
}

}  // namespace

int main(int argc, char** argv) {
    int its = 9999999, nx = 30, nr = 11, balance = 1, cost = 1, quiet = 0, prog = 0, graph = 0;
    int precision = LULESH_FP64;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a.rfind("--hpx:", 0) == 0) continue;
        // --name=value, which the reference's option parser accepts too
        std::string inline_value;
        bool has_inline = false;
        if (const size_t eq = a.find('='); eq != std::string::npos && a.rfind("--", 0) == 0) {
            inline_value = a.substr(eq + 1);
            a = a.substr(0, eq);
            has_inline = true;
        }
        if (a == "--q") { quiet = 1; continue; }
        if (a == "--p") { prog = 1; continue; }
        if (a == "--v") {
            std::printf("Use of --v requires a build with viz output (Silo); lulesh-gb300 has none\n");
            return -1;
        }
        if (a == "--graph") { graph = 1; continue; }
        if (!has_inline && i + 1 >= argc) {
            std::fprintf(stderr, "option %s needs a value\n", a.c_str());
            return 2;
        }
        std::string v = has_inline ? inline_value : std::string(argv[++i]);
        if (a == "--s") nx = std::atoi(v.c_str());
        else if (a == "--r") nr = std::atoi(v.c_str());
        else if (a == "--i") its = std::atoi(v.c_str());
        else if (a == "--b") balance = std::atoi(v.c_str());
        else if (a == "--c") cost = std::atoi(v.c_str());
        else if (a == "--f" || a == "--elems-per-task" || a == "--task-size") continue;
        else if (a == "--precision") {
            if (v == "fp64") precision = LULESH_FP64;
            else if (v == "fp64_exact") precision = LULESH_FP64_EXACT;
            else if (v == "mixed") precision = LULESH_MIXED;
            else {
                std::fprintf(stderr, "unknown precision %s\n", v.c_str());
                return 2;
            }
        } else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            return 2;
        }
    }

    lulesh_domain* dom = nullptr;
    int st = lulesh_domain_create(nx, nr, balance, cost, 1.0, &dom);
    if (st != LULESH_OK) return die("lulesh_domain_create", st);
    lulesh_domain_view* view = lulesh_domain_get_view(dom);
    lulesh_dev* dev = nullptr;
    st = lulesh_dev_create(view, precision, &dev);
    if (st != LULESH_OK) return die("lulesh_dev_create", st);

    if (!quiet) {
        std::printf("Running problem size %d^3 per domain until completion\n", nx);
        std::printf("Num processors: 1 (one GB300)\n");
        std::printf("Total number of elements: %lld \n\n", (long long)nx * nx * nx);
    }

    lulesh_time_state* ts = view->time;
    const double t0 = now_s();
    while (ts->time < ts->stoptime && ts->cycle < its) {
        // run in chunks of 100 cycles so --p can report progress as the
        // reference does every 100 cycles (lulesh.cc:2380-2385)
        const int target = (prog && !quiet) ? std::min(its, (ts->cycle / 100 + 1) * 100) : its;
        int32_t n = 0;
        st = graph ? lulesh_dev_run_graph(dev, ts, target, 64, &n) : lulesh_dev_run(dev, ts, target, &n);
        if (st != LULESH_OK) return die("step", st);
        if (prog && !quiet && ts->cycle % 100 == 0)
            std::printf("cycle = %d, time = %e, dt=%e\n", ts->cycle, ts->time, ts->deltatime);
        if (n == 0) break;
    }
    const double elapsed = now_s() - t0;

    // the final report is computed on the device: no field is downloaded
    lulesh_verify_result vr{};
    st = lulesh_dev_verify(dev, ts->cycle, &vr);
    if (st != LULESH_OK) return die("lulesh_dev_verify", st);
    if (quiet) {
        std::printf("%d,%d,%d,%d,%g,%12.6e\n", nx, nr, ts->cycle, 1, elapsed, vr.e0);
    } else {
        const double sym[3] = {vr.maxabs, vr.totabs, vr.maxrel};
        const double nz = double(nx) * nx * nx;
        const double grind = ts->cycle ? (elapsed * 1e6 / ts->cycle) / nz : 0.0;
        std::printf("Run completed:\n");
        std::printf("   Problem size        =  %d\n", nx);
        std::printf("   Iteration count     =  %d\n", ts->cycle);
        std::printf("   Final Origin Energy =  %12.6e\n", vr.e0);
        std::printf("   Testing Plane 0 of Energy Array on rank 0:\n");
        std::printf("        MaxAbsDiff   = %12.6e\n", sym[0]);
        std::printf("        TotalAbsDiff = %12.6e\n", sym[1]);
        std::printf("        MaxRelDiff   = %12.6e\n\n", sym[2]);
        std::printf("Elapsed time         = %10.2f (s)\n", elapsed);
        std::printf("Grind time (us/z/c)  = %10.8f (per dom)  (%10.8f overall)\n", grind, elapsed);
        std::printf("FOM                  = %10.8f (z/ms)  (%.6e zone-cycles/s)\n\n",
                    grind > 0 ? 1000.0 / grind : 0.0, grind > 0 ? 1e6 / grind : 0.0);
        std::printf("RESULT s=%d cycles=%d e0=%.17e maxabs=%.17e totabs=%.17e maxrel=%.17e\n", nx,
                    ts->cycle, vr.e0, sym[0], sym[1], sym[2]);
    }
    lulesh_dev_destroy(dev);
    lulesh_domain_destroy(dom);
    return 0;
}
