// Replacement for the reference's lulesh-util.cc, linked with the unmodified
// reference lulesh.cc / lulesh-init.cc / lulesh-viz.cc to build the oracle
// binary oracle/_ref/lulesh-ref. Test infrastructure only.
//
// It provides the two functions lulesh-util.cc defines:
//   ParseCommandLineOptions   - same options and defaults as lulesh-util.cc:36-56
//   VerifyAndWriteFinalOutput - the report of lulesh-util.cc:60-115 (cycle
//                               count, origin energy, plane-0 symmetry diffs),
//                               printed at full precision as one parseable
//                               line, plus an optional binary field dump.
//
// Field dump: when LULESH_DUMP names a file, the final Domain state is written
// there in the layout read by tests/golden tooling and by the oracle port
// (lulesh_oracle.c, lo_dump): magic "LULESHD1", int32 {s, numElem, numNode,
// cycle, numReg, 0}, double {time, deltatime, dtcourant, dthydro}, then the
// node arrays x y z xd yd zd xdd ydd zdd fx fy fz (numNode each) and the
// element arrays e p q ql qq v vnew delv vdov arealg ss (numElem each).
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstdint>
#include <vector>

#include "lulesh.h"

void ParseCommandLineOptions(hpx::program_options::variables_map& vm, Int_t myRank,
                             struct cmdLineOpts* opts) {
    (void)myRank;
    opts->its = vm["i"].as<Int_t>();
    opts->nx = vm["s"].as<Int_t>();
    opts->numReg = vm["r"].as<Int_t>();
    opts->numFiles = vm["f"].as<Int_t>();
    opts->balance = vm["b"].as<Int_t>();
    opts->cost = vm["c"].as<Int_t>();
    if (vm.count("p")) opts->showProg = 1;
    if (vm.count("q")) opts->quiet = 1;
    if (vm.count("v")) {
        std::printf("Use of -v requires compiling with -DVIZ_MESH\n");
        std::exit(-1);
    }
}

static void dump_fields(const char* path, Domain& d, Int_t nx) {
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        std::perror(path);
        std::exit(2);
    }
    const char magic[8] = {'L', 'U', 'L', 'E', 'S', 'H', 'D', '1'};
    std::fwrite(magic, 1, 8, f);
    int32_t hdr[6] = {nx, d.numElem(), d.numNode(), d.cycle(), d.numReg(), 0};
    std::fwrite(hdr, sizeof(int32_t), 6, f);
    double t[4] = {d.time(), d.deltatime(), d.dtcourant(), d.dthydro()};
    std::fwrite(t, sizeof(double), 4, f);
    const Index_t nn = d.numNode(), ne = d.numElem();
    std::vector<double> buf;
    auto put = [&](auto get, Index_t n) {
        buf.resize(n);
        for (Index_t i = 0; i < n; ++i) buf[i] = get(i);
        std::fwrite(buf.data(), sizeof(double), n, f);
    };
    put([&](Index_t i) { return d.x(i); }, nn);
    put([&](Index_t i) { return d.y(i); }, nn);
    put([&](Index_t i) { return d.z(i); }, nn);
    put([&](Index_t i) { return d.xd(i); }, nn);
    put([&](Index_t i) { return d.yd(i); }, nn);
    put([&](Index_t i) { return d.zd(i); }, nn);
    put([&](Index_t i) { return d.xdd(i); }, nn);
    put([&](Index_t i) { return d.ydd(i); }, nn);
    put([&](Index_t i) { return d.zdd(i); }, nn);
    put([&](Index_t i) { return d.fx(i); }, nn);
    put([&](Index_t i) { return d.fy(i); }, nn);
    put([&](Index_t i) { return d.fz(i); }, nn);
    put([&](Index_t i) { return d.e(i); }, ne);
    put([&](Index_t i) { return d.p(i); }, ne);
    put([&](Index_t i) { return d.q(i); }, ne);
    put([&](Index_t i) { return d.ql(i); }, ne);
    put([&](Index_t i) { return d.qq(i); }, ne);
    put([&](Index_t i) { return d.v(i); }, ne);
    put([&](Index_t i) { return d.vnew(i); }, ne);
    put([&](Index_t i) { return d.delv(i); }, ne);
    put([&](Index_t i) { return d.vdov(i); }, ne);
    put([&](Index_t i) { return d.arealg(i); }, ne);
    put([&](Index_t i) { return d.ss(i); }, ne);
    std::fclose(f);
}

void VerifyAndWriteFinalOutput(Real_t elapsed_time, Domain& locDom, Int_t nx, Int_t numRanks) {
    // Same plane-0 symmetry statistics as lulesh-util.cc:77-103.
    Real_t MaxAbsDiff = 0.0, TotalAbsDiff = 0.0, MaxRelDiff = 0.0;
    for (Index_t j = 0; j < nx; ++j) {
        for (Index_t k = j + 1; k < nx; ++k) {
            Real_t AbsDiff = FABS(locDom.e(j * nx + k) - locDom.e(k * nx + j));
            TotalAbsDiff += AbsDiff;
            if (MaxAbsDiff < AbsDiff) MaxAbsDiff = AbsDiff;
            Real_t RelDiff =
                FABS(locDom.e(k * nx + j)) > 1e-8 ? AbsDiff / locDom.e(k * nx + j) : 0.0;
            if (MaxRelDiff < RelDiff) MaxRelDiff = RelDiff;
        }
    }
    int64_t nx8 = nx;
    double grind = ((elapsed_time * 1e6) / locDom.cycle()) / double(nx8 * nx8 * nx8 * numRanks);
    std::printf(
        "RESULT s=%d cycles=%d e0=%.17e maxabs=%.17e totabs=%.17e maxrel=%.17e "
        "elapsed=%.6f grind_us=%.6f time=%.17e dt=%.17e\n",
        nx, locDom.cycle(), locDom.e(0), MaxAbsDiff, TotalAbsDiff, MaxRelDiff, elapsed_time,
        grind, locDom.time(), locDom.deltatime());
    if (const char* path = std::getenv("LULESH_DUMP")) dump_fields(path, locDom, nx);
}
