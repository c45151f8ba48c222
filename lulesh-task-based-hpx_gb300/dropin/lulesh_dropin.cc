// lulesh-dropin: the reference program's time loop with the GB300 step in
// place of LagrangeLeapFrogWithTasks (lulesh.cc:2361-2407), built against
// the reference's own, unmodified lulesh.h and lulesh-init.cc (its Domain
// and set-up) and liblulesh_gb300.so:
//
//   g++ -std=c++17 -O2 -I<hpx headers or a stand-in> -I<reference> -I<repo>/include
//       -I<repo>/lulesh-task-based-hpx_gb300/dropin lulesh_dropin.cc <reference>/lulesh-init.cc
//       -L<repo>/lulesh-task-based-hpx_gb300 -llulesh_gb300 -Wl,-rpath,<...>
//
// lulesh.cc itself defines main and keeps TimeIncrement file-local, so this
// program carries the loop of hpx_main and takes TimeIncrement from the
// library (lulesh_time_increment, the same steps); inside lulesh.cc the
// maintainer swaps the one call as lulesh_gb300_dropin.h shows.
//
//   lulesh-dropin [--s N] [--r N] [--b N] [--c N] [--i N] [--precision fp64|fp64_exact|mixed]
//       runs to stoptime (or --i cycles) on the GPU through LuleshGb300::leapfrog
//       and prints the reference's CSV line s,regions,cycles,threads,elapsed,e0
//   lulesh-dropin --check [--s N] [--r N] [--b N] [--c N]
//       host only: builds the reference's Domain and this library's host
//       Domain of the same problem and compares the view of the reference's
//       arrays with it, array by array (no GPU needed)
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "lulesh.h"
#include "lulesh_gb300_dropin.h"

namespace {

double now_s() {
    timeval t;
    gettimeofday(&t, nullptr);
    return double(t.tv_sec) + double(t.tv_usec) / 1e6;
}

// TimeIncrement (lulesh.cc:182-229) through the library on the Domain's fields.
void time_increment(Domain& d) {
    lulesh_time_state t = LuleshGb300::time_of(d);
    lulesh_time_increment(&t);
    d.time() = t.time;
    d.deltatime() = t.deltatime;
    d.cycle() = t.cycle;
}

template <class T>
int compare(const char* name, const T* a, const T* b, long n) {
    if (n == 0) return 0;
    if (!a || !b) {
        std::printf("mismatch %s: missing array\n", name);
        return 1;
    }
    for (long i = 0; i < n; ++i)
        if (std::memcmp(a + i, b + i, sizeof(T)) != 0) {
            std::printf("mismatch %s at %ld\n", name, i);
            return 1;
        }
    return 0;
}

// The view of the reference Domain against the library's own host Domain of
// the same problem: sizes, every array bit for bit, the parameters and the
// time state.
int check_view(Domain& d, int nx, int nr, int balance, int cost) {
    std::vector<Index_t> starts;
    lulesh_time_state ts = LuleshGb300::time_of(d);
    lulesh_domain_view v;
    LuleshGb300::make_view(d, starts, &ts, v);
    lulesh_domain* mine = nullptr;
    if (lulesh_domain_create(nx, nr, balance, cost, 1.0, &mine) != LULESH_OK) return 2;
    const lulesh_domain_view& w = *lulesh_domain_get_view(mine);
    int bad = 0;
    const int32_t sv[8] = {v.numElem, v.numNode, v.sizeX, v.numReg, v.cost, v.numSymmX, v.numSymmY, v.numSymmZ};
    const int32_t sw[8] = {w.numElem, w.numNode, w.sizeX, w.numReg, w.cost, w.numSymmX, w.numSymmY, w.numSymmZ};
    bad += compare("sizes", sv, sw, 8);
    if (bad) return bad;
    const long ne = v.numElem, nn = v.numNode;
    bad += compare("x", v.x, w.x, nn) + compare("y", v.y, w.y, nn) + compare("z", v.z, w.z, nn);
    bad += compare("xd", v.xd, w.xd, nn) + compare("yd", v.yd, w.yd, nn) + compare("zd", v.zd, w.zd, nn);
    bad += compare("xdd", v.xdd, w.xdd, nn) + compare("fx", v.fx, w.fx, nn);
    bad += compare("nodalMass", v.nodalMass, w.nodalMass, nn);
    bad += compare("symmX", v.symmX, w.symmX, v.numSymmX) + compare("symmY", v.symmY, w.symmY, v.numSymmY) +
           compare("symmZ", v.symmZ, w.symmZ, v.numSymmZ);
    bad += compare("nodelist", v.nodelist, w.nodelist, 8 * ne);
    bad += compare("lxim", v.lxim, w.lxim, ne) + compare("lxip", v.lxip, w.lxip, ne) +
           compare("letam", v.letam, w.letam, ne) + compare("letap", v.letap, w.letap, ne) +
           compare("lzetam", v.lzetam, w.lzetam, ne) + compare("lzetap", v.lzetap, w.lzetap, ne);
    bad += compare("elemBC", v.elemBC, w.elemBC, ne);
    bad += compare("e", v.e, w.e, ne) + compare("p", v.p, w.p, ne) + compare("q", v.q, w.q, ne);
    bad += compare("v", v.v, w.v, ne) + compare("ss", v.ss, w.ss, ne);
    bad += compare("volo", v.volo, w.volo, ne) + compare("elemMass", v.elemMass, w.elemMass, ne);
    bad += compare("nodeElemStart", v.nodeElemStart, w.nodeElemStart, nn + 1);
    bad += compare("nodeElemCornerList", v.nodeElemCornerList, w.nodeElemCornerList, long(v.nodeElemStart[nn]));
    bad += compare("regNumList", v.regNumList, w.regNumList, ne);
    bad += compare("params", &v.params, &w.params, 1);
    const lulesh_time_state& tw = *w.time;
    const double a[9] = {ts.time, ts.deltatime, ts.dtcourant, ts.dthydro, ts.dtfixed,
                         ts.deltatimemultlb, ts.deltatimemultub, ts.dtmax, ts.stoptime};
    const double b[9] = {tw.time, tw.deltatime, tw.dtcourant, tw.dthydro, tw.dtfixed,
                         tw.deltatimemultlb, tw.deltatimemultub, tw.dtmax, tw.stoptime};
    bad += compare("time state", a, b, 9);
    lulesh_domain_destroy(mine);
    if (!bad) std::printf("view ok: s=%d r=%d b=%d c=%d, %d elements, %d nodes\n", nx, nr, balance, cost,
                          v.numElem, v.numNode);
    return bad;
}

}  // namespace

int main(int argc, char** argv) {
    int nx = 30, nr = 11, balance = 1, cost = 1, its = 9999999, check = 0;
    int32_t precision = LULESH_FP64;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--check") {
            check = 1;
            continue;
        }
        if (i + 1 >= argc) {
            std::fprintf(stderr, "option %s needs a value\n", a.c_str());
            return 2;
        }
        const std::string v = argv[++i];
        if (a == "--s") nx = std::atoi(v.c_str());
        else if (a == "--r") nr = std::atoi(v.c_str());
        else if (a == "--b") balance = std::atoi(v.c_str());
        else if (a == "--c") cost = std::atoi(v.c_str());
        else if (a == "--i") its = std::atoi(v.c_str());
        else if (a == "--precision")
            precision = v == "mixed" ? LULESH_MIXED : v == "fp64_exact" ? LULESH_FP64_EXACT : LULESH_FP64;
        else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            return 2;
        }
    }
    // the set-up of hpx_main (lulesh.cc:2361-2366), one rank
    Int_t col, row, plane, side;
    InitMeshDecomp(1, 0, &col, &row, &plane, &side);
    Domain* locDom = new Domain(1, col, row, plane, nx, side, nr, balance, cost);
    if (check) {
        const int bad = check_view(*locDom, nx, nr, balance, cost);
        delete locDom;
        return bad ? 1 : 0;
    }

    LuleshGb300 gpu;
    int st = gpu.attach(*locDom, precision);
    if (st != LULESH_OK) {
        std::fprintf(stderr, "lulesh_dev_create: %s\n", lulesh_strerror(st));
        return 2;
    }
    const double t0 = now_s();
    while ((locDom->time() < locDom->stoptime()) && (locDom->cycle() < its)) {
        time_increment(*locDom);
        st = gpu.leapfrog(*locDom);  // was: LagrangeLeapFrogWithTasks(*locDom);
        if (st == LULESH_EVOLUME) std::exit(VolumeError);
        if (st != LULESH_OK) {
            std::fprintf(stderr, "lulesh_leapfrog: %s\n", lulesh_strerror(st));
            return 2;
        }
    }
    const double elapsed = now_s() - t0;
    // the reference's CSV line (lulesh.cc:2405-2407), threads = 1 (one GPU)
    std::printf("%d,%d,%d,%d,%g,%12.6e\n", nx, nr, locDom->cycle(), 1, elapsed, locDom->e(0));
    delete locDom;
    return 0;
}
