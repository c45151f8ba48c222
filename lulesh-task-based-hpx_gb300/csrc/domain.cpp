// Host-side Domain of the Sedov problem and the host scalar routines of the
// time loop.
//
// HostDomain keeps the reference Domain's SoA layout (lulesh.h:465-605) and
// builds the same initial state as Domain::Domain (lulesh-init.cc:10-183):
// uniform cube of edge 1.125, node->corner CSR, glibc rand() region sets,
// symmetry node sets, face neighbours and BC masks, volumes, masses, origin
// energy and the analytic first dt. Region assignment must draw the same
// rand() sequence as the reference, so it keeps the reference's order of
// draws (lulesh-init.cc:366-415).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "lulesh_dev.h"
#include "portable_cbrt.h"

namespace lulesh {

struct HostDomain {
    int s = 0, numElem = 0, numNode = 0, numReg = 0, cost = 0, balance = 0;
    std::vector<double> x, y, z, xd, yd, zd, xdd, ydd, zdd, fx, fy, fz, nodalMass;
    std::vector<int32_t> symmX, symmY, symmZ;
    std::vector<int32_t> nodelist, lxim, lxip, letam, letap, lzetam, lzetap, elemBC;
    std::vector<double> e, p, q, ql, qq, v, vnew, delv, vdov, arealg, ss, volo, elemMass;
    std::vector<int32_t> nodeElemStart, nodeElemCornerList, regNumList;
    lulesh_time_state ts{};
    lulesh_domain_view view{};

    void build(int s_, int nr, int balance_, int cost_, double energy_scale);

   private:
    void mesh();
    void corner_csr();
    void regions();
    void symmetry();
    void connectivity();
    void fill_view();
};

// CalcElemVolume (lulesh.cc:592-665), used for the initial volumes.
static double hex_volume_host(const double x[8], const double y[8], const double z[8]) {
    auto tp = [](double x1, double y1, double z1, double x2, double y2, double z2, double x3,
                 double y3, double z3) {
        return x1 * (y2 * z3 - z2 * y3) + x2 * (z1 * y3 - y1 * z3) + x3 * (y1 * z2 - z1 * y2);
    };
    const double twelveth = 1.0 / 12.0;
    double dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    double dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    double dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    double dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    double dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    double dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    double dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    double dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    double dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    double dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    double dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    double dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
    double vol = tp(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
                 tp(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
                 tp(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
    vol *= twelveth;
    return vol;
}

void HostDomain::mesh() {
    const int en = s + 1;
    int n = 0;
    for (int pl = 0; pl < en; ++pl)
        for (int row = 0; row < en; ++row)
            for (int col = 0; col < en; ++col, ++n) {
                x[n] = 1.125 * double(col) / double(s);
                y[n] = 1.125 * double(row) / double(s);
                z[n] = 1.125 * double(pl) / double(s);
            }
    // element (col,row,plane) -> its 8 corner nodes, counter-clockwise on
    // the bottom face then the top face (lulesh-init.cc:236-244)
    int el = 0;
    for (int pl = 0; pl < s; ++pl)
        for (int row = 0; row < s; ++row)
            for (int col = 0; col < s; ++col, ++el) {
                const int base = (pl * en + row) * en + col;
                int32_t* c = &nodelist[8 * size_t(el)];
                c[0] = base;
                c[1] = base + 1;
                c[2] = base + en + 1;
                c[3] = base + en;
                c[4] = base + en * en;
                c[5] = base + en * en + 1;
                c[6] = base + en * en + en + 1;
                c[7] = base + en * en + en;
            }
}

void HostDomain::corner_csr() {
    std::vector<int32_t> count(numNode, 0);
    for (size_t k = 0; k < nodelist.size(); ++k) ++count[nodelist[k]];
    nodeElemStart[0] = 0;
    for (int n = 0; n < numNode; ++n) nodeElemStart[n + 1] = nodeElemStart[n] + count[n];
    std::fill(count.begin(), count.end(), 0);
    for (int el = 0; el < numElem; ++el)
        for (int k = 0; k < 8; ++k) {
            const int nd = nodelist[8 * size_t(el) + k];
            nodeElemCornerList[nodeElemStart[nd] + count[nd]++] = 8 * el + k;
        }
}

void region_runs(int numElem, int numReg, int balance, std::vector<RegionRun>& runs) {
    runs.clear();
    srand(0);
    if (numReg == 1) {
        runs.push_back({0, numElem, 1});
        return;
    }
    std::vector<int> binEnd(numReg);
    int costDen = 0;
    for (int r = 0; r < numReg; ++r) {
        costDen += std::pow(r + 1, balance);  // truncated to int, as the reference does
        binEnd[r] = costDen;
    }
    auto draw_region = [&]() {
        const int var = rand() % costDen;
        int r = 0;
        while (var >= binEnd[r]) ++r;
        return (r % numReg) + 1;
    };
    int next = 0, last = -1;
    while (next < numElem) {
        int reg = draw_region();
        while (reg == last) reg = draw_region();
        const int bin = rand() % 1000;
        int run;
        if (bin < 773) run = rand() % 15 + 1;
        else if (bin < 937) run = rand() % 16 + 16;
        else if (bin < 970) run = rand() % 32 + 32;
        else if (bin < 974) run = rand() % 64 + 64;
        else if (bin < 978) run = rand() % 128 + 128;
        else if (bin < 981) run = rand() % 256 + 256;
        else run = rand() % 1537 + 512;
        const int count = std::min(run, numElem - next);
        runs.push_back({next, count, reg});
        next += count;
        last = reg;
    }
}

void default_params(lulesh_params& P) {
    P = lulesh_params{};
    P.e_cut = 1.0e-7;
    P.p_cut = 1.0e-7;
    P.q_cut = 1.0e-7;
    P.v_cut = 1.0e-10;
    P.u_cut = 1.0e-7;
    P.hgcoef = 3.0;
    P.ss4o3 = 4.0 / 3.0;
    P.qstop = 1.0e+12;
    P.monoq_max_slope = 1.0;
    P.monoq_limiter_mult = 2.0;
    P.qlc_monoq = 0.5;
    P.qqc_monoq = 2.0 / 3.0;
    P.qqc = 2.0;
    P.eosvmax = 1.0e+9;
    P.eosvmin = 1.0e-9;
    P.pmin = 0.0;
    P.emin = -1.0e+15;
    P.dvovmax = 0.1;
    P.refdens = 1.0;
}

void initial_time_state(int s, double energy_scale, lulesh_time_state& ts, double& einit) {
    ts = lulesh_time_state{};
    ts.dtfixed = -1.0e-6;
    ts.stoptime = 1.0e-2;
    ts.deltatimemultlb = 1.1;
    ts.deltatimemultub = 1.2;
    ts.dtcourant = 1.0e+20;
    ts.dthydro = 1.0e+20;
    ts.dtmax = 1.0e-2;
    ts.time = 0.0;
    ts.cycle = 0;
    const double ebase = 3.948746e+7;
    const double scale = s / 45.0;
    einit = ebase * scale * scale * scale;
    if (energy_scale != 1.0) einit = einit * energy_scale;
    // element 0's volume from its corner coordinates (as mesh() places them)
    double xl[8], yl[8], zl[8];
    const int dc[8] = {0, 1, 1, 0, 0, 1, 1, 0}, dr[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    for (int k = 0; k < 8; ++k) {
        xl[k] = 1.125 * double(dc[k]) / double(s);
        yl[k] = 1.125 * double(dr[k]) / double(s);
        zl[k] = 1.125 * double(k / 4) / double(s);
    }
    ts.deltatime = (.5 * cbrt(hex_volume_host(xl, yl, zl))) / sqrt(2.0 * einit);
}

void HostDomain::regions() {
    std::vector<RegionRun> runs;
    region_runs(numElem, numReg, balance, runs);
    for (const RegionRun& r : runs) std::fill_n(regNumList.begin() + r.first, r.count, r.reg);
}

void HostDomain::symmetry() {
    const int en = s + 1;
    int k = 0;
    for (int i = 0; i < en; ++i)
        for (int j = 0; j < en; ++j, ++k) {
            symmZ[k] = i * en + j;
            symmY[k] = i * en * en + j;
            symmX[k] = i * en * en + j * en;
        }
}

void HostDomain::connectivity() {
    const int ne = numElem, s2 = s * s;
    for (int i = 0; i < ne; ++i) {
        lxim[i] = (i == 0) ? 0 : i - 1;
        lxip[i] = (i == ne - 1) ? ne - 1 : i + 1;
        letam[i] = (i < s) ? i : i - s;
        letap[i] = (i >= ne - s) ? i : i + s;
        lzetam[i] = (i < s2) ? i : i - s2;
        lzetap[i] = (i >= ne - s2) ? i : i + s2;
        elemBC[i] = 0;
    }
    // one domain: symmetry on the minus faces, free surface on the plus faces
    for (int i = 0; i < s; ++i)
        for (int j = 0; j < s; ++j) {
            const int planeInc = i * s2, rowInc = i * s;
            elemBC[rowInc + j] |= ZETA_M_SYMM;
            elemBC[rowInc + j + ne - s2] |= ZETA_P_FREE;
            elemBC[planeInc + j] |= ETA_M_SYMM;
            elemBC[planeInc + j + s2 - s] |= ETA_P_FREE;
            elemBC[planeInc + j * s] |= XI_M_SYMM;
            elemBC[planeInc + j * s + s - 1] |= XI_P_FREE;
        }
}

void HostDomain::build(int s_, int nr, int balance_, int cost_, double energy_scale) {
    s = s_;
    numReg = nr;
    balance = balance_;
    cost = cost_;
    numElem = s * s * s;
    numNode = (s + 1) * (s + 1) * (s + 1);
    const size_t nn = numNode, ne = numElem, ns = size_t(s + 1) * (s + 1);
    for (auto* f : {&x, &y, &z, &xd, &yd, &zd, &xdd, &ydd, &zdd, &fx, &fy, &fz, &nodalMass})
        f->assign(nn, 0.0);
    for (auto* f : {&symmX, &symmY, &symmZ}) f->assign(ns, 0);
    nodelist.assign(8 * ne, 0);
    for (auto* f : {&lxim, &lxip, &letam, &letap, &lzetam, &lzetap, &elemBC, &regNumList})
        f->assign(ne, 0);
    for (auto* f : {&e, &p, &q, &ql, &qq, &vnew, &delv, &vdov, &arealg, &ss, &volo, &elemMass})
        f->assign(ne, 0.0);
    v.assign(ne, 1.0);
    nodeElemStart.assign(nn + 1, 0);
    nodeElemCornerList.assign(8 * ne, 0);

    mesh();
    corner_csr();
    regions();
    symmetry();
    connectivity();

    double einit = 0.0;
    initial_time_state(s, energy_scale, ts, einit);

    for (int el = 0; el < numElem; ++el) {
        double xl[8], yl[8], zl[8];
        const int32_t* c = &nodelist[8 * size_t(el)];
        for (int k = 0; k < 8; ++k) {
            xl[k] = x[c[k]];
            yl[k] = y[c[k]];
            zl[k] = z[c[k]];
        }
        const double vol = hex_volume_host(xl, yl, zl);
        volo[el] = vol;
        elemMass[el] = vol;
        for (int k = 0; k < 8; ++k) nodalMass[c[k]] += vol / 8.0;
    }
    e[0] = einit;
    fill_view();
}

void HostDomain::fill_view() {
    lulesh_domain_view& w = view;
    w = lulesh_domain_view{};
    w.numElem = numElem;
    w.numNode = numNode;
    w.sizeX = s;
    w.numReg = numReg;
    w.cost = cost;
    w.numSymmX = w.numSymmY = w.numSymmZ = int32_t(symmX.size());
    w.x = x.data(); w.y = y.data(); w.z = z.data();
    w.xd = xd.data(); w.yd = yd.data(); w.zd = zd.data();
    w.xdd = xdd.data(); w.ydd = ydd.data(); w.zdd = zdd.data();
    w.fx = fx.data(); w.fy = fy.data(); w.fz = fz.data();
    w.nodalMass = nodalMass.data();
    w.symmX = symmX.data(); w.symmY = symmY.data(); w.symmZ = symmZ.data();
    w.nodelist = nodelist.data();
    w.lxim = lxim.data(); w.lxip = lxip.data(); w.letam = letam.data();
    w.letap = letap.data(); w.lzetam = lzetam.data(); w.lzetap = lzetap.data();
    w.elemBC = elemBC.data();
    w.e = e.data(); w.p = p.data(); w.q = q.data(); w.ql = ql.data(); w.qq = qq.data();
    w.v = v.data(); w.vnew = vnew.data(); w.delv = delv.data(); w.vdov = vdov.data();
    w.arealg = arealg.data(); w.ss = ss.data();
    w.volo = volo.data(); w.elemMass = elemMass.data();
    w.nodeElemStart = nodeElemStart.data();
    w.nodeElemCornerList = nodeElemCornerList.data();
    w.regNumList = regNumList.data();
    default_params(w.params);
    w.time = &ts;
}

}  // namespace lulesh

struct lulesh_domain {
    lulesh::HostDomain d;
};

namespace {
// Calls f(pointer, bytes) for every host array a step reads or writes.
template <class F>
void for_each_mutable(lulesh::HostDomain& h, F&& f) {
    for (auto* v : {&h.x, &h.y, &h.z, &h.xd, &h.yd, &h.zd, &h.xdd, &h.ydd, &h.zdd, &h.fx, &h.fy,
                    &h.fz, &h.e, &h.p, &h.q, &h.ql, &h.qq, &h.v, &h.vnew, &h.delv, &h.vdov,
                    &h.arealg, &h.ss})
        f(v->data(), v->size() * sizeof(double));
}
}  // namespace

extern "C" {

int lulesh_domain_create(int32_t s, int32_t nr, int32_t balance, int32_t cost, double energy_scale,
                         lulesh_domain** out) {
    if (!out) return LULESH_EINVAL;
    *out = nullptr;
    // s^3 elements and 8 s^3 corner indices must fit Index_t (int32)
    if (s < 1 || s > 640 || nr < 1 || nr > 1000000 || balance < 0 || cost < 0 ||
        !(energy_scale > 0.0))
        return LULESH_EINVAL;
    lulesh_domain* d = new (std::nothrow) lulesh_domain;
    if (!d) return LULESH_ENOMEM;
    try {
        d->d.build(s, nr, balance, cost, energy_scale);
    } catch (const std::bad_alloc&) {
        delete d;
        return LULESH_ENOMEM;
    }
    *out = d;
    return LULESH_OK;
}

lulesh_domain_view* lulesh_domain_get_view(lulesh_domain* d) { return d ? &d->d.view : nullptr; }

int lulesh_domain_pin(lulesh_domain* d, int32_t pin) {
    if (!d) return LULESH_EINVAL;
    int st = LULESH_OK;
    for_each_mutable(d->d, [&](void* p, size_t bytes) {
        const cudaError_t e = pin ? cudaHostRegister(p, bytes, cudaHostRegisterDefault)
                                  : cudaHostUnregister(p);
        if (e != cudaSuccess && st == LULESH_OK) st = LULESH_ECUDA;
    });
    return st;
}

void lulesh_domain_destroy(lulesh_domain* d) { delete d; }

int lulesh_time_increment(lulesh_time_state* t) {
    if (!t) return LULESH_EINVAL;
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
    return LULESH_OK;
}

int lulesh_symmetry(const lulesh_domain_view* v, double out[3]) {
    if (!v || !out || !v->e || v->sizeX < 1) return LULESH_EINVAL;
    const int nx = v->sizeX;
    double maxAbs = 0.0, totAbs = 0.0, maxRel = 0.0;
    for (int j = 0; j < nx; ++j)
        for (int k = j + 1; k < nx; ++k) {
            const double a = std::fabs(v->e[j * nx + k] - v->e[k * nx + j]);
            totAbs += a;
            if (maxAbs < a) maxAbs = a;
            const double r = std::fabs(v->e[k * nx + j]) > 1e-8 ? a / v->e[k * nx + j] : 0.0;
            if (maxRel < r) maxRel = r;
        }
    out[0] = maxAbs;
    out[1] = totAbs;
    out[2] = maxRel;
    return LULESH_OK;
}

double lulesh_cbrt_portable(double x) { return lulesh::cbrt_portable(x); }

const char* lulesh_strerror(int32_t st) {
    switch (st) {
        case LULESH_OK: return "ok";
        case LULESH_EVOLUME: return "VolumeError: non-positive element volume";
        case LULESH_EQSTOP: return "QStopError";
        case LULESH_EINVAL: return "invalid argument";
        case LULESH_ECUDA: return "CUDA runtime error";
        case LULESH_ENOMEM: return "out of memory";
        case LULESH_ENODEV: return "no CUDA device";
        case LULESH_ETIMEOUT: return "device-side wait timed out";
        default: return "unknown status";
    }
}

}  // extern "C"
