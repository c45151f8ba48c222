// C ABI of the device path: handle life cycle, host<->device copies, one
// cycle, and the two forms of the time loop (host TimeIncrement per cycle, or
// device TimeIncrement with the cycle replayed from a CUDA graph).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "lulesh_dev.h"

namespace {

using lulesh::DevTime;
using lulesh::Mesh;
using lulesh::StepResult;

struct Launchers {
    int (*forces)(const Mesh&, cudaStream_t);
    int (*nodes)(const Mesh&, double, cudaStream_t);
    int (*kinematics)(const Mesh&, double, cudaStream_t);
    int (*material)(const Mesh&, cudaStream_t);
    int (*forces_range)(const Mesh&, int, int, cudaStream_t);
    int (*material_range)(const Mesh&, int, int, bool, cudaStream_t);
    // the resident loop's geometry form (fast double variant; else null):
    // kinematics store the element geometry the next forces read
    int (*forces_geo)(const Mesh&, cudaStream_t);
    int (*kinematics_geo)(const Mesh&, double, cudaStream_t);
    int (*geometry)(const Mesh&, cudaStream_t);
    // lulesh_leapfrog's kinematics slabs: elements [first, end)
    int (*kinematics_range)(const Mesh&, double, int, int, cudaStream_t);
    int (*kinematics_geo_range)(const Mesh&, double, int, int, cudaStream_t);
};

Launchers launchers_for(int precision) {
    switch (precision) {
        case LULESH_FP64:
            return {lulesh::fp64::launch_forces, lulesh::fp64::launch_nodes,
                    lulesh::fp64::launch_kinematics, lulesh::fp64::launch_material,
                    lulesh::fp64::launch_forces_range, lulesh::fp64::launch_material_range,
                    lulesh::fp64::launch_forces_geo, lulesh::fp64::launch_kinematics_geo,
                    lulesh::fp64::launch_geometry, lulesh::fp64::launch_kinematics_range, lulesh::fp64::launch_kinematics_geo_range};
        case LULESH_FP64_EXACT:
            return {lulesh::fp64x::launch_forces, lulesh::fp64x::launch_nodes,
                    lulesh::fp64x::launch_kinematics, lulesh::fp64x::launch_material,
                    lulesh::fp64x::launch_forces_range, lulesh::fp64x::launch_material_range,
                    nullptr, nullptr, nullptr, lulesh::fp64x::launch_kinematics_range, nullptr};
        default:
            return {lulesh::mixed::launch_forces, lulesh::mixed::launch_nodes,
                    lulesh::mixed::launch_kinematics, lulesh::mixed::launch_material,
                    lulesh::mixed::launch_forces_range, lulesh::mixed::launch_material_range,
                    nullptr, nullptr, nullptr, lulesh::mixed::launch_kinematics_range, nullptr};
    }
}

// Carves typed arrays out of one device allocation (256-byte aligned).
struct Arena {
    size_t used = 0;
    char* base = nullptr;
    template <class T>
    T* take(size_t n) {
        used = (used + 255) & ~size_t(255);
        T* p = base ? reinterpret_cast<T*>(base + used) : nullptr;
        used += n * sizeof(T);
        return p;
    }
};

}  // namespace

struct lulesh_dev {
    int precision = LULESH_FP64;
    cudaStream_t stream = nullptr;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    Mesh m{};
    StepResult* h_result = nullptr;  // pinned: [0] the step's, [1 + k] material slab k's (lulesh_leapfrog)
    DevTime* d_time = nullptr;
    DevTime* h_time = nullptr;       // pinned
    cudaGraphExec_t graph = nullptr;
    int graph_kernels = 0;
    int64_t launches = 0;
    int32_t err_elem = -1;
    int32_t nx = 0;                  // edge of the cube (Domain::sizeX)
    double* d_verify = nullptr;      // [4] lulesh_dev_verify output (arena)
    double* h_verify = nullptr;      // [4] pinned
    // lulesh_leapfrog's upload and download streams and its hand-off events
    // (created on first use)
    cudaStream_t cstream = nullptr;  // uploads
    cudaStream_t mstream = nullptr;  // downloads of the compute stream's results
    cudaStream_t stream2 = nullptr;  // second compute stream: every other slab
    cudaStream_t mstream2 = nullptr; // downloads of the second compute stream's results
    cudaStream_t nstream = nullptr;  // the node ranges, beside the force slabs
    cudaEvent_t ev_up = nullptr, ev_e = nullptr, ev_s2 = nullptr, ev_join = nullptr, ev_s1 = nullptr;
    // one per slab: upload, mirror (mixed), node range, kinematics and material done
    std::vector<cudaEvent_t> ev_slab, ev_mir, ev_node, ev_kin, ev_mat;
    // lulesh_leapfrog's stage timeline (lulesh_leapfrog_timeline): mark 0 is
    // the call's first device work, marks 1.. the stage boundaries
    bool tl_on = false;
    cudaEvent_t tl_ev[LULESH_TL_MAX + 1] = {};
    int tl_n = 0;
    lulesh_timeline tl_last{};
    int32_t* upload_flag = nullptr;  // [kLeapfrogSlabs] per-slab "host changed a coordinate" (arena)
    StepResult* slab_result = nullptr;  // [kLeapfrogSlabs] per material slab: dt minima and block counter
    int32_t* matOrderSlab = nullptr;           // [N_e] slab-major material order (arena)
    Launchers L{};
    // m.geo holds the geometry of the current coordinates (set by the
    // geometry form's kinematics and the geometry pass; cleared by anything
    // that writes coordinates or runs the phases another way)
    bool geo_valid = false;
    // lulesh_leapfrog's copies of the uploaded coordinates (with m.geo)
    double* stage[3] = {nullptr, nullptr, nullptr};
    // device-side timing (lulesh_dev_profile_begin/end)
    bool profiling = false;
    cudaEvent_t ev[2][5] = {};  // per-phase boundaries; two sets, for a cycle and the next one's forces
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    cudaEvent_t ev_done = nullptr;  // a cycle's readback of its dt minima and error word
    double kernel_ms[4] = {0, 0, 0, 0};
    int64_t prof_cycles = 0, prof_launch0 = 0;
};

// Slabs of lulesh_leapfrog (element planes per slab = s / slabs). At s=150
// the drop-in ran at 3.79e8, 3.82e8 and 3.60e8 zone-cycles/s with 4, 8 and
// 16 slabs: fewer leave more of the copies exposed, more add copy and
// launch overhead.
constexpr int kLeapfrogSlabs = 8;

// Slabs of a handle's problem: whole element planes of the cube of edge s
// (one slab when the mesh is not an s^3 cube).
int slab_count(int s, int64_t numElem) {
    const bool cube = s >= 1 && int64_t(s) * s * s == numElem;
    return cube ? std::min(s, kLeapfrogSlabs) : 1;
}
// Element planes [p0, p1) of slab sl.
void slab_planes(int s, int slabs, int sl, int& p0, int& p1) {
    p0 = int(int64_t(s) * sl / slabs);
    p1 = int(int64_t(s) * (sl + 1) / slabs);
}

#define CK(call)                                          \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return LULESH_ECUDA;       \
    } while (0)

namespace {

int check_view(const lulesh_domain_view* v) {
    if (!v || v->numElem < 1 || v->numNode < 8 || v->numReg < 1 || v->cost < 0) return LULESH_EINVAL;
    if ((int64_t)v->numElem * 8 > INT32_MAX) return LULESH_EINVAL;
    const void* req[] = {v->x, v->y, v->z, v->xd, v->yd, v->zd, v->xdd, v->ydd, v->zdd, v->fx,
                         v->fy, v->fz, v->nodalMass, v->nodelist, v->lxim, v->lxip, v->letam,
                         v->letap, v->lzetam, v->lzetap, v->elemBC, v->e, v->p, v->q, v->ql,
                         v->qq, v->v, v->vnew, v->delv, v->vdov, v->arealg, v->ss, v->volo,
                         v->elemMass, v->nodeElemStart, v->nodeElemCornerList, v->regNumList};
    for (const void* p : req)
        if (!p) return LULESH_EINVAL;
    const int ne = v->numElem, nn = v->numNode;
    // every index the kernels dereference must stay inside its array
    for (int64_t k = 0; k < 8LL * ne; ++k)
        if (v->nodelist[k] < 0 || v->nodelist[k] >= nn) return LULESH_EINVAL;
    const int32_t* nb[] = {v->lxim, v->lxip, v->letam, v->letap, v->lzetam, v->lzetap};
    for (const int32_t* a : nb)
        for (int i = 0; i < ne; ++i)
            if (a[i] < 0 || a[i] >= ne) return LULESH_EINVAL;
    if (v->nodeElemStart[0] != 0) return LULESH_EINVAL;
    for (int n = 0; n < nn; ++n)
        if (v->nodeElemStart[n + 1] < v->nodeElemStart[n]) return LULESH_EINVAL;
    if (v->nodeElemStart[nn] != 8 * ne) return LULESH_EINVAL;
    for (int64_t k = 0; k < 8LL * ne; ++k)
        if (v->nodeElemCornerList[k] < 0 || v->nodeElemCornerList[k] >= 8 * ne) return LULESH_EINVAL;
    for (int i = 0; i < ne; ++i)
        if (v->regNumList[i] < 1 || v->regNumList[i] > v->numReg) return LULESH_EINVAL;
    for (int n = 0; n < nn; ++n)
        if (!(v->nodalMass[n] > 0.0)) return LULESH_EINVAL;  // a = f / m needs m > 0
    const int32_t* sy[] = {v->symmX, v->symmY, v->symmZ};
    const int32_t cnt[] = {v->numSymmX, v->numSymmY, v->numSymmZ};
    for (int a = 0; a < 3; ++a) {
        if (cnt[a] < 0 || (cnt[a] > 0 && !sy[a])) return LULESH_EINVAL;
        for (int k = 0; k < cnt[a]; ++k)
            if (sy[a][k] < 0 || sy[a][k] >= nn) return LULESH_EINVAL;
    }
    return LULESH_OK;
}

// Lays out the mesh arrays of one problem in the arena; with base == null it
// only measures.
void carve_mesh(Mesh& m, Arena& a, int precision, int ne, int nn) {
    const bool mixed = precision == LULESH_MIXED;
    m.geo = nullptr;
    for (double** f : {&m.x, &m.y, &m.z, &m.xd, &m.yd, &m.zd, &m.xdd, &m.ydd, &m.zdd, &m.fx, &m.fy,
                       &m.fz})
        *f = a.take<double>(nn);
    m.nodalMass = a.take<double>(nn);
    m.invMass = a.take<double>(nn);
    m.nodeSymm = a.take<uint8_t>(nn);
    m.nodelist = a.take<int32_t>(8 * size_t(ne));
    for (const int32_t** f : {&m.lxim, &m.lxip, &m.letam, &m.letap, &m.lzetam, &m.lzetap, &m.elemBC})
        *f = a.take<int32_t>(ne);
    for (double** f : {&m.e, &m.p, &m.q, &m.ql, &m.qq, &m.v, &m.vnew, &m.delv, &m.vdov, &m.arealg,
                       &m.ss})
        *f = a.take<double>(ne);
    m.volo = a.take<double>(ne);
    m.elemMass = a.take<double>(ne);
    m.nodeElemStart = a.take<int32_t>(size_t(nn) + 1);
    m.nodeElemCornerList = a.take<int32_t>(8 * size_t(ne));
    m.matOrder = a.take<int32_t>(ne);
    m.elemRep = a.take<int32_t>(ne);
    if (mixed) {
        for (float2** f : {&m.pxp, &m.pyp, &m.pzp, &m.vxp, &m.vyp, &m.vzp}) *f = a.take<float2>(nn);
        for (float** f : {&m.fcx, &m.fcy, &m.fcz}) *f = a.take<float>(8 * size_t(ne));
        for (float** f : {&m.gvxi, &m.gveta, &m.gvzeta, &m.gxxi, &m.gxeta, &m.gxzeta})
            *f = a.take<float>(ne);
    } else {
        for (double** f : {&m.fsx, &m.fsy, &m.fsz}) *f = a.take<double>(8 * size_t(ne));
        // separate hourglass corner forces only for the exact variant
        if (precision == LULESH_FP64_EXACT)
            for (double** f : {&m.fhx, &m.fhy, &m.fhz}) *f = a.take<double>(8 * size_t(ne));
        for (double** f : {&m.dvxi, &m.dveta, &m.dvzeta, &m.dxxi, &m.dxeta, &m.dxzeta})
            *f = a.take<double>(ne);
        // the fast double variant's element geometry (kinematics -> next forces)
        if (precision == LULESH_FP64) m.geo = a.take<double>(size_t(lulesh::kGeoWords) * ne);
    }
}

// Every device array of a single-problem handle: the mesh, then the
// reduction scratch and the graph form's time state.
void layout(lulesh_dev* d, Arena& a, int ne, int nn, int matGrid) {
    Mesh& m = d->m;
    carve_mesh(m, a, d->precision, ne, nn);
    // one partial per block of the material launch: the full grid, or the
    // slab launches of lulesh_leapfrog with one thread per element, each in
    // its own part (at most one block more per slab than one launch over all)
    m.partials = a.take<lulesh::DtPartial>(
        std::max(matGrid, lulesh::blocks_for(ne, lulesh::kMatBlock) + kLeapfrogSlabs));
    m.result = a.take<StepResult>(1);
    for (double*& p : d->stage) p = d->L.forces_geo ? a.take<double>(nn) : nullptr;
    d->upload_flag = a.take<int32_t>(kLeapfrogSlabs);
    d->slab_result = a.take<StepResult>(kLeapfrogSlabs);
    d->d_time = a.take<DevTime>(1);
    d->d_verify = a.take<double>(4);
    d->matOrderSlab = a.take<int32_t>(ne);
}

struct Copy {
    void* dev;
    const void* host;
    size_t bytes;
};

// The (device, host) pairs of the field groups in `mask`.
std::vector<Copy> groups(const Mesh& m, const lulesh_domain_view* v, uint32_t mask) {
    const size_t nb = sizeof(double) * size_t(m.numNode), eb = sizeof(double) * size_t(m.numElem);
    std::vector<Copy> c;
    if (mask & LULESH_F_POS) c.insert(c.end(), {{m.x, v->x, nb}, {m.y, v->y, nb}, {m.z, v->z, nb}});
    if (mask & LULESH_F_VEL) c.insert(c.end(), {{m.xd, v->xd, nb}, {m.yd, v->yd, nb}, {m.zd, v->zd, nb}});
    if (mask & LULESH_F_ACC)
        c.insert(c.end(), {{m.xdd, v->xdd, nb}, {m.ydd, v->ydd, nb}, {m.zdd, v->zdd, nb}});
    if (mask & LULESH_F_FORCE)
        c.insert(c.end(), {{m.fx, v->fx, nb}, {m.fy, v->fy, nb}, {m.fz, v->fz, nb}});
    if (mask & LULESH_F_EPQ) c.insert(c.end(), {{m.e, v->e, eb}, {m.p, v->p, eb}, {m.q, v->q, eb}});
    if (mask & LULESH_F_V) c.push_back({m.v, v->v, eb});
    if (mask & LULESH_F_QLQQ) c.insert(c.end(), {{m.ql, v->ql, eb}, {m.qq, v->qq, eb}});
    if (mask & LULESH_F_KIN)
        c.insert(c.end(), {{m.vnew, v->vnew, eb}, {m.delv, v->delv, eb}, {m.vdov, v->vdov, eb},
                           {m.arealg, v->arealg, eb}});
    if (mask & LULESH_F_SS) c.push_back({m.ss, v->ss, eb});
    if (mask & LULESH_F_MESH) {
        const size_t ib = sizeof(int32_t) * size_t(m.numElem);
        c.insert(c.end(), {{const_cast<double*>(m.nodalMass), v->nodalMass, nb},
                           {const_cast<double*>(m.volo), v->volo, eb},
                           {const_cast<double*>(m.elemMass), v->elemMass, eb},
                           {const_cast<int32_t*>(m.nodelist), v->nodelist, 8 * ib},
                           {const_cast<int32_t*>(m.lxim), v->lxim, ib},
                           {const_cast<int32_t*>(m.lxip), v->lxip, ib},
                           {const_cast<int32_t*>(m.letam), v->letam, ib},
                           {const_cast<int32_t*>(m.letap), v->letap, ib},
                           {const_cast<int32_t*>(m.lzetam), v->lzetam, ib},
                           {const_cast<int32_t*>(m.lzetap), v->lzetap, ib},
                           {const_cast<int32_t*>(m.elemBC), v->elemBC, ib},
                           {const_cast<int32_t*>(m.nodeElemStart), v->nodeElemStart,
                            sizeof(int32_t) * (size_t(m.numNode) + 1)},
                           {const_cast<int32_t*>(m.nodeElemCornerList), v->nodeElemCornerList, 8 * ib}});
    }
    return c;
}

// Uploads topology, derived per-node/per-element arrays and the whole
// mutable state of v into the carved mesh m, refreshes the mixed path's
// float-pair mirrors, and waits for the copies (some read host vectors that
// live only in this call).
int upload_mesh(const Mesh& m, const lulesh_domain_view* v, int precision, cudaStream_t s, int slabs,
                int32_t* slab_order) {
    const int ne = v->numElem, nn = v->numNode;
    // per-node symmetry bits, per-element EOS repeat count and the
    // repeat-count grouping of the material phase
    std::vector<uint8_t> symm(nn, 0);
    for (int k = 0; k < v->numSymmX; ++k) symm[v->symmX[k]] |= 1;
    for (int k = 0; k < v->numSymmY; ++k) symm[v->symmY[k]] |= 2;
    for (int k = 0; k < v->numSymmZ; ++k) symm[v->symmZ[k]] |= 4;
    std::vector<double> invMass(nn);
    for (int k = 0; k < nn; ++k) invMass[k] = 1.0 / v->nodalMass[k];
    std::vector<int32_t> rep(ne), order(ne);
    for (int i = 0; i < ne; ++i) rep[i] = lulesh::region_rep(v->regNumList[i] - 1, v->numReg, v->cost);
    for (int i = 0; i < ne; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rep[a] > rep[b]; });
    std::vector<int32_t> sorder;
    if (slab_order && slabs > 1) {
        // the same order split by slab of whole element planes (a stable
        // partition: repeat-count order within each slab)
        const int sx = v->sizeX, s2 = sx * sx;
        std::vector<int> slab_of(sx);
        for (int sl = 0; sl < slabs; ++sl) {
            int p0, p1;
            slab_planes(sx, slabs, sl, p0, p1);
            for (int pl = p0; pl < p1; ++pl) slab_of[pl] = sl;
        }
        sorder = order;
        std::stable_sort(sorder.begin(), sorder.end(),
                         [&](int a, int b) { return slab_of[a / s2] < slab_of[b / s2]; });
        CK(cudaMemcpyAsync(slab_order, sorder.data(), sizeof(int32_t) * size_t(ne), cudaMemcpyHostToDevice, s));
    }

    const size_t eb = sizeof(int32_t) * size_t(ne);
    const Copy consts[] = {
        {const_cast<double*>(m.nodalMass), v->nodalMass, sizeof(double) * size_t(nn)},
        {const_cast<double*>(m.invMass), invMass.data(), sizeof(double) * size_t(nn)},
        {const_cast<uint8_t*>(m.nodeSymm), symm.data(), size_t(nn)},
        {const_cast<int32_t*>(m.nodelist), v->nodelist, 8 * eb},
        {const_cast<int32_t*>(m.lxim), v->lxim, eb},
        {const_cast<int32_t*>(m.lxip), v->lxip, eb},
        {const_cast<int32_t*>(m.letam), v->letam, eb},
        {const_cast<int32_t*>(m.letap), v->letap, eb},
        {const_cast<int32_t*>(m.lzetam), v->lzetam, eb},
        {const_cast<int32_t*>(m.lzetap), v->lzetap, eb},
        {const_cast<int32_t*>(m.elemBC), v->elemBC, eb},
        {const_cast<double*>(m.volo), v->volo, sizeof(double) * size_t(ne)},
        {const_cast<double*>(m.elemMass), v->elemMass, sizeof(double) * size_t(ne)},
        {const_cast<int32_t*>(m.nodeElemStart), v->nodeElemStart, sizeof(int32_t) * (size_t(nn) + 1)},
        {const_cast<int32_t*>(m.nodeElemCornerList), v->nodeElemCornerList, 8 * eb},
        {const_cast<int32_t*>(m.matOrder), order.data(), eb},
        {const_cast<int32_t*>(m.elemRep), rep.data(), eb},
    };
    for (const Copy& c : consts) CK(cudaMemcpyAsync(c.dev, c.host, c.bytes, cudaMemcpyHostToDevice, s));
    for (const Copy& c : groups(m, v, LULESH_F_ALL))
        CK(cudaMemcpyAsync(c.dev, c.host, c.bytes, cudaMemcpyHostToDevice, s));
    if (precision == LULESH_MIXED) {
        lulesh::mixed::launch_mirror(m, s);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
}

// A cycle in three parts, so that the host loop can queue the next cycle's
// force phase, which reads neither dt nor the time, before it waits for the
// current cycle's dt minima (lulesh_dev_run). `set` picks the profiling
// events of the cycle (two sets: a cycle's and the next one's forces).
//
// The force phase: the error word cleared, the element geometry formed where
// it is stale, forces.
int queue_forces(lulesh_dev* d, int set) {
    const Mesh& m = d->m;
    const bool prof = d->profiling;
    CK(cudaMemsetAsync(&m.result->err, 0, 3 * sizeof(int32_t), d->stream));
    const bool geo = d->L.forces_geo != nullptr;
    if (prof) CK(cudaEventRecord(d->ev[set][0], d->stream));
    if (geo) {
        if (!d->geo_valid) d->launches += d->L.geometry(m, d->stream);
        d->launches += d->L.forces_geo(m, d->stream);
    } else {
        d->launches += d->L.forces(m, d->stream);
    }
    if (prof) CK(cudaEventRecord(d->ev[set][1], d->stream));
    return LULESH_OK;
}
// The rest of the cycle with time step dt, then the readback of its dt
// minima and error word (event ev_done).
int queue_rest(lulesh_dev* d, double dt, int set) {
    const Mesh& m = d->m;
    const bool prof = d->profiling;
    const bool geo = d->L.forces_geo != nullptr;
    if (!d->ev_done) CK(cudaEventCreateWithFlags(&d->ev_done, cudaEventDisableTiming));
    d->launches += d->L.nodes(m, dt, d->stream);
    if (prof) CK(cudaEventRecord(d->ev[set][2], d->stream));
    d->launches += geo ? d->L.kinematics_geo(m, dt, d->stream) : d->L.kinematics(m, dt, d->stream);
    d->geo_valid = geo;
    if (prof) CK(cudaEventRecord(d->ev[set][3], d->stream));
    d->launches += d->L.material(m, d->stream);
    if (prof) CK(cudaEventRecord(d->ev[set][4], d->stream));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(d->h_result, m.result, sizeof(StepResult), cudaMemcpyDeviceToHost, d->stream));
    CK(cudaEventRecord(d->ev_done, d->stream));
    return LULESH_OK;
}
// Waits for the cycle's readback (not for work queued after it) and returns
// its status.
int finish_cycle(lulesh_dev* d, int set) {
    CK(cudaEventSynchronize(d->ev_done));
    if (d->profiling) {
        for (int k = 0; k < 4; ++k) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, d->ev[set][k], d->ev[set][k + 1]));
            d->kernel_ms[k] += ms;
        }
        ++d->prof_cycles;
    }
    if (d->h_result->err != 0) {
        d->err_elem = d->h_result->err_elem;
        return d->h_result->err;
    }
    return LULESH_OK;
}

int run_cycle(lulesh_dev* d, double dt) {
    int st = queue_forces(d, 0);
    if (st == LULESH_OK) st = queue_rest(d, dt, 0);
    return st == LULESH_OK ? finish_cycle(d, 0) : st;
}

int build_graph(lulesh_dev* d) {
    if (d->graph) return LULESH_OK;
    Mesh gm = d->m;
    gm.dtime = d->d_time;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
    int k = 0;
    const bool geo = d->L.forces_geo != nullptr;
    k += lulesh::launch_time_increment(d->d_time, gm.result, d->stream);
    k += geo ? d->L.forces_geo(gm, d->stream) : d->L.forces(gm, d->stream);
    k += d->L.nodes(gm, 0.0, d->stream);
    k += geo ? d->L.kinematics_geo(gm, 0.0, d->stream) : d->L.kinematics(gm, 0.0, d->stream);
    k += d->L.material(gm, d->stream);
    k += lulesh::launch_time_finish(d->d_time, gm.result, d->stream);
    cudaError_t ce = cudaStreamEndCapture(d->stream, &g);
    if (ce != cudaSuccess) return LULESH_ECUDA;
    ce = cudaGraphInstantiate(&d->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        d->graph = nullptr;
        return LULESH_ECUDA;
    }
    d->graph_kernels = k;
    return LULESH_OK;
}

// A handle for ne elements and nn nodes: the arena carved, the stream and
// the pinned result buffers created, the device result word cleared. The
// mesh arrays are left for the caller to fill.
int new_handle(int32_t precision, int ne, int nn, lulesh_dev** out) {
    if (precision != LULESH_FP64 && precision != LULESH_FP64_EXACT && precision != LULESH_MIXED)
        return LULESH_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return LULESH_ENODEV;
    int dev_id = 0, sms = 0;
    CK(cudaGetDevice(&dev_id));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
    lulesh_dev* d = new (std::nothrow) lulesh_dev;
    if (!d) return LULESH_ENOMEM;
    d->precision = precision;
    d->L = launchers_for(precision);
    // Material blocks per SM of the grid-stride launch (elements in
    // repeat-count order; 6 blocks of 78 registers fit per SM): a sweep of
    // 6, 8, 12 per SM and one thread per element at s=150 gave the double
    // kernel 1.38, 1.34, 1.37, 1.51 ms and the mixed kernel 0.92, 0.98, 0.95,
    // 1.08 ms
    const int mat_per_sm = precision == LULESH_MIXED ? 6 : 8;
    const int matGrid = std::max(1, std::min(lulesh::blocks_for(ne, lulesh::kMatBlock), sms * mat_per_sm));
    Arena measure;
    layout(d, measure, ne, nn, matGrid);
    d->arena_bytes = measure.used;
    auto fail = [&](int code) {
        lulesh_dev_destroy(d);
        return code;
    };
    if (cudaMalloc(&d->arena, d->arena_bytes) != cudaSuccess) return fail(LULESH_ENOMEM);
    Arena carve;
    carve.base = static_cast<char*>(d->arena);
    layout(d, carve, ne, nn, matGrid);
    Mesh& m = d->m;
    m.numElem = ne;
    m.numNode = nn;
    m.matGrid = matGrid;
    m.dtime = nullptr;
    if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(LULESH_ECUDA);
    if (cudaMallocHost(&d->h_result, sizeof(StepResult) * (1 + kLeapfrogSlabs)) != cudaSuccess)
        return fail(LULESH_ENOMEM);
    if (cudaMallocHost(&d->h_time, sizeof(DevTime)) != cudaSuccess) return fail(LULESH_ENOMEM);
    if (cudaMallocHost(&d->h_verify, 4 * sizeof(double)) != cudaSuccess) return fail(LULESH_ENOMEM);
    if (cudaMemsetAsync(m.result, 0, sizeof(StepResult), d->stream) != cudaSuccess)
        return fail(LULESH_ECUDA);
    *out = d;
    return LULESH_OK;
}

}  // namespace

extern "C" {

int lulesh_dev_create(const lulesh_domain_view* v, int32_t precision, lulesh_dev** out) {
    if (!out) return LULESH_EINVAL;
    *out = nullptr;
    int st = check_view(v);
    if (st != LULESH_OK) return st;
    lulesh_dev* d = nullptr;
    st = new_handle(precision, v->numElem, v->numNode, &d);
    if (st != LULESH_OK) return st;
    d->m.prm = v->params;
    d->nx = v->sizeX;
    st = upload_mesh(d->m, v, precision, d->stream, slab_count(v->sizeX, v->numElem), d->matOrderSlab);
    if (st != LULESH_OK) {
        lulesh_dev_destroy(d);
        return st;
    }
    if (precision == LULESH_MIXED) ++d->launches;  // the float-pair mirror kernel
    *out = d;
    return LULESH_OK;
}

int lulesh_dev_create_problem(const lulesh_problem* p, int32_t precision, lulesh_time_state* ts,
                              lulesh_dev** out) {
    if (!out || !ts) return LULESH_EINVAL;
    *out = nullptr;
    int st = lulesh::check_problem(p);
    if (st != LULESH_OK) return st;
    const int ne = p->s * p->s * p->s, nn = (p->s + 1) * (p->s + 1) * (p->s + 1);
    lulesh_dev* d = nullptr;
    st = new_handle(precision, ne, nn, &d);
    if (st != LULESH_OK) return st;
    d->nx = p->s;
    st = lulesh::mesh_fill_problem(d->m, p, precision, d->stream, ts, nullptr, slab_count(p->s, ne),
                                   d->matOrderSlab);
    if (st != LULESH_OK) {
        lulesh_dev_destroy(d);
        return st;
    }
    // the build kernels, the material orders (and the mirror)
    d->launches += 5 + (slab_count(p->s, ne) > 1 ? 1 : 0) + (precision == LULESH_MIXED ? 1 : 0);
    *out = d;
    return LULESH_OK;
}

void lulesh_dev_destroy(lulesh_dev* d) {
    if (!d) return;
    if (d->stream) cudaStreamSynchronize(d->stream);
    for (auto& set : d->ev)
        for (cudaEvent_t e : set)
            if (e) cudaEventDestroy(e);
    if (d->ev_done) cudaEventDestroy(d->ev_done);
    for (cudaEvent_t e : d->tl_ev)
        if (e) cudaEventDestroy(e);
    if (d->ev_begin) cudaEventDestroy(d->ev_begin);
    if (d->ev_end) cudaEventDestroy(d->ev_end);
    if (d->graph) cudaGraphExecDestroy(d->graph);
    if (d->arena) cudaFree(d->arena);
    if (d->h_result) cudaFreeHost(d->h_result);
    if (d->h_time) cudaFreeHost(d->h_time);
    if (d->h_verify) cudaFreeHost(d->h_verify);
    if (d->cstream) cudaStreamSynchronize(d->cstream);
    for (cudaEvent_t e : {d->ev_up, d->ev_e, d->ev_s2, d->ev_join, d->ev_s1})
        if (e) cudaEventDestroy(e);
    for (auto* evs : {&d->ev_slab, &d->ev_mir, &d->ev_node, &d->ev_kin, &d->ev_mat})
        for (cudaEvent_t e : *evs) cudaEventDestroy(e);
    for (cudaStream_t st : {d->stream2, d->mstream2, d->nstream}) {
        if (!st) continue;
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (d->mstream) {
        cudaStreamSynchronize(d->mstream);
        cudaStreamDestroy(d->mstream);
    }
    if (d->cstream) cudaStreamDestroy(d->cstream);
    if (d->stream) cudaStreamDestroy(d->stream);
    delete d;
}

int lulesh_dev_verify(lulesh_dev* d, int32_t cycle, lulesh_verify_result* out) {
    if (!d || !out) return LULESH_EINVAL;
    const int nx = d->nx;
    if (nx < 1 || int64_t(nx) * nx * nx != int64_t(d->m.numElem)) return LULESH_EINVAL;
    d->launches += lulesh::launch_verify(d->m.e, nx, d->d_verify, d->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(d->h_verify, d->d_verify, 4 * sizeof(double), cudaMemcpyDeviceToHost, d->stream));
    CK(cudaStreamSynchronize(d->stream));
    out->e0 = d->h_verify[0];
    out->maxabs = d->h_verify[1];
    out->totabs = d->h_verify[2];
    out->maxrel = d->h_verify[3];
    out->cycle = cycle;
    out->nx = nx;
    return LULESH_OK;
}

int lulesh_dev_upload(lulesh_dev* d, const lulesh_domain_view* v, uint32_t mask) {
    if (!d || !v || v->numElem != d->m.numElem || v->numNode != d->m.numNode) return LULESH_EINVAL;
    if (mask & LULESH_F_MESH) return LULESH_EINVAL;  // the mesh is fixed at creation
    if (mask & LULESH_F_POS) d->geo_valid = false;  // the element geometry follows the coordinates
    for (const Copy& c : groups(d->m, v, mask)) {
        if (!c.host) return LULESH_EINVAL;
        CK(cudaMemcpyAsync(c.dev, c.host, c.bytes, cudaMemcpyHostToDevice, d->stream));
    }
    if (d->precision == LULESH_MIXED && (mask & (LULESH_F_POS | LULESH_F_VEL))) {
        d->launches += lulesh::mixed::launch_mirror(d->m, d->stream);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(d->stream));
    return LULESH_OK;
}

int lulesh_dev_download(lulesh_dev* d, lulesh_domain_view* v, uint32_t mask) {
    if (!d || !v || v->numElem != d->m.numElem || v->numNode != d->m.numNode) return LULESH_EINVAL;
    for (const Copy& c : groups(d->m, v, mask)) {
        if (!c.host) return LULESH_EINVAL;
        CK(cudaMemcpyAsync(const_cast<void*>(c.host), c.dev, c.bytes, cudaMemcpyDeviceToHost, d->stream));
    }
    CK(cudaStreamSynchronize(d->stream));
    return LULESH_OK;
}

int lulesh_dev_step(lulesh_dev* d, double dt, double* dtcourant, double* dthydro) {
    if (!d || !(dt > 0.0)) return LULESH_EINVAL;
    const int st = run_cycle(d, dt);
    if (st != LULESH_OK) return st;
    if (dtcourant) *dtcourant = d->h_result->dtcourant;
    if (dthydro) *dthydro = d->h_result->dthydro;
    return LULESH_OK;
}

int lulesh_leapfrog(lulesh_dev* d, lulesh_domain_view* v) {
    if (!d || !v || !v->time || v->numElem != d->m.numElem || v->numNode != d->m.numNode)
        return LULESH_EINVAL;
    if (!(v->time->deltatime > 0.0)) return LULESH_EINVAL;
    // The coordinates come from the host buffers. With the geometry form they
    // upload into copies, and slabs whose nodes the host left as the previous
    // step made them reuse the geometry that step stored.
    const bool geo = d->L.forces_geo != nullptr;
    const bool have_geo = geo && d->geo_valid;
    d->geo_valid = false;
    const auto in = groups(d->m, v, LULESH_F_STEP_IN);
    const auto out_nodes = groups(d->m, v, LULESH_F_POS | LULESH_F_VEL | LULESH_F_ACC | LULESH_F_FORCE);
    const auto out_kin = groups(d->m, v, LULESH_F_V | LULESH_F_KIN);
    const auto out_mat = groups(d->m, v, LULESH_F_EPQ | LULESH_F_QLQQ | LULESH_F_SS);
    for (const auto* g : {&in, &out_nodes, &out_kin, &out_mat})
        for (const Copy& c : *g)
            if (!c.host) return LULESH_EINVAL;
    if (!d->cstream) {
        CK(cudaStreamCreateWithFlags(&d->cstream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&d->mstream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&d->stream2, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&d->mstream2, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&d->nstream, cudaStreamNonBlocking));
        for (cudaEvent_t* e : {&d->ev_up, &d->ev_e, &d->ev_s2, &d->ev_join, &d->ev_s1})
            CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    const Mesh& m = d->m;
    const double dt = v->time->deltatime;
    // The cycle runs in slabs of whole element planes (the handle's matOrder
    // is slab-major), on six streams: uploads (cstream), compute (stream,
    // and stream2 for every other slab, so that the tail of one slab's
    // launch overlaps the next; nstream for the node ranges, beside the
    // force slabs) and downloads (mstream for the results of stream and
    // nstream, mstream2 for those of stream2, so that each goes down as soon
    // as it is ready).
    // The host<->device link (about 190 GB/s each way on GB300's C2C,
    // against 930 MB a cycle at s=150) paces the call as much as the GPU
    // does, so every transfer overlaps a phase:
    //   upload slab k (its elements' inputs and its nodes: its planes and the
    //     next node plane; the energy, read only by the material phase, last)
    //     -> forces of slab k;
    //   node update in ranges, one after every two force slabs (the node
    //     planes below the next slab's, whose corner forces are then all
    //     formed; later slabs' uploads, checks and forces touch only node
    //     planes above them, so the ranges run beside the force phase) and
    //     the rest after the last, each range's fields going down behind it;
    //   kinematics in slabs of two force slabs, each one's fields going down
    //     while the next runs, so that they are down before the material
    //     phase's fields are ready;
    //   material slab by slab on both compute streams, each slab's fields
    //     going down behind it; each slab lowers its own dt minima (its own
    //     block partials and counter), folded on the host at the end.
    const int s = d->nx;
    const int slabs = slab_count(s, m.numElem);
    const bool cube = slabs > 1 || (s >= 1 && int64_t(s) * s * s == int64_t(m.numElem));
    const int64_t plane_n = cube ? int64_t(s + 1) * (s + 1) : m.numNode;
    const int64_t plane_e = cube ? int64_t(s) * s : m.numElem;
    if (d->ev_slab.size() < size_t(slabs)) {
        for (auto* evs : {&d->ev_slab, &d->ev_mir, &d->ev_node, &d->ev_kin, &d->ev_mat}) {
            for (cudaEvent_t e : *evs) cudaEventDestroy(e);
            evs->assign(slabs, nullptr);
            for (cudaEvent_t& e : *evs) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
    }
    // elements [e_lo, e_hi) and the nodes of their corners [n_lo, n_hi) of each slab
    std::vector<int64_t> e_lo(slabs), e_hi(slabs), n_lo(slabs), n_hi(slabs);
    for (int sl = 0; sl < slabs; ++sl) {
        int p0 = 0, p1 = 1;
        if (cube) slab_planes(s, slabs, sl, p0, p1);
        e_lo[sl] = cube ? p0 * plane_e : 0;
        e_hi[sl] = cube ? p1 * plane_e : m.numElem;
        n_lo[sl] = cube ? p0 * plane_n : 0;
        n_hi[sl] = cube ? (p1 + 1) * plane_n : m.numNode;
    }
    CK(cudaMemsetAsync(&m.result->err, 0, 3 * sizeof(int32_t), d->stream));
    if (have_geo) CK(cudaMemsetAsync(d->upload_flag, 0, sizeof(int32_t) * slabs, d->stream));
    CK(cudaMemsetAsync(d->slab_result, 0, sizeof(StepResult) * slabs, d->stream));
    const auto t_call = std::chrono::steady_clock::now();
    d->tl_n = 0;
    if (d->tl_on) CK(cudaEventRecord(d->tl_ev[0], d->stream));
    // a stage boundary of the timeline, on the stream that did the work
    auto mark = [&](int stage, int index, cudaStream_t st) -> int {
        if (!d->tl_on || d->tl_n >= LULESH_TL_MAX) return LULESH_OK;
        CK(cudaEventRecord(d->tl_ev[1 + d->tl_n], st));
        d->tl_last.stage[d->tl_n] = stage;
        d->tl_last.index[d->tl_n] = index;
        ++d->tl_n;
        return LULESH_OK;
    };
    // the copy streams start after the previous cycle's work on the compute stream
    CK(cudaEventRecord(d->ev_up, d->stream));
    CK(cudaStreamWaitEvent(d->cstream, d->ev_up, 0));
    CK(cudaStreamWaitEvent(d->mstream, d->ev_up, 0));
    CK(cudaStreamWaitEvent(d->stream2, d->ev_up, 0));
    CK(cudaStreamWaitEvent(d->mstream2, d->ev_up, 0));

    // Element fields [e0, e1) in `out` go down once the work queued so far on
    // compute stream st is done (event ev), on st's download stream.
    // (stage and index: the timeline's marks of the work and of its download)
    auto elem_down = [&](const std::vector<Copy>& out, int64_t e0, int64_t e1, cudaEvent_t ev,
                         cudaStream_t st, int stage, int index) -> int {
        cudaStream_t down = st == d->stream2 ? d->mstream2 : d->mstream;
        CK(cudaEventRecord(ev, st));
        if (int r = mark(stage, index, st)) return r;
        CK(cudaStreamWaitEvent(down, ev, 0));
        const size_t off = size_t(e0), cnt = size_t(e1 - e0);
        for (const Copy& c : out)
            CK(cudaMemcpyAsync(static_cast<double*>(const_cast<void*>(c.host)) + off,
                               static_cast<const double*>(c.dev) + off, sizeof(double) * cnt,
                               cudaMemcpyDeviceToHost, down));
        return mark(stage + 1, index, down);
    };

    // Node update of nodes [a, b) on the node stream after both compute
    // streams' work so far, then those node fields go down. With the
    // geometry form the positions advanced are the uploaded copies.
    auto node_range = [&](int64_t a, int64_t b, cudaEvent_t ev, int r) -> int {
        CK(cudaEventRecord(d->ev_s1, d->stream));
        CK(cudaEventRecord(d->ev_s2, d->stream2));
        CK(cudaStreamWaitEvent(d->nstream, d->ev_s1, 0));
        CK(cudaStreamWaitEvent(d->nstream, d->ev_s2, 0));
        Mesh mn = m;  // nodes [a, b) as a mesh of b - a nodes at offset a
        mn.numNode = int(b - a);
        for (double** f : {&mn.x, &mn.y, &mn.z, &mn.xd, &mn.yd, &mn.zd, &mn.xdd, &mn.ydd, &mn.zdd, &mn.fx,
                           &mn.fy, &mn.fz})
            *f += a;
        mn.nodalMass += a;
        mn.invMass += a;
        mn.nodeSymm += a;
        mn.nodeElemStart += a;
        if (mn.pxp)
            for (float2** f : {&mn.pxp, &mn.pyp, &mn.pzp, &mn.vxp, &mn.vyp, &mn.vzp}) *f += a;
        d->launches += geo ? lulesh::fp64::launch_nodes_upload(mn, dt, d->stage[0] + a, d->stage[1] + a,
                                                               d->stage[2] + a, d->nstream)
                           : d->L.nodes(mn, dt, d->nstream);
        CK(cudaEventRecord(ev, d->nstream));
        if (int st = mark(LULESH_TL_NODES, r, d->nstream)) return st;
        CK(cudaStreamWaitEvent(d->mstream, ev, 0));
        for (const Copy& c : out_nodes)
            CK(cudaMemcpyAsync(static_cast<double*>(const_cast<void*>(c.host)) + a,
                               static_cast<const double*>(c.dev) + a, sizeof(double) * size_t(b - a),
                               cudaMemcpyDeviceToHost, d->mstream));
        return mark(LULESH_TL_NODES_DOWN, r, d->mstream);
    };
    int64_t node_next = 0;  // first node not yet updated
    int nranges = 0;

    const Copy* e_in = nullptr;
    int64_t node_done = 0;
    for (int sl = 0; sl < slabs; ++sl) {
        if (cube && sl > 0 && (sl & 1) == 0) {  // the node planes below slab sl's
            if (int st = node_range(node_next, n_lo[sl], d->ev_node[nranges], nranges)) return st;
            ++nranges;
            node_next = n_lo[sl];
        }
        const int64_t e0 = e_lo[sl], e1 = e_hi[sl], n1 = n_hi[sl];
        for (const Copy& c : in) {
            if (c.dev == m.e) {
                e_in = &c;
                continue;
            }
            const bool node = c.bytes == sizeof(double) * size_t(m.numNode);
            const int64_t a = node ? node_done : e0, b = node ? n1 : e1;
            double* dst = static_cast<double*>(c.dev);
            if (geo) {
                if (dst == m.x) dst = d->stage[0];
                else if (dst == m.y) dst = d->stage[1];
                else if (dst == m.z) dst = d->stage[2];
            }
            if (b > a)
                CK(cudaMemcpyAsync(dst + a, static_cast<const double*>(c.host) + a, sizeof(double) * size_t(b - a),
                                   cudaMemcpyHostToDevice, d->cstream));
        }
        CK(cudaEventRecord(d->ev_slab[sl], d->cstream));
        if (int st = mark(LULESH_TL_UPLOAD, sl, d->cstream)) return st;
        cudaStream_t cs = (sl & 1) ? d->stream2 : d->stream;
        CK(cudaStreamWaitEvent(cs, d->ev_slab[sl], 0));
        if (d->precision == LULESH_MIXED) {
            // float-pair mirrors of the slab's new nodes; its first node
            // plane's come from the previous slab's mirror launch
            d->launches += lulesh::mixed::launch_mirror_range(m, int(node_done), int(n1), cs);
            CK(cudaEventRecord(d->ev_mir[sl], cs));
            if (sl > 0) CK(cudaStreamWaitEvent(cs, d->ev_mir[sl - 1], 0));
        }
        if (geo && have_geo) {
            // the slab's nodes against the device's own: the stored geometry
            // where none changed, else the geometry of the uploaded values
            int32_t* flag = d->upload_flag + sl;
            d->launches += lulesh::fp64::launch_upload_check(m, d->stage[0], d->stage[1], d->stage[2],
                                                             int(n_lo[sl]), int(n1), flag, cs);
            d->launches += lulesh::fp64::launch_forces_geo_unless(m, int(e0), int(e1), flag, cs);
            d->launches += lulesh::fp64::launch_forces_upload(m, d->stage[0], d->stage[1], d->stage[2], int(e0),
                                                              int(e1), flag, cs);
        } else if (geo) {
            d->launches += lulesh::fp64::launch_forces_upload(m, d->stage[0], d->stage[1], d->stage[2], int(e0),
                                                              int(e1), nullptr, cs);
        } else {
            d->launches += d->L.forces_range(m, int(e0), int(e1), cs);
        }
        if (int st = mark(LULESH_TL_FORCES, sl, cs)) return st;
        node_done = n1;
    }

    if (e_in) CK(cudaMemcpyAsync(e_in->dev, e_in->host, e_in->bytes, cudaMemcpyHostToDevice, d->cstream));
    CK(cudaEventRecord(d->ev_e, d->cstream));
    if (int st = mark(LULESH_TL_ENERGY_UP, 0, d->cstream)) return st;
    if (int st = node_range(node_next, m.numNode, d->ev_node[nranges], nranges)) return st;
    // the kinematics read every node: both compute streams wait for the last range
    CK(cudaStreamWaitEvent(d->stream, d->ev_node[nranges], 0));
    CK(cudaStreamWaitEvent(d->stream2, d->ev_node[nranges], 0));
    for (int k = 0; k < slabs; k += 2) {
        const int64_t e0 = e_lo[k], e1 = e_hi[std::min(k + 1, slabs - 1)];
        cudaStream_t cs = (k & 2) ? d->stream2 : d->stream;
        d->launches += geo ? d->L.kinematics_geo_range(m, dt, int(e0), int(e1), cs)
                           : d->L.kinematics_range(m, dt, int(e0), int(e1), cs);
        if (int st = elem_down(out_kin, e0, e1, d->ev_kin[k], cs, LULESH_TL_KIN, k / 2)) return st;
    }
    // the material phase reads the kinematics of both compute streams (the
    // Q limiter reads neighbouring elements' gradients) and the energy
    CK(cudaEventRecord(d->ev_s2, d->stream2));
    CK(cudaStreamWaitEvent(d->stream, d->ev_s2, 0));
    CK(cudaEventRecord(d->ev_join, d->stream));
    CK(cudaStreamWaitEvent(d->stream2, d->ev_join, 0));
    CK(cudaStreamWaitEvent(d->stream, d->ev_e, 0));
    CK(cudaStreamWaitEvent(d->stream2, d->ev_e, 0));
    Mesh ms = m;  // the slab-major material order: positions [e_lo, e_hi) are the slab's elements
    if (slabs > 1) ms.matOrder = d->matOrderSlab;
    int part = 0;  // first block partial of the slab
    for (int sl = 0; sl < slabs; ++sl) {
        // one thread per element: blocks schedule dynamically, the slab's
        // most expensive elements first (repeat-count order within a slab)
        cudaStream_t cs = (sl & 1) ? d->stream2 : d->stream;
        ms.matGrid = std::max(1, lulesh::blocks_for(int(e_hi[sl] - e_lo[sl]), lulesh::kMatBlock));
        ms.partials = m.partials + part;
        ms.result = d->slab_result + sl;
        part += ms.matGrid;
        d->launches += d->L.material_range(ms, int(e_lo[sl]), int(e_hi[sl]), false, cs);
        if (int st = elem_down(out_mat, e_lo[sl], e_hi[sl], d->ev_mat[sl], cs, LULESH_TL_MAT, sl)) return st;
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(d->ev_s2, d->stream2));
    CK(cudaStreamWaitEvent(d->stream, d->ev_s2, 0));
    CK(cudaMemcpyAsync(d->h_result, m.result, sizeof(StepResult), cudaMemcpyDeviceToHost, d->stream));
    CK(cudaMemcpyAsync(d->h_result + 1, d->slab_result, sizeof(StepResult) * slabs, cudaMemcpyDeviceToHost,
                       d->stream));
    if (int st = mark(LULESH_TL_END, 0, d->stream)) return st;
    for (cudaStream_t st : {d->stream, d->cstream, d->mstream, d->mstream2}) CK(cudaStreamSynchronize(st));
    if (d->tl_on) {
        d->tl_last.n = d->tl_n;
        for (int k = 0; k < d->tl_n; ++k) CK(cudaEventElapsedTime(&d->tl_last.ms[k], d->tl_ev[0], d->tl_ev[1 + k]));
        d->tl_last.wall_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_call).count();
    }
    if (d->h_result->err != 0) {
        d->err_elem = d->h_result->err_elem;
        return d->h_result->err;
    }
    // the step's minima: the least of the slabs' (exact, so in any order)
    double dtc = d->h_result[1].dtcourant, dth = d->h_result[1].dthydro;
    for (int sl = 1; sl < slabs; ++sl) {
        dtc = std::min(dtc, d->h_result[1 + sl].dtcourant);
        dth = std::min(dth, d->h_result[1 + sl].dthydro);
    }
    v->time->dtcourant = dtc;
    v->time->dthydro = dth;
    d->geo_valid = geo;
    return LULESH_OK;
}

int lulesh_leapfrog_timeline(lulesh_dev* d, int32_t on) {
    if (!d) return LULESH_EINVAL;
    if (on && !d->tl_ev[0])
        for (cudaEvent_t& e : d->tl_ev) CK(cudaEventCreate(&e));
    d->tl_on = on != 0;
    return LULESH_OK;
}

int lulesh_leapfrog_timeline_read(const lulesh_dev* d, lulesh_timeline* out) {
    if (!d || !out) return LULESH_EINVAL;
    *out = d->tl_last;
    return LULESH_OK;
}

int lulesh_dev_run(lulesh_dev* d, lulesh_time_state* ts, int32_t max_cycles, int32_t* cycles_run) {
    if (!d || !ts) return LULESH_EINVAL;
    int32_t n = 0;
    int st = LULESH_OK;
    // The time loop of hpx_main (lulesh.cc:2374-2386): TimeIncrement on the
    // host, then the cycle. The loop condition of the next cycle is known
    // once this cycle's TimeIncrement has run, so when another cycle follows,
    // its force phase (which reads neither dt nor the time) is queued before
    // the host waits for this cycle's dt minima: the GPU computes it while
    // the minima come back and the next TimeIncrement runs. Same operations,
    // same order on the stream, same results.
    bool forces_queued = false;
    int set = 0;
    while (ts->time < ts->stoptime && ts->cycle < max_cycles) {
        lulesh_time_increment(ts);
        if (!forces_queued) st = queue_forces(d, set);
        if (st == LULESH_OK) st = queue_rest(d, ts->deltatime, set);
        if (st != LULESH_OK) break;
        forces_queued = ts->time < ts->stoptime && ts->cycle < max_cycles;
        if (forces_queued) st = queue_forces(d, set ^ 1);
        if (st == LULESH_OK) st = finish_cycle(d, set);
        if (st != LULESH_OK) break;  // a queued force phase just runs on scratch arrays
        ts->dtcourant = d->h_result->dtcourant;
        ts->dthydro = d->h_result->dthydro;
        set ^= 1;
        ++n;
    }
    if (cycles_run) *cycles_run = n;
    return st;
}

int lulesh_dev_run_graph(lulesh_dev* d, lulesh_time_state* ts, int32_t max_cycles,
                         int32_t sync_every, int32_t* cycles_run) {
    if (!d || !ts || sync_every < 1) return LULESH_EINVAL;
    int st = build_graph(d);
    if (st != LULESH_OK) return st;
    DevTime& h = *d->h_time;
    h = DevTime{};
    h.time = ts->time;
    h.deltatime = ts->deltatime;
    h.dtcourant = ts->dtcourant;
    h.dthydro = ts->dthydro;
    h.dtfixed = ts->dtfixed;
    h.deltatimemultlb = ts->deltatimemultlb;
    h.deltatimemultub = ts->deltatimemultub;
    h.dtmax = ts->dtmax;
    h.stoptime = ts->stoptime;
    h.cycle = ts->cycle;
    h.max_cycles = max_cycles;
    h.active = 1;
    const int32_t start = ts->cycle;
    CK(cudaMemsetAsync(d->m.result, 0, sizeof(StepResult), d->stream));
    CK(cudaMemcpyAsync(d->d_time, d->h_time, sizeof(DevTime), cudaMemcpyHostToDevice, d->stream));
    if (d->L.forces_geo) {
        if (!d->geo_valid) {
            d->launches += d->L.geometry(d->m, d->stream);
            CK(cudaGetLastError());
        }
        d->geo_valid = true;
    }
    for (;;) {
        for (int k = 0; k < sync_every; ++k) {
            CK(cudaGraphLaunch(d->graph, d->stream));
            d->launches += d->graph_kernels;
        }
        CK(cudaMemcpyAsync(d->h_time, d->d_time, sizeof(DevTime), cudaMemcpyDeviceToHost, d->stream));
        CK(cudaMemcpyAsync(d->h_result, d->m.result, sizeof(StepResult), cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
        if (!h.active) break;
    }
    ts->time = h.time;
    ts->deltatime = h.deltatime;
    ts->dtcourant = h.dtcourant;
    ts->dthydro = h.dthydro;
    ts->cycle = h.cycle;
    if (cycles_run) *cycles_run = h.cycle - start;
    if (d->h_result->err != 0) {
        d->err_elem = d->h_result->err_elem;
        return d->h_result->err;
    }
    return LULESH_OK;
}

int lulesh_dev_phase(lulesh_dev* d, int32_t phase, double dt) {
    if (!d) return LULESH_EINVAL;
    const Mesh& m = d->m;
    d->geo_valid = false;  // the single phases use the forming kernels
    CK(cudaMemsetAsync(&m.result->err, 0, 3 * sizeof(int32_t), d->stream));
    switch (phase) {
        case LULESH_PHASE_FORCES: d->launches += d->L.forces(m, d->stream); break;
        case LULESH_PHASE_NODES: d->launches += d->L.nodes(m, dt, d->stream); break;
        case LULESH_PHASE_KINEMATICS: d->launches += d->L.kinematics(m, dt, d->stream); break;
        case LULESH_PHASE_MATERIAL: d->launches += d->L.material(m, d->stream); break;
        default: return LULESH_EINVAL;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(d->h_result, m.result, sizeof(StepResult), cudaMemcpyDeviceToHost, d->stream));
    CK(cudaStreamSynchronize(d->stream));
    if (d->h_result->err != 0) {
        d->err_elem = d->h_result->err_elem;
        return d->h_result->err;
    }
    return LULESH_OK;
}

int lulesh_dev_corner_forces(lulesh_dev* d, double* fx8, double* fy8, double* fz8) {
    if (!d || !fx8 || !fy8 || !fz8) return LULESH_EINVAL;
    const Mesh& m = d->m;
    const size_t N = size_t(m.numElem), n8 = 8 * N;
    double* outs[3] = {fx8, fy8, fz8};
    if (d->precision == LULESH_MIXED) {
        std::vector<float> buf(n8);
        const float* src[3] = {m.fcx, m.fcy, m.fcz};
        for (int a = 0; a < 3; ++a) {
            CK(cudaMemcpy(buf.data(), src[a], n8 * sizeof(float), cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < N; ++i)
                for (int k = 0; k < 8; ++k) outs[a][8 * i + k] = double(buf[k * N + i]);
        }
        return LULESH_OK;
    }
    // the exact variant keeps stress and hourglass apart; the fast one stores the sum
    std::vector<double> s(n8), h(n8, 0.0);
    const double* ss[3] = {m.fsx, m.fsy, m.fsz};
    const double* hh[3] = {m.fhx, m.fhy, m.fhz};
    for (int a = 0; a < 3; ++a) {
        CK(cudaMemcpy(s.data(), ss[a], n8 * sizeof(double), cudaMemcpyDeviceToHost));
        if (hh[a]) CK(cudaMemcpy(h.data(), hh[a], n8 * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < N; ++i)
            for (int k = 0; k < 8; ++k) outs[a][8 * i + k] = s[k * N + i] + h[k * N + i];
    }
    return LULESH_OK;
}

int lulesh_dev_gradients(lulesh_dev* d, double* out6) {
    if (!d || !out6) return LULESH_EINVAL;
    const Mesh& m = d->m;
    const size_t N = size_t(m.numElem);
    if (d->precision == LULESH_MIXED) {
        std::vector<float> buf(N);
        const float* src[6] = {m.gvxi, m.gveta, m.gvzeta, m.gxxi, m.gxeta, m.gxzeta};
        for (int a = 0; a < 6; ++a) {
            CK(cudaMemcpy(buf.data(), src[a], N * sizeof(float), cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < N; ++i) out6[a * N + i] = double(buf[i]);
        }
        return LULESH_OK;
    }
    const double* src[6] = {m.dvxi, m.dveta, m.dvzeta, m.dxxi, m.dxeta, m.dxzeta};
    for (int a = 0; a < 6; ++a)
        CK(cudaMemcpy(out6 + a * N, src[a], N * sizeof(double), cudaMemcpyDeviceToHost));
    return LULESH_OK;
}

int lulesh_dev_profile_begin(lulesh_dev* d) {
    if (!d) return LULESH_EINVAL;
    if (!d->ev_begin) {
        for (auto& set : d->ev)
            for (cudaEvent_t& e : set) CK(cudaEventCreate(&e));
        CK(cudaEventCreate(&d->ev_begin));
        CK(cudaEventCreate(&d->ev_end));
    }
    for (double& k : d->kernel_ms) k = 0.0;
    d->prof_cycles = 0;
    d->prof_launch0 = d->launches;
    d->profiling = true;
    CK(cudaEventRecord(d->ev_begin, d->stream));
    return LULESH_OK;
}

int lulesh_dev_profile_end(lulesh_dev* d, lulesh_profile* out) {
    if (!d || !out || !d->profiling) return LULESH_EINVAL;
    d->profiling = false;
    CK(cudaEventRecord(d->ev_end, d->stream));
    CK(cudaEventSynchronize(d->ev_end));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, d->ev_begin, d->ev_end));
    out->total_ms = ms;
    for (int k = 0; k < 4; ++k) out->kernel_ms[k] = d->kernel_ms[k];
    out->cycles = d->prof_cycles;
    out->launches = d->launches - d->prof_launch0;
    return LULESH_OK;
}

int lulesh_set_device(int32_t device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return LULESH_ENODEV;
    if (device < 0 || device >= n) return LULESH_EINVAL;
    CK(cudaSetDevice(device));
    return LULESH_OK;
}

int32_t lulesh_dev_error_elem(const lulesh_dev* d) { return d ? d->err_elem : -1; }

int64_t lulesh_dev_launch_count(const lulesh_dev* d) { return d ? d->launches : 0; }

}  // extern "C"

namespace lulesh {

int validate_view(const lulesh_domain_view* v) { return check_view(v); }

size_t mesh_bytes(int precision, int numElem, int numNode) {
    Mesh m{};
    Arena a;
    carve_mesh(m, a, precision, numElem, numNode);
    return (a.used + 255) & ~size_t(255);
}

int mesh_init(Mesh& m, char* base, const lulesh_domain_view* v, int precision, cudaStream_t s) {
    Arena a;
    a.base = base;
    carve_mesh(m, a, precision, v->numElem, v->numNode);
    m.numElem = v->numElem;
    m.numNode = v->numNode;
    m.prm = v->params;
    return upload_mesh(m, v, precision, s, 1, nullptr);
}

int check_problem(const lulesh_problem* p) {
    if (!p) return LULESH_EINVAL;
    // s^3 elements and 8 s^3 corner indices must fit the int32 indices
    if (p->s < 1 || p->s > 640 || p->nr < 1 || p->balance < 0 || p->cost < 0 || !(p->energy_scale > 0.0))
        return LULESH_EINVAL;
    return LULESH_OK;
}

namespace {
// Material order as (first, count) element ranges with prefix offsets:
// the runs ordered by key(run) ascending, then repeat count descending
// (a stable sort, so element order within equal keys).
template <class Key>
void order_ranges(const std::vector<RegionRun>& runs, const std::vector<int>& rep, Key key,
                  std::vector<int2>& order, std::vector<int32_t>& off, std::vector<int>* idx_out = nullptr) {
    const int n = int(runs.size());
    std::vector<int> idx(n);
    for (int r = 0; r < n; ++r) idx[r] = r;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        return key(a) != key(b) ? key(a) < key(b) : rep[a] > rep[b];
    });
    order.resize(n);
    off.assign(n + 1, 0);
    for (int k = 0; k < n; ++k) {
        order[k] = make_int2(runs[idx[k]].first, runs[idx[k]].count);
        off[k + 1] = off[k] + runs[idx[k]].count;
    }
    if (idx_out) idx_out->swap(idx);
}
}  // namespace

int mesh_fill_problem(Mesh& m, const lulesh_problem* p, int precision, cudaStream_t s, lulesh_time_state* ts,
                      std::vector<int2>* classes, int slabs, int32_t* slab_order) {
    const int ne = m.numElem;
    default_params(m.prm);
    double einit = 0.0;
    initial_time_state(p->s, p->energy_scale, *ts, einit);
    if (p->stoptime > 0.0) ts->stoptime = p->stoptime;
    // region runs in element order, and the same runs ordered by repeat
    // count (largest first, element order within a count): the material
    // phase's matOrder as (first, count) ranges
    std::vector<RegionRun> runs;
    region_runs(ne, p->nr, p->balance, runs);
    std::vector<int> rep(runs.size());
    for (size_t r = 0; r < runs.size(); ++r) rep[r] = region_rep(runs[r].reg - 1, p->nr, p->cost);
    std::vector<int2> order;
    std::vector<int32_t> off;
    std::vector<int> idx;
    order_ranges(runs, rep, [](int) { return 0; }, order, off, &idx);
    if (classes) {
        classes->clear();
        for (size_t k = 0; k < idx.size(); ++k) {
            const int r = rep[idx[k]];
            if (classes->empty() || classes->back().x != r) classes->push_back(make_int2(r, 0));
            classes->back().y += runs[idx[k]].count;
        }
    }
    // the slab-major order: runs cut at the slab boundaries (whole element
    // planes), ordered by slab, then repeat count
    std::vector<int2> sorder;
    std::vector<int32_t> soff;
    const bool with_slabs = slab_order && slabs > 1;
    if (with_slabs) {
        std::vector<int64_t> bound;
        for (int sl = 1; sl < slabs; ++sl) {
            int p0, p1;
            slab_planes(p->s, slabs, sl, p0, p1);
            bound.push_back(int64_t(p0) * p->s * p->s);
        }
        std::vector<RegionRun> cut;
        std::vector<int> cut_rep, slab_of;
        for (size_t r = 0; r < runs.size(); ++r) {
            int64_t a = runs[r].first;
            const int64_t end = a + runs[r].count;
            int sl = int(std::upper_bound(bound.begin(), bound.end(), a) - bound.begin());
            while (a < end) {
                const int64_t b = sl < int(bound.size()) ? std::min(end, bound[sl]) : end;
                cut.push_back({int32_t(a), int32_t(b - a), runs[r].reg});
                cut_rep.push_back(rep[r]);
                slab_of.push_back(sl);
                a = b;
                ++sl;
            }
        }
        order_ranges(cut, cut_rep, [&](int k) { return slab_of[k]; }, sorder, soff);
    }
    // the tables in one stream-ordered temporary allocation
    const int nruns = int(runs.size()), ncut = int(sorder.size());
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t b_runs = al(sizeof(RegionRun) * nruns), b_order = al(sizeof(int2) * nruns),
                 b_off = al(sizeof(int32_t) * (nruns + 1)), b_sorder = al(sizeof(int2) * ncut),
                 b_soff = al(sizeof(int32_t) * (ncut + 1));
    char* tab = nullptr;
    CK(cudaMallocAsync(reinterpret_cast<void**>(&tab), b_runs + b_order + b_off + b_sorder + b_soff, s));
    RegionRun* d_runs = reinterpret_cast<RegionRun*>(tab);
    int2* d_order = reinterpret_cast<int2*>(tab + b_runs);
    int32_t* d_off = reinterpret_cast<int32_t*>(tab + b_runs + b_order);
    int2* d_sorder = reinterpret_cast<int2*>(tab + b_runs + b_order + b_off);
    int32_t* d_soff = reinterpret_cast<int32_t*>(tab + b_runs + b_order + b_off + b_sorder);
    int st = LULESH_OK;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (st == LULESH_OK && bytes && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
            st = LULESH_ECUDA;
    };
    up(d_runs, runs.data(), sizeof(RegionRun) * nruns);
    up(d_order, order.data(), sizeof(int2) * nruns);
    up(d_off, off.data(), sizeof(int32_t) * (nruns + 1));
    if (with_slabs) {
        up(d_sorder, sorder.data(), sizeof(int2) * ncut);
        up(d_soff, soff.data(), sizeof(int32_t) * (ncut + 1));
    }
    if (st == LULESH_OK) {
        launch_build(m, p->s, einit, d_runs, nruns, p->nr, p->cost, s);
        launch_build_order(const_cast<int32_t*>(m.matOrder), ne, d_order, d_off, nruns, s);
        if (with_slabs) launch_build_order(slab_order, ne, d_sorder, d_soff, ncut, s);
        if (precision == LULESH_MIXED) mixed::launch_mirror(m, s);
        if (cudaGetLastError() != cudaSuccess) st = LULESH_ECUDA;
    }
    cudaFreeAsync(tab, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) st = LULESH_ECUDA;
    return st;
}

int mesh_init_problem(Mesh& m, char* base, const lulesh_problem* p, int precision, cudaStream_t s,
                      lulesh_time_state* ts, std::vector<int2>* classes) {
    Arena a;
    a.base = base;
    const int ne = p->s * p->s * p->s, nn = (p->s + 1) * (p->s + 1) * (p->s + 1);
    carve_mesh(m, a, precision, ne, nn);
    m.numElem = ne;
    m.numNode = nn;
    return mesh_fill_problem(m, p, precision, s, ts, classes, 1, nullptr);
}

int copy_fields(const Mesh& m, const lulesh_domain_view* v, uint32_t mask, bool to_device, cudaStream_t s) {
    if (to_device && (mask & LULESH_F_MESH)) return LULESH_EINVAL;  // the mesh is fixed at admission
    for (const Copy& c : groups(m, v, mask)) {
        if (!c.host) return LULESH_EINVAL;
        if (to_device) CK(cudaMemcpyAsync(c.dev, c.host, c.bytes, cudaMemcpyHostToDevice, s));
        else CK(cudaMemcpyAsync(const_cast<void*>(c.host), c.dev, c.bytes, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
}

}  // namespace lulesh
