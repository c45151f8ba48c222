// Double-precision kernels of the Lagrange-leapfrog step.
//
// This header is compiled twice:
//   fp64_fast.cu   LULESH_VARIANT=fp64,  LULESH_EXACT=0, FMA contraction on
//   fp64_exact.cu  LULESH_VARIANT=fp64x, LULESH_EXACT=1, nvcc --fmad=false
// With the reference's operand order kept in step_math.cuh, the exact
// variant rounds every operation as the reference does and matches the CPU
// oracle bit for bit (the oracle then uses the same portable cube root); the
// fast variant lets nvcc fuse multiply-adds, which moves results by a few
// ulps and saves FP64-pipe instructions.
//
// One cycle = four phases, each a per-element (or per-node) device function
// used both by the single-problem kernels below and by the batched
// persistent kernels of batch_kernels.cuh:
//   forces_elem      stress + FB hourglass corner forces   (lulesh.cc:787-1113)
//   nodes_node       CSR gather, a = f/m, symmetry BC, v, x (lulesh.cc:838-862, 1115-1158, 566-588)
//   kinematics_elem  volume, arealg, vdov, v <- vnew, Q gradients (lulesh.cc:1169-1418)
//   material_elem    Q limiter, EOS x rep, sound speed, save, dt constraints
//                    (lulesh.cc:1420-1974)
#pragma once

#include "step_math.cuh"

namespace lulesh {
namespace LULESH_VARIANT {

__device__ __forceinline__ double cube_root(double x) {
#if LULESH_EXACT
    return cbrt_portable(x);
#else
    return cbrt(x);
#endif
}

#if LULESH_EXACT
// Stress and hourglass corner forces of element i, stored separately
// (corner-major) so that the node gather adds them in the reference's order
// (lulesh.cc:849-856).
__device__ __forceinline__ void forces_elem(const Mesh& m, int i) {
    const size_t N = (size_t)m.numElem;
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    double x[8], y[8], z[8];
    gather8(m.x, nl, x);
    gather8(m.y, nl, y);
    gather8(m.z, nl, z);

    // stress (InitIntegrateStressForElemsTask, lulesh.cc:787-836)
    {
        const double sig = -LD(m.p + i) - LD(m.q + i);
        if (jacobian_singular(x, y, z)) raise_error(m.result, i, PHASE_FORCES);
        double nx[8], ny[8], nz[8];
        node_normals(nx, ny, nz, x, y, z);          // 16 x the normals
        const double sigs = sig * kInvNormalScale;  // a power of two: exact
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            m.fsx[k * N + i] = -(sigs * nx[k]);
            m.fsy[k * N + i] = -(sigs * ny[k]);
            m.fsz[k * N + i] = -(sigs * nz[k]);
        }
    }

    // hourglass (CalcHourglassForElemsTask, lulesh.cc:864-1113)
    const double determ = LD(m.volo + i) * LD(m.v + i);
    if (determ <= 0.0) {
        raise_error(m.result, i, PHASE_FORCES);
        return;
    }
    double hg[8][4];
    {
        double dvdx[8], dvdy[8], dvdz[8];
        volume_derivs(dvdx, dvdy, dvdz, x, y, z);
        hourgam_all(hg, x, y, z, dvdx, dvdy, dvdz, rcp(determ));
    }
    const double coefficient =
        -m.prm.hgcoef * 0.01 * LD(m.ss + i) * LD(m.elemMass + i) / cube_root(determ);
    double vel[8], f[8];
    double* outs[3] = {m.fhx, m.fhy, m.fhz};
    const double* vels[3] = {m.xd, m.yd, m.zd};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        gather8(vels[a], nl, vel);
        fb_force_axis(hg, vel, coefficient, f);
#pragma unroll
        for (int k = 0; k < 8; ++k) outs[a][k * N + i] = f[k];
    }
}
#else
// Element geometry (fast variant): everything the force phase derives from
// the corner coordinates alone. J holds the body-diagonal sums (8 x the
// centre Jacobian, columns along xi, eta, zeta) and h the hourglass mode sums
// of each coordinate, both from one Walsh-Hadamard transform; c the cofactors
// of J; fa the six faces' t x s, unscaled. The kinematics phase forms the
// same geometry of the updated coordinates for its own needs (J and c for
// the Q gradients and vdov, fa for the characteristic length) and, in the
// resident loop, stores it for the next cycle's force phase, whose
// coordinates those are. Every path forms it with the same operations, so
// stored and recomputed geometry are the same bits.
struct ElemGeo {
    double J[3][3], c[3][3], h[3][4], fa[6][3];
};
#define LULESH_GEO_FORM 1

__device__ __forceinline__ void elem_geometry(const double x[8], const double y[8], const double z[8],
                                              ElemGeo& g) {
    walsh7(x, g.J[0], g.h[0]);
    walsh7(y, g.J[1], g.h[1]);
    walsh7(z, g.J[2], g.h[2]);
    cofactors(g.J, g.c);
    face_txs<0, 1, 2, 3>(x, y, z, g.fa[0]);
    face_txs<0, 4, 5, 1>(x, y, z, g.fa[1]);
    face_txs<1, 5, 6, 2>(x, y, z, g.fa[2]);
    face_txs<2, 6, 7, 3>(x, y, z, g.fa[3]);
    face_txs<3, 7, 4, 0>(x, y, z, g.fa[4]);
    face_txs<4, 7, 6, 5>(x, y, z, g.fa[5]);
}

// Mesh::geo word q of element i is geo[q * numElem + i]: J, c, h, fa in
// row-major order.
__device__ __forceinline__ void geo_store(const Mesh& m, int i, const ElemGeo& g) {
    const size_t N = (size_t)m.numElem;
    double* o = m.geo + i;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            o[(3 * a + d) * N] = g.J[a][d];
            o[(9 + 3 * a + d) * N] = g.c[a][d];
        }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 4; ++k) o[(18 + 4 * a + k) * N] = g.h[a][k];
#pragma unroll
    for (int f = 0; f < 6; ++f)
#pragma unroll
        for (int d = 0; d < 3; ++d) o[(30 + 3 * f + d) * N] = g.fa[f][d];
}
__device__ __forceinline__ void geo_load(const Mesh& m, int i, ElemGeo& g) {
    const size_t N = (size_t)m.numElem;
    const double* o = m.geo + i;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            g.J[a][d] = LD(o + (3 * a + d) * N);
            g.c[a][d] = LD(o + (9 + 3 * a + d) * N);
        }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 4; ++k) g.h[a][k] = LD(o + (18 + 4 * a + k) * N);
#pragma unroll
    for (int f = 0; f < 6; ++f)
#pragma unroll
        for (int d = 0; d < 3; ++d) g.fa[f][d] = LD(o + (30 + 3 * f + d) * N);
}

// Stress plus hourglass corner force of element i from its geometry, summed
// in registers and stored once (corner-major fsx, fsy, fsz). The zero test
// on the centre Jacobian's determinant (lulesh.cc:817-821) is taken in
// another summation order: zero for the same collapsed elements, though a
// near-singular element may round differently. The hourglass vectors come
// from the volume gradient (192 x dV/dx_k) and the mode sums scaled by
// volinv / 192. The stress force (p + q) n enters through the face vectors
// scaled by (p + q) / 8 and starts each corner's hourglass multiply-add
// chain. Elements that fail a test store nothing: the step reports the
// error and its state is not used.
__device__ __forceinline__ void forces_from_geo(const Mesh& m, int i, const int nl[8], const ElemGeo& g) {
    const size_t N = (size_t)m.numElem;
    if (f_is_zero(g.J[0][0] * g.c[0][0] + g.J[1][0] * g.c[1][0] + g.J[2][0] * g.c[2][0]))
        raise_error(m.result, i, PHASE_FORCES);
    const double determ = LD(m.volo + i) * LD(m.v + i);
    if (f_le(determ, 0.0)) {
        raise_error(m.result, i, PHASE_FORCES);
        return;
    }
    double hg[8][4];
    {
        double gx[8], gy[8], gz[8], hx[4], hy[4], hz[4];
        volume_gradient(g.J, g.c, g.h[0], g.h[1], g.h[2], gx, gy, gz);
        const double sc = rcp(determ) * (1.0 / 192.0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            hx[k] = pmul(g.h[0][k], sc);
            hy[k] = pmul(g.h[1][k], sc);
            hz[k] = pmul(g.h[2][k], sc);
        }
        hourgam_mode_h<0>(hg, hx[0], hy[0], hz[0], gx, gy, gz);
        hourgam_mode_h<1>(hg, hx[1], hy[1], hz[1], gx, gy, gz);
        hourgam_mode_h<2>(hg, hx[2], hy[2], hz[2], gx, gy, gz);
        hourgam_mode_h<3>(hg, hx[3], hy[3], hz[3], gx, gy, gz);
    }
    double fa[6][3];
    const double scale = (LD(m.p + i) + LD(m.q + i)) * kInvNormalScale;
#pragma unroll
    for (int f = 0; f < 6; ++f)
#pragma unroll
        for (int d = 0; d < 3; ++d) fa[f][d] = pmul(g.fa[f][d], scale);
    const double coefficient = -m.prm.hgcoef * 0.01 * LD(m.ss + i) * LD(m.elemMass + i) * rcbrt_pos(determ);
    double* outs[3] = {m.fsx, m.fsy, m.fsz};
    const double* vels[3] = {m.xd, m.yd, m.zd};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double st[8], vel[8], f[8];
        corner_sums(fa, a, st);
        gather8(vels[a], nl, vel);
        fb_force_axis_plus(hg, vel, coefficient, st, f);
#pragma unroll
        for (int k = 0; k < 8; ++k) outs[a][k * N + i] = f[k];
    }
}

// Forces of element i from its coordinates (geometry formed here).
__device__ __forceinline__ void forces_elem(const Mesh& m, int i) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    ElemGeo g;
    {
        double x[8], y[8], z[8];
        gather8(m.x, nl, x);
        gather8(m.y, nl, y);
        gather8(m.z, nl, z);
        elem_geometry(x, y, z, g);
    }
    forces_from_geo(m, i, nl, g);
}

// Forces of element i from the stored geometry.
__device__ __forceinline__ void forces_geo_elem(const Mesh& m, int i) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    ElemGeo g;
    geo_load(m, i, g);
    forces_from_geo(m, i, nl, g);
}

// Forces of element i in lulesh_leapfrog with the geometry formed from the
// coordinates just uploaded from the host (sx, sy, sz), the step's own.
__device__ __forceinline__ void forces_upload_elem(const Mesh& m, const double* __restrict__ sx,
                                                   const double* __restrict__ sy,
                                                   const double* __restrict__ sz, int i) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    ElemGeo g;
    {
        double x[8], y[8], z[8];
        gather8(sx, nl, x);
        gather8(sy, nl, y);
        gather8(sz, nl, z);
        elem_geometry(x, y, z, g);
    }
    forces_from_geo(m, i, nl, g);
}

// Stores the geometry of element i's current coordinates.
__device__ __forceinline__ void geometry_elem(const Mesh& m, int i) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    double x[8], y[8], z[8];
    gather8(m.x, nl, x);
    gather8(m.y, nl, y);
    gather8(m.z, nl, z);
    ElemGeo g;
    elem_geometry(x, y, z, g);
    geo_store(m, i, g);
}
#endif

// Node n: gather in CSR order, stress then hourglass per corner
// (combineVolumeForcesTaskFunc, lulesh.cc:838-862), then the node update
// (of positions px, py, pz when given, see node_update).
__device__ __forceinline__ void nodes_node(const Mesh& m, int n, double dt, const double* px = nullptr,
                                           const double* py = nullptr, const double* pz = nullptr) {
    const size_t N = (size_t)m.numElem;
    const int b = LD(m.nodeElemStart + n), e = LD(m.nodeElemStart + n + 1);
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int j = b; j < e; ++j) {
        const int c = LD(m.nodeElemCornerList + j);
        const size_t idx = (size_t)(c & 7) * N + (size_t)(c >> 3);
#if LULESH_EXACT
        fx += LD(m.fsx + idx);
        fx += LD(m.fhx + idx);
        fy += LD(m.fsy + idx);
        fy += LD(m.fhy + idx);
        fz += LD(m.fsz + idx);
        fz += LD(m.fhz + idx);
#else
        fx += LD(m.fsx + idx);  // stress + hourglass, combined by forces_elem
        fy += LD(m.fsy + idx);
        fz += LD(m.fsz + idx);
#endif
    }
    node_update(m, n, fx, fy, fz, dt, px, py, pz);
}

// CalcKinematicsForElemsTask (lulesh.cc:1169-1275) and
// CalcMonotonicQGradientsForElemsTask (lulesh.cc:1277-1418) of element i:
// both read the same updated node positions and velocities.
#if LULESH_EXACT
__device__ __forceinline__ void kinematics_elem(const Mesh& m, int i, double dt) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    double x[8], y[8], z[8], xv[8], yv[8], zv[8];
    gather8(m.x, nl, x);
    gather8(m.y, nl, y);
    gather8(m.z, nl, z);
    const double volume = hex_volume(x, y, z);
    const double relv = quot_refined(volume, LD(m.volo + i));
    const double vold = m.v[i];
    m.vnew[i] = relv;
    m.delv[i] = relv - vold;
    m.arealg[i] = char_length(x, y, z, volume);

    gather8(m.xd, nl, xv);
    gather8(m.yd, nl, yv);
    gather8(m.zd, nl, zv);
    double g[6];
    m.vdov[i] = gradients_vdov(x, y, z, xv, yv, zv, LD(m.volo + i) * relv, 0.5 * dt, g);
    m.dvxi[i] = g[0];
    m.dveta[i] = g[1];
    m.dvzeta[i] = g[2];
    m.dxxi[i] = g[3];
    m.dxeta[i] = g[4];
    m.dxzeta[i] = g[5];
    update_volume(m, i, vold, relv);
}
#else
// Characteristic length 4 V / sqrt(largest face measure) from the faces'
// t x s: the reference's face measure is 4 |t x s|^2 (Lagrange's identity),
// so the length is 2 V / sqrt(max |t x s|^2).
__device__ __forceinline__ double char_length_faces(const double fa[6][3], double volume) {
    double cl = fma(fa[0][2], fa[0][2], fma(fa[0][1], fa[0][1], pmul(fa[0][0], fa[0][0])));
#pragma unroll
    for (int f = 1; f < 6; ++f)
        cl = nonneg_max(cl, fma(fa[f][2], fa[f][2], fma(fa[f][1], fa[f][1], pmul(fa[f][0], fa[f][0]))));
    return div_sqrt(2.0 * volume, cl);
}

// Kinematics of element i; STORE_GEO: also store the element geometry of the
// updated coordinates for the next force phase (Mesh::geo).
template <bool STORE_GEO>
__device__ __forceinline__ void kinematics_fast(const Mesh& m, int i, double dt) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    double relv, vold;
    ElemGeo g;
    {
        double x[8], y[8], z[8];
        gather8(m.x, nl, x);
        gather8(m.y, nl, y);
        gather8(m.z, nl, z);
        const double volume = hex_volume(x, y, z);
        relv = quot_refined(volume, LD(m.volo + i));
        vold = m.v[i];
        m.vnew[i] = relv;
        m.delv[i] = relv - vold;
        elem_geometry(x, y, z, g);
        m.arealg[i] = char_length_faces(g.fa, volume);
    }
    if (STORE_GEO) geo_store(m, i, g);
    double xv[8], yv[8], zv[8];
    gather8(m.xd, nl, xv);
    gather8(m.yd, nl, yv);
    gather8(m.zd, nl, zv);
    double gr[6];
    m.vdov[i] = gradients_vdov_xc(g.J, g.c, xv, yv, zv, pmul(LD(m.volo + i), relv), 0.5 * dt, gr);
    m.dvxi[i] = gr[0];
    m.dveta[i] = gr[1];
    m.dvzeta[i] = gr[2];
    m.dxxi[i] = gr[3];
    m.dxeta[i] = gr[4];
    m.dxzeta[i] = gr[5];
    update_volume(m, i, vold, relv);
}
__device__ __forceinline__ void kinematics_elem(const Mesh& m, int i, double dt) { kinematics_fast<false>(m, i, dt); }
#endif

// Material phase of the element at position t of the repeat-count order
// (matOrder): Q limiter and q terms, rep EOS passes, sound speed and save;
// folds its Courant and hydro constraints into dtc, dth.
__device__ __forceinline__ void material_elem(const Mesh& m, int t, double& dtc, double& dth) {
    const int i = LD(m.matOrder + t);
    const double vnew = LD(m.vnew + i), vdov = LD(m.vdov + i);
    double ql, qq;
    q_terms<double>(m, i, m.dvxi, m.dveta, m.dvzeta, m.dxxi, m.dxeta, m.dxzeta, vnew, vdov, ql, qq);
    m.qq[i] = qq;
    m.ql[i] = ql;
    double vnewc = vnew;
    if (!f_is_zero(m.prm.eosvmin) && f_lt(vnewc, m.prm.eosvmin)) vnewc = m.prm.eosvmin;
    if (!f_is_zero(m.prm.eosvmax) && f_gt(vnewc, m.prm.eosvmax)) vnewc = m.prm.eosvmax;
    const double ss = eos_element(m, i, vnewc, LD(m.elemRep + i));
    dt_constraints(m.prm, ss, vdov, LD(m.arealg + i), dtc, dth);
}

// --- single-problem kernels -------------------------------------------------

// all elements, or (RANGED) elements [first, end)
template <bool RANGED>
__global__ void __launch_bounds__(kForceBlock) k_forces(Mesh m, int first, int end) {
    if (m.dtime && !m.dtime->active) return;
    const int i = (RANGED ? first : 0) + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (RANGED ? end : m.numElem)) forces_elem(m, i);
}

__global__ void __launch_bounds__(kNodeBlock) k_nodes(Mesh m, double dt) {
    if (m.dtime) {
        if (!m.dtime->active) return;
        dt = m.dtime->deltatime;
    }
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < m.numNode) nodes_node(m, n, dt);
}

// all elements, or (RANGED) elements [first, end)
template <bool RANGED>
__global__ void __launch_bounds__(kKinBlock) k_kinematics(Mesh m, double dt, int first, int end) {
    if (m.dtime) {
        if (!m.dtime->active) return;
        dt = m.dtime->deltatime;
    }
    const int i = (RANGED ? first : 0) + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (RANGED ? end : m.numElem)) kinematics_elem(m, i, dt);
}

#if !LULESH_EXACT
// The resident loop's form: forces from the stored geometry, kinematics that
// store it, and the pass that forms it from the current coordinates.
__global__ void __launch_bounds__(kForceBlock) k_forces_geo(Mesh m) {
    if (m.dtime && !m.dtime->active) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m.numElem) forces_geo_elem(m, i);
}
// At least 3 blocks of 128 per SM (at most 168 registers): with the
// integer-pipe products the compiler's own choice, 240 registers and 2
// blocks, left the FP64 pipe waiting (2.09 -> 2.00 ms at s=150).
template <bool RANGED>
__global__ void __launch_bounds__(kKinBlock, 3) k_kinematics_geo(Mesh m, double dt, int first, int end) {
    if (m.dtime) {
        if (!m.dtime->active) return;
        dt = m.dtime->deltatime;
    }
    const int i = (RANGED ? first : 0) + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (RANGED ? end : m.numElem)) kinematics_fast<true>(m, i, dt);
}

// lulesh_leapfrog's check of one slab: *flag = 1 when the host's uploaded
// coordinates (sx, sy, sz) of a node in [first, end) differ, bit for bit,
// from the device's own (the previous step's results). Every thread of a
// warp reaches the vote; the flag starts at 0 (cleared by the host call).
__global__ void __launch_bounds__(kNodeBlock) k_upload_check(Mesh m, const double* sx, const double* sy,
                                                              const double* sz, int first, int end, int* flag) {
    const int n = first + blockIdx.x * blockDim.x + threadIdx.x;
    bool differs = false;
    if (n < end)
        differs = dbits(LD(sx + n)) != dbits(LD(m.x + n)) || dbits(LD(sy + n)) != dbits(LD(m.y + n)) ||
                  dbits(LD(sz + n)) != dbits(LD(m.z + n));
    if (__any_sync(0xffffffffu, differs) && (threadIdx.x & 31) == 0) *flag = 1;
}
// lulesh_leapfrog's node phase: every node, the positions advanced being the
// uploaded copies sx, sy, sz (the step's own coordinates).
__global__ void __launch_bounds__(kNodeBlock) k_nodes_upload(Mesh m, double dt, const double* sx,
                                                              const double* sy, const double* sz) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < m.numNode) nodes_node(m, n, dt, sx, sy, sz);
}
// Forces of elements [first, end) from the stored geometry, unless the
// slab's check found a changed node (*flag).
__global__ void __launch_bounds__(kForceBlock) k_forces_geo_unless(Mesh m, int first, int end,
                                                                    const int* flag) {
    if (*flag) return;
    const int i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < end) forces_geo_elem(m, i);
}
// Forces of elements [first, end) with the geometry formed from the uploaded
// coordinates: always (flag null) or when the slab's check found a changed
// node (*flag). The two kernels give the same bits for an unchanged element
// (the stored geometry is formed by the same function from the same values).
__global__ void __launch_bounds__(kForceBlock) k_forces_upload(Mesh m, const double* sx, const double* sy,
                                                                const double* sz, int first, int end,
                                                                const int* flag) {
    if (flag && !*flag) return;
    const int i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < end) forces_upload_elem(m, sx, sy, sz, i);
}
__global__ void __launch_bounds__(kForceBlock) k_geometry(Mesh m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m.numElem) geometry_elem(m, i);
}
#endif

// Elements visited in repeat-count order so a warp's lanes run the same
// number of EOS passes; the dt minima end in a last-block reduction.
// 8 blocks of 128 per SM (64 registers): the EOS passes are a chain of
// dependent integer-pipe products and FP64 operations, latency-bound at 6
// blocks per SM (1.34 -> 1.02 ms at s=150 with 8).
__global__ void __launch_bounds__(kMatBlock, 8) k_material(Mesh m, int first, int end, int accumulate) {
    if (m.dtime && !m.dtime->active) return;
    double dtc = 1.0e+20, dth = 1.0e+20;  // lulesh.cc:2214-2215
    for (int t = first + blockIdx.x * blockDim.x + threadIdx.x; t < end; t += gridDim.x * blockDim.x)
        material_elem(m, t, dtc, dth);
    finish_dt_reduction(m, dtc, dth, accumulate != 0);
}

int launch_forces(const Mesh& m, cudaStream_t s) {
    k_forces<false><<<blocks_for(m.numElem, kForceBlock), kForceBlock, 0, s>>>(m, 0, m.numElem);
    return 1;
}
int launch_forces_range(const Mesh& m, int first, int end, cudaStream_t s) {
    if (end <= first) return 0;
    k_forces<true><<<blocks_for(end - first, kForceBlock), kForceBlock, 0, s>>>(m, first, end);
    return 1;
}
int launch_nodes(const Mesh& m, double dt, cudaStream_t s) {
    k_nodes<<<blocks_for(m.numNode, kNodeBlock), kNodeBlock, 0, s>>>(m, dt);
    return 1;
}
int launch_kinematics(const Mesh& m, double dt, cudaStream_t s) {
    k_kinematics<false><<<blocks_for(m.numElem, kKinBlock), kKinBlock, 0, s>>>(m, dt, 0, m.numElem);
    return 1;
}
int launch_kinematics_range(const Mesh& m, double dt, int first, int end, cudaStream_t s) {
    if (end <= first) return 0;
    k_kinematics<true><<<blocks_for(end - first, kKinBlock), kKinBlock, 0, s>>>(m, dt, first, end);
    return 1;
}
int launch_material(const Mesh& m, cudaStream_t s) {
    k_material<<<m.matGrid, kMatBlock, 0, s>>>(m, 0, m.numElem, 0);
    return 1;
}
int launch_material_range(const Mesh& m, int first, int end, bool accumulate, cudaStream_t s) {
    k_material<<<m.matGrid, kMatBlock, 0, s>>>(m, first, end, accumulate ? 1 : 0);
    return 1;
}
#if !LULESH_EXACT
int launch_forces_geo(const Mesh& m, cudaStream_t s) {
    k_forces_geo<<<blocks_for(m.numElem, kForceBlock), kForceBlock, 0, s>>>(m);
    return 1;
}
int launch_kinematics_geo(const Mesh& m, double dt, cudaStream_t s) {
    k_kinematics_geo<false><<<blocks_for(m.numElem, kKinBlock), kKinBlock, 0, s>>>(m, dt, 0, m.numElem);
    return 1;
}
int launch_kinematics_geo_range(const Mesh& m, double dt, int first, int end, cudaStream_t s) {
    if (end <= first) return 0;
    k_kinematics_geo<true><<<blocks_for(end - first, kKinBlock), kKinBlock, 0, s>>>(m, dt, first, end);
    return 1;
}
int launch_nodes_upload(const Mesh& m, double dt, const double* sx, const double* sy, const double* sz,
                        cudaStream_t s) {
    k_nodes_upload<<<blocks_for(m.numNode, kNodeBlock), kNodeBlock, 0, s>>>(m, dt, sx, sy, sz);
    return 1;
}
int launch_upload_check(const Mesh& m, const double* sx, const double* sy, const double* sz, int first, int end,
                        int32_t* flag, cudaStream_t s) {
    if (end <= first) return 0;
    k_upload_check<<<blocks_for(end - first, kNodeBlock), kNodeBlock, 0, s>>>(m, sx, sy, sz, first, end, flag);
    return 1;
}
int launch_forces_geo_unless(const Mesh& m, int first, int end, const int32_t* flag, cudaStream_t s) {
    if (end <= first) return 0;
    k_forces_geo_unless<<<blocks_for(end - first, kForceBlock), kForceBlock, 0, s>>>(m, first, end, flag);
    return 1;
}
int launch_forces_upload(const Mesh& m, const double* sx, const double* sy, const double* sz, int first, int end,
                         const int32_t* flag, cudaStream_t s) {
    if (end <= first) return 0;
    k_forces_upload<<<blocks_for(end - first, kForceBlock), kForceBlock, 0, s>>>(m, sx, sy, sz, first, end, flag);
    return 1;
}
int launch_geometry(const Mesh& m, cudaStream_t s) {
    k_geometry<<<blocks_for(m.numElem, kForceBlock), kForceBlock, 0, s>>>(m);
    return 1;
}
#endif

}  // namespace LULESH_VARIANT
}  // namespace lulesh

#include "batch_kernels.cuh"
