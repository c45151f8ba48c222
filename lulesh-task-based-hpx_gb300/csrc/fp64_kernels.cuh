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
// Fast variant: stress plus hourglass corner force of element i summed in
// registers and stored once (corner-major fsx, fsy, fsz). The stress force
// (p + q) n enters through the six face vectors scaled by (p + q) / 8, each
// corner's stress is the start of its hourglass multiply-add chain.
// Elements that fail the determinant test store nothing: the step reports
// the error and its state is not used.
__device__ __forceinline__ void forces_elem(const Mesh& m, int i) {
    const size_t N = (size_t)m.numElem;
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    double x[8], y[8], z[8];
    gather8(m.x, nl, x);
    gather8(m.y, nl, y);
    gather8(m.z, nl, z);
    // 8 x the centre Jacobian and its cofactors; the zero test on its
    // determinant (lulesh.cc:817-821) in another summation order: zero for
    // the same collapsed elements, though a near-singular element may round
    // differently
    double J[3][3], c[3][3], hx[4], hy[4], hz[4];
    walsh7(x, J[0], hx);
    walsh7(y, J[1], hy);
    walsh7(z, J[2], hz);
    cofactors(J, c);
    if (f_is_zero(J[0][0] * c[0][0] + J[1][0] * c[1][0] + J[2][0] * c[2][0]))
        raise_error(m.result, i, PHASE_FORCES);
    const double determ = LD(m.volo + i) * LD(m.v + i);
    if (f_le(determ, 0.0)) {
        raise_error(m.result, i, PHASE_FORCES);
        return;
    }
    double hg[8][4];
    {
        // hourglass vectors from the volume gradient (192 x dV/dx_k) and the
        // mode sums scaled by volinv / 192
        double gx[8], gy[8], gz[8];
        volume_gradient(J, c, hx, hy, hz, gx, gy, gz);
        const double sc = rcp(determ) * (1.0 / 192.0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            hx[k] *= sc;
            hy[k] *= sc;
            hz[k] *= sc;
        }
        hourgam_mode_h<0>(hg, hx[0], hy[0], hz[0], gx, gy, gz);
        hourgam_mode_h<1>(hg, hx[1], hy[1], hz[1], gx, gy, gz);
        hourgam_mode_h<2>(hg, hx[2], hy[2], hz[2], gx, gy, gz);
        hourgam_mode_h<3>(hg, hx[3], hy[3], hz[3], gx, gy, gz);
    }
    double fa[6][3];
    face_vectors(x, y, z, (LD(m.p + i) + LD(m.q + i)) * kInvNormalScale, fa);
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
#endif

// Node n: gather in CSR order, stress then hourglass per corner
// (combineVolumeForcesTaskFunc, lulesh.cc:838-862), then the node update.
__device__ __forceinline__ void nodes_node(const Mesh& m, int n, double dt) {
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
    node_update(m, n, fx, fy, fz, dt);
}

// CalcKinematicsForElemsTask (lulesh.cc:1169-1275) and
// CalcMonotonicQGradientsForElemsTask (lulesh.cc:1277-1418) of element i:
// both read the same updated node positions and velocities.
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

__global__ void __launch_bounds__(kKinBlock) k_kinematics(Mesh m, double dt) {
    if (m.dtime) {
        if (!m.dtime->active) return;
        dt = m.dtime->deltatime;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m.numElem) kinematics_elem(m, i, dt);
}

// Elements visited in repeat-count order so a warp's lanes run the same
// number of EOS passes; the dt minima end in a last-block reduction.
__global__ void __launch_bounds__(kMatBlock) k_material(Mesh m, int first, int end, int accumulate) {
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
    k_kinematics<<<blocks_for(m.numElem, kKinBlock), kKinBlock, 0, s>>>(m, dt);
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

}  // namespace LULESH_VARIANT
}  // namespace lulesh

#include "batch_kernels.cuh"
