// Mixed-precision kernels of the Lagrange-leapfrog step (LULESH_MIXED).
//
// State stays double: positions, velocities, e, p, q, v and its cutoffs, the
// element volume, the EOS with its repeat loop, the sound speed and the dt
// minima. The element force, kinematic and Q-gradient temporaries run in
// float, which on GB300 issues at 60x the FP64 rate.
//
// Float inputs without cancellation. Every element function works on node
// coordinates and velocities relative to the element's corner 0: the stress
// and hourglass forces, face areas, Q gradients and velocity gradient are
// all invariant under a common shift of the corners (the hourglass vectors'
// corner sums vanish), and relative values keep float's 24 bits for the
// element-scale differences instead of spending them on the absolute
// position. To form those differences with float arithmetic only, the node
// update also stores each position and velocity component as a float pair
// (hi = fl(x), lo = fl(x - hi)); (hi_k - hi_0) + (lo_k - lo_0) is then within
// about one float ulp of x_k - x_0.
//
// Node forces are gathered from float corner forces with a Neumaier
// compensated sum and then promoted to double for the node update.
#define LULESH_VARIANT mixed
#define LULESH_EXACT 0
#define LULESH_FLOAT_Q 1
#include "step_math.cuh"
#include "float_pair.cuh"

namespace lulesh {
namespace mixed {

// Corner values relative to corner 0 from float-pair node data.
__device__ __forceinline__ void rel8(const float2* __restrict__ p, const int nl[8], float r[8]) {
    float2 a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = __ldg(p + nl[k]);
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = (a[k].x - a[0].x) + (a[k].y - a[0].y);
}

__device__ __forceinline__ void mirror_node(const Mesh& m, int n) {
    m.pxp[n] = split(m.x[n]);
    m.pyp[n] = split(m.y[n]);
    m.pzp[n] = split(m.z[n]);
    m.vxp[n] = split(m.xd[n]);
    m.vyp[n] = split(m.yd[n]);
    m.vzp[n] = split(m.zd[n]);
}

// Stress + hourglass corner forces of element i in float, stored combined
// (corner-major).
__device__ __forceinline__ void forces_elem(const Mesh& m, int i) {
    const size_t N = (size_t)m.numElem;
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    float x[8], y[8], z[8];
    rel8(m.pxp, nl, x);
    rel8(m.pyp, nl, y);
    rel8(m.pzp, nl, z);

    float fx[8], fy[8], fz[8];
    {
        // node_normals returns 8 x the normals: fold the 1/8 into the stress
        const float sig = float(-LD(m.p + i) - LD(m.q + i)) * float(kInvNormalScale);
        if (jacobian_singular(x, y, z)) raise_error(m.result, i, PHASE_FORCES);
        float nx[8], ny[8], nz[8];
        node_normals(nx, ny, nz, x, y, z);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            fx[k] = -(sig * nx[k]);
            fy[k] = -(sig * ny[k]);
            fz[k] = -(sig * nz[k]);
        }
    }
    const double determ = LD(m.volo + i) * LD(m.v + i);
    if (determ <= 0.0) {
        raise_error(m.result, i, PHASE_FORCES);
        return;
    }
    const float detf = float(determ);
    float hg[8][4];
    {
        float dvdx[8], dvdy[8], dvdz[8];
        volume_derivs(dvdx, dvdy, dvdz, x, y, z);
        hourgam_all(hg, x, y, z, dvdx, dvdy, dvdz, 1.0f / detf);
    }
    const float coefficient = -float(m.prm.hgcoef) * 0.01f * float(LD(m.ss + i)) *
                              float(LD(m.elemMass + i)) / cbrtf(detf);
    float vel[8], f[8];
    rel8(m.vxp, nl, vel);
    fb_force_axis(hg, vel, coefficient, f);
#pragma unroll
    for (int k = 0; k < 8; ++k) m.fcx[k * N + i] = fx[k] + f[k];
    rel8(m.vyp, nl, vel);
    fb_force_axis(hg, vel, coefficient, f);
#pragma unroll
    for (int k = 0; k < 8; ++k) m.fcy[k * N + i] = fy[k] + f[k];
    rel8(m.vzp, nl, vel);
    fb_force_axis(hg, vel, coefficient, f);
#pragma unroll
    for (int k = 0; k < 8; ++k) m.fcz[k * N + i] = fz[k] + f[k];
}

// Neumaier's compensated summation: s + c carries the sum of the terms with
// an error independent of their count for the short sums here.
struct Neumaier {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float t = s + v;
        if (fabsf(s) >= fabsf(v)) c += (s - t) + v;
        else c += (v - t) + s;
        s = t;
    }
    __device__ __forceinline__ double value() const { return widen(s) + widen(c); }
};

__device__ __forceinline__ void nodes_node(const Mesh& m, int n, double dt) {
    const size_t N = (size_t)m.numElem;
    const int b = LD(m.nodeElemStart + n), e = LD(m.nodeElemStart + n + 1);
    Neumaier sx, sy, sz;
    for (int j = b; j < e; ++j) {
        const int c = LD(m.nodeElemCornerList + j);
        const size_t idx = (size_t)(c & 7) * N + (size_t)(c >> 3);
        sx.add(LD(m.fcx + idx));
        sy.add(LD(m.fcy + idx));
        sz.add(LD(m.fcz + idx));
    }
    node_update(m, n, sx.value(), sy.value(), sz.value(), dt);
    mirror_node(m, n);
}

__device__ __forceinline__ void kinematics_elem(const Mesh& m, int i, double dt) {
    int nl[8];
    load_nodelist(m.nodelist, i, nl);
    double volume;
    {
        double xd8[8], yd8[8], zd8[8];
        gather8(m.x, nl, xd8);
        gather8(m.y, nl, yd8);
        gather8(m.z, nl, zd8);
        volume = hex_volume(xd8, yd8, zd8);  // double: relative volume and delv need it
    }
    const double relv = quot_refined(volume, LD(m.volo + i));
    const double vold = m.v[i];
    m.vnew[i] = relv;
    m.delv[i] = relv - vold;

    float x[8], y[8], z[8], xv[8], yv[8], zv[8];
    rel8(m.pxp, nl, x);
    rel8(m.pyp, nl, y);
    rel8(m.pzp, nl, z);
    m.arealg[i] = widen(char_length(x, y, z, narrow(volume)));
    rel8(m.vxp, nl, xv);
    rel8(m.vyp, nl, yv);
    rel8(m.vzp, nl, zv);
    float g[6];
    m.vdov[i] = widen(gradients_vdov(x, y, z, xv, yv, zv, narrow(LD(m.volo + i) * relv), narrow(0.5 * dt), g));
    m.gvxi[i] = g[0];
    m.gveta[i] = g[1];
    m.gvzeta[i] = g[2];
    m.gxxi[i] = g[3];
    m.gxeta[i] = g[4];
    m.gxzeta[i] = g[5];
    update_volume(m, i, vold, relv);
}

__device__ __forceinline__ void material_elem(const Mesh& m, int t, double& dtc, double& dth) {
    const int i = LD(m.matOrder + t);
    const double vnew = LD(m.vnew + i), vdov = LD(m.vdov + i);
    double ql, qq;
    q_terms<float>(m, i, m.gvxi, m.gveta, m.gvzeta, m.gxxi, m.gxeta, m.gxzeta, vnew, vdov, ql, qq);
    m.qq[i] = qq;
    m.ql[i] = ql;
    double vnewc = vnew;
    if (!f_is_zero(m.prm.eosvmin) && f_lt(vnewc, m.prm.eosvmin)) vnewc = m.prm.eosvmin;
    if (!f_is_zero(m.prm.eosvmax) && f_gt(vnewc, m.prm.eosvmax)) vnewc = m.prm.eosvmax;
    const double ss = eos_element(m, i, vnewc, LD(m.elemRep + i));
    dt_constraints(m.prm, ss, vdov, LD(m.arealg + i), dtc, dth);
}

// --- single-problem kernels -------------------------------------------------

// Refreshes the float-pair mirrors from the double state (after the host
// uploads positions or velocities).
__global__ void __launch_bounds__(kNodeBlock) k_mirror(Mesh m, int first, int end) {
    const int n = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (n < end) mirror_node(m, n);
}

// all elements, or (RANGED) elements [first, end). At least 5 blocks of 128
// per SM (at most 96 registers, a few spilled to L1): the corner gathers
// need the warps (s=150: 0.204 -> 0.195 ms against 4 blocks at 128).
template <bool RANGED>
__global__ void __launch_bounds__(kForceBlock, 5) k_forces(Mesh m, int first, int end) {
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

__global__ void __launch_bounds__(kMatBlock) k_material(Mesh m, int first, int end, int accumulate) {
    if (m.dtime && !m.dtime->active) return;
    double dtc = 1.0e+20, dth = 1.0e+20;
    for (int t = first + blockIdx.x * blockDim.x + threadIdx.x; t < end; t += gridDim.x * blockDim.x)
        material_elem(m, t, dtc, dth);
    finish_dt_reduction(m, dtc, dth, accumulate != 0);
}

int launch_mirror(const Mesh& m, cudaStream_t s) {
    k_mirror<<<blocks_for(m.numNode, kNodeBlock), kNodeBlock, 0, s>>>(m, 0, m.numNode);
    return 1;
}
int launch_mirror_range(const Mesh& m, int first, int end, cudaStream_t s) {
    if (end <= first) return 0;
    k_mirror<<<blocks_for(end - first, kNodeBlock), kNodeBlock, 0, s>>>(m, first, end);
    return 1;
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

}  // namespace mixed
}  // namespace lulesh

#include "batch_kernels.cuh"
