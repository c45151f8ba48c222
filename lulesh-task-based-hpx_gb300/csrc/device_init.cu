// Initial state of a Sedov problem built on the device (Domain::Domain,
// lulesh-init.cc:10-183; BuildMesh 202-250, SetupThreadSupportStructures
// 254-310, SetupSymmetryPlanes 449-470, SetupElementConnectivities 473-511,
// SetupBoundaryConditions 514-606 for one domain).
//
// The cube is analytic: node coordinates, the element node lists, the
// node -> corner CSR, the face neighbours, the boundary masks and the
// symmetry bits follow from the (column, row, plane) index of each node or
// element. The element volumes use the reference's CalcElemVolume with the
// same corner coordinates, and each node adds vol / 8 over its elements in
// ascending element order, as the reference's element loop does; built with
// --fmad=false, every value has the bits of the host build. Region sets come
// from the reference's rand() sequence, so the host draws them as runs and
// the last kernel expands the runs into the per-element repeat counts and
// the repeat-count order of the material phase.
#define LULESH_VARIANT setup
#define LULESH_EXACT 1
#include "step_math.cuh"

namespace lulesh {
namespace {

constexpr int kBuildBlock = 256;

// Coordinate of grid line c (BuildMesh, lulesh-init.cc:213-233).
__device__ __forceinline__ double grid(int c, int s) { return 1.125 * double(c) / double(s); }

// Elements adjacent to grid line c along one axis: c - 1 and c, where they exist.
__device__ __forceinline__ int adj(int c, int s) { return int(c > 0) + int(c < s); }
// Sum of adj over the lines before c (c <= s): 1 + 2 (c - 1).
__device__ __forceinline__ int adj_before(int c) { return c == 0 ? 0 : 2 * c - 1; }

// Corner index of node (dx, dy, dz) relative to its element's first node
// (the element node list order, lulesh-init.cc:236-244).
__device__ __forceinline__ int corner_of(int dx, int dy, int dz) {
    return 4 * dz + (dy ? (dx ? 2 : 3) : (dx ? 1 : 0));
}

__global__ void __launch_bounds__(kBuildBlock) k_build_nodes(Mesh m, int s) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= m.numNode) return;
    const int en = s + 1;
    const int col = n % en, row = (n / en) % en, pl = n / (en * en);
    m.x[n] = grid(col, s);
    m.y[n] = grid(row, s);
    m.z[n] = grid(pl, s);
    m.xd[n] = m.yd[n] = m.zd[n] = 0.0;
    m.xdd[n] = m.ydd[n] = m.zdd[n] = 0.0;
    m.fx[n] = m.fy[n] = m.fz[n] = 0.0;
    // symmetry planes x = 0, y = 0, z = 0 (SetupSymmetryPlanes)
    const_cast<uint8_t*>(m.nodeSymm)[n] = uint8_t(int(col == 0) | int(row == 0) << 1 | int(pl == 0) << 2);
    // CSR start: the element counts of every node before n in (plane, row,
    // column) order, a separable sum
    const int T = 2 * s;
    const int start = adj_before(pl) * T * T + adj(pl, s) * (adj_before(row) * T + adj(row, s) * adj_before(col));
    int32_t* nes = const_cast<int32_t*>(m.nodeElemStart);
    nes[n] = start;
    if (n == m.numNode - 1) nes[n + 1] = 8 * m.numElem;
    // this node's corners, elements in ascending order
    int32_t* list = const_cast<int32_t*>(m.nodeElemCornerList);
    int j = start;
    for (int pe = pl - 1; pe <= pl; ++pe) {
        if (pe < 0 || pe >= s) continue;
        for (int re = row - 1; re <= row; ++re) {
            if (re < 0 || re >= s) continue;
            for (int ce = col - 1; ce <= col; ++ce) {
                if (ce < 0 || ce >= s) continue;
                const int el = (pe * s + re) * s + ce;
                list[j++] = 8 * el + corner_of(col - ce, row - re, pl - pe);
            }
        }
    }
}

__global__ void __launch_bounds__(kBuildBlock) k_build_elems(Mesh m, int s, double einit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int ne = m.numElem;
    if (i >= ne) return;
    const int en = s + 1, s2 = s * s;
    const int ce = i % s, re = (i / s) % s, pe = i / s2;
    const int base = (pe * en + re) * en + ce;
    const int dc[8] = {0, 1, 1, 0, 0, 1, 1, 0}, dr[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    int32_t* nl = const_cast<int32_t*>(m.nodelist) + 8 * size_t(i);
    double x[8], y[8], z[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int dz = k >> 2;
        nl[k] = base + dz * en * en + dr[k] * en + dc[k];
        x[k] = grid(ce + dc[k], s);
        y[k] = grid(re + dr[k], s);
        z[k] = grid(pe + dz, s);
    }
    const double vol = setup::hex_volume(x, y, z);
    const_cast<double*>(m.volo)[i] = vol;
    const_cast<double*>(m.elemMass)[i] = vol;
    m.v[i] = 1.0;
    m.e[i] = (i == 0) ? einit : 0.0;
    m.p[i] = m.q[i] = m.ql[i] = m.qq[i] = 0.0;
    m.vnew[i] = m.delv[i] = m.vdov[i] = m.arealg[i] = m.ss[i] = 0.0;
    // face neighbours (SetupElementConnectivities): neighbours in the flat
    // index, clamped at the ends of the whole range
    const_cast<int32_t*>(m.lxim)[i] = (i == 0) ? 0 : i - 1;
    const_cast<int32_t*>(m.lxip)[i] = (i == ne - 1) ? ne - 1 : i + 1;
    const_cast<int32_t*>(m.letam)[i] = (i < s) ? i : i - s;
    const_cast<int32_t*>(m.letap)[i] = (i >= ne - s) ? i : i + s;
    const_cast<int32_t*>(m.lzetam)[i] = (i < s2) ? i : i - s2;
    const_cast<int32_t*>(m.lzetap)[i] = (i >= ne - s2) ? i : i + s2;
    // one domain: symmetry on the minus faces, free surface on the plus faces
    int bc = 0;
    if (pe == 0) bc |= ZETA_M_SYMM;
    if (pe == s - 1) bc |= ZETA_P_FREE;
    if (re == 0) bc |= ETA_M_SYMM;
    if (re == s - 1) bc |= ETA_P_FREE;
    if (ce == 0) bc |= XI_M_SYMM;
    if (ce == s - 1) bc |= XI_P_FREE;
    const_cast<int32_t*>(m.elemBC)[i] = bc;
}

// Nodal masses: vol / 8 of each adjacent element, added in ascending
// element order starting from 0 (the reference's element loop, per node).
__global__ void __launch_bounds__(kBuildBlock) k_build_mass(Mesh m, int s) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= m.numNode) return;
    const int en = s + 1;
    const int col = n % en, row = (n / en) % en, pl = n / (en * en);
    double mass = 0.0;
    for (int pe = pl - 1; pe <= pl; ++pe) {
        if (pe < 0 || pe >= s) continue;
        for (int re = row - 1; re <= row; ++re) {
            if (re < 0 || re >= s) continue;
            for (int ce = col - 1; ce <= col; ++ce) {
                if (ce < 0 || ce >= s) continue;
                mass += m.volo[(pe * s + re) * s + ce] / 8.0;
            }
        }
    }
    const_cast<double*>(m.nodalMass)[n] = mass;
    const_cast<double*>(m.invMass)[n] = 1.0 / mass;
}

// elemRep from the region runs (element order), by binary search.
__global__ void __launch_bounds__(kBuildBlock) k_build_rep(Mesh m, const RegionRun* __restrict__ runs, int nruns,
                                                          int numReg, int cost) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.numElem) return;
    int lo = 0, hi = nruns - 1;  // last run with first <= i
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (runs[mid].first <= i) lo = mid;
        else hi = mid - 1;
    }
    const_cast<int32_t*>(m.elemRep)[i] = region_rep(runs[lo].reg - 1, numReg, cost);
}

// An element order from (first, count) ranges with prefix offsets, by
// binary search over the offsets.
__global__ void __launch_bounds__(kBuildBlock) k_build_order(int32_t* __restrict__ out, int numElem,
                                                            const int2* __restrict__ ranges,
                                                            const int32_t* __restrict__ off, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= numElem) return;
    int lo = 0, hi = n - 1;  // last range with offset <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    out[t] = ranges[lo].x + (t - off[lo]);
}

}  // namespace

int launch_build(const Mesh& m, int s, double einit, const RegionRun* runs, int nruns, int numReg, int cost,
                 cudaStream_t st) {
    k_build_nodes<<<blocks_for(m.numNode, kBuildBlock), kBuildBlock, 0, st>>>(m, s);
    k_build_elems<<<blocks_for(m.numElem, kBuildBlock), kBuildBlock, 0, st>>>(m, s, einit);
    k_build_mass<<<blocks_for(m.numNode, kBuildBlock), kBuildBlock, 0, st>>>(m, s);
    k_build_rep<<<blocks_for(m.numElem, kBuildBlock), kBuildBlock, 0, st>>>(m, runs, nruns, numReg, cost);
    return 4;
}

int launch_build_order(int32_t* out, int numElem, const int2* ranges, const int32_t* off, int n, cudaStream_t st) {
    k_build_order<<<blocks_for(numElem, kBuildBlock), kBuildBlock, 0, st>>>(out, numElem, ranges, off, n);
    return 1;
}

}  // namespace lulesh
