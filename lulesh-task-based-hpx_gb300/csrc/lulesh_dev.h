// Internal declarations shared by the device translation units.
//
// HBM layout (one handle, numElem = N_e, numNode = N_n):
//   node SoA      x y z xd yd zd xdd ydd zdd fx fy fz nodalMass : double[N_n]
//                 nodeSymm : uint8[N_n] (bit 0/1/2 = in symmX/Y/Z)
//   element SoA   e p q ql qq v vnew delv vdov arealg ss volo elemMass : double[N_e]
//                 nodelist : int32[8 N_e] (element-major, as Domain)
//                 lxim..lzetap, elemBC : int32[N_e]
//   CSR           nodeElemStart : int32[N_n+1], nodeElemCornerList : int32[8 N_e]
//   material      matOrder : int32[N_e]  elements grouped by EOS repeat count
//                 (largest first, ascending index within a group), elemRep : int32[N_e]
//   scratch       corner forces, corner-major (index corner*N_e + elem):
//                   double path: stress fsx fsy fsz and hourglass fhx fhy fhz
//                   mixed path : combined float fcx fcy fcz
//                 mixed path: float2 (hi, lo) mirrors of x y z xd yd zd[N_n]
//                 gradients delv_xi.. delx_zeta: double[N_e] (float[N_e] mixed)
//                 dt partial minima: one DtPartial per material block,
//                 StepResult + block counter.
// Corner-major corner forces make both the force kernel's stores and the
// node gather's loads unit-stride across a warp on the structured mesh.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "lulesh_gb300.h"

namespace lulesh {

// Boundary-condition bits of an element face (reference lulesh.h:46-74).
constexpr int XI_M = 0x00007, XI_M_SYMM = 0x00001, XI_M_FREE = 0x00002, XI_M_COMM = 0x00004;
constexpr int XI_P = 0x00038, XI_P_SYMM = 0x00008, XI_P_FREE = 0x00010, XI_P_COMM = 0x00020;
constexpr int ETA_M = 0x001c0, ETA_M_SYMM = 0x00040, ETA_M_FREE = 0x00080, ETA_M_COMM = 0x00100;
constexpr int ETA_P = 0x00e00, ETA_P_SYMM = 0x00200, ETA_P_FREE = 0x00400, ETA_P_COMM = 0x00800;
constexpr int ZETA_M = 0x07000, ZETA_M_SYMM = 0x01000, ZETA_M_FREE = 0x02000, ZETA_M_COMM = 0x04000;
constexpr int ZETA_P = 0x38000, ZETA_P_SYMM = 0x08000, ZETA_P_FREE = 0x10000, ZETA_P_COMM = 0x20000;

// Phase ids recorded with a device error.
constexpr int PHASE_FORCES = 1, PHASE_KINEMATICS = 2;

struct DtPartial {
    double dtc, dth;
};

// Written by the last material block; read by the host once per cycle.
struct StepResult {
    double dtcourant, dthydro;
    int32_t err;       // 0 or LULESH_EVOLUME (first error wins)
    int32_t err_elem;  // element that raised it
    int32_t err_phase; // PHASE_*
    uint32_t blocks_done;
};

// Device time state for the graph form (mirror of lulesh_time_state plus the
// loop limit and a done flag).
struct DevTime {
    double time, deltatime, dtcourant, dthydro, dtfixed;
    double deltatimemultlb, deltatimemultub, dtmax, stoptime;
    int32_t cycle, max_cycles;
    int32_t active;      // 1 while time < stoptime && cycle < max_cycles
    int32_t pad_;
};

// Device pointers and sizes handed to every kernel by value.
struct Mesh {
    int32_t numElem, numNode;
    // node-centred
    double *x, *y, *z, *xd, *yd, *zd, *xdd, *ydd, *zdd, *fx, *fy, *fz;
    const double* nodalMass;
    const double* invMass;  // 1 / nodalMass (fast variants multiply by it)
    const uint8_t* nodeSymm;
    // element-centred
    const int32_t* nodelist;
    const int32_t *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elemBC;
    double *e, *p, *q, *ql, *qq, *v, *vnew, *delv, *vdov, *arealg, *ss;
    const double *volo, *elemMass;
    const int32_t *nodeElemStart, *nodeElemCornerList;
    const int32_t *matOrder, *elemRep;
    // scratch, double path
    double *fsx, *fsy, *fsz, *fhx, *fhy, *fhz;
    double *dvxi, *dveta, *dvzeta, *dxxi, *dxeta, *dxzeta;
    // fast double path of a single handle: the element geometry of the
    // current coordinates, kGeoWords arrays of numElem doubles (else null)
    double* geo;
    // mixed path: float-pair mirrors (hi, lo) of positions and velocities
    float2 *pxp, *pyp, *pzp, *vxp, *vyp, *vzp;
    // scratch, mixed path
    float *fcx, *fcy, *fcz;
    float *gvxi, *gveta, *gvzeta, *gxxi, *gxeta, *gxzeta;
    // reduction scratch
    DtPartial* partials;
    StepResult* result;
    DevTime* dtime;  // non-null only in the graph form: kernels take dt from here
    int32_t matGrid; // blocks of the material kernel (= entries of partials)
    lulesh_params prm;
};

// Words of element geometry stored per element (Mesh::geo): direction sums
// (9), their cofactors (9), hourglass mode sums (12), face vectors (18).
constexpr int kGeoWords = 48;

// Launch configuration shared by host and device code.
constexpr int kForceBlock = 128;
constexpr int kNodeBlock = 256;
constexpr int kKinBlock = 128;
constexpr int kMatBlock = 128;

inline int blocks_for(int n, int b) { return (n + b - 1) / b; }

// Launchers, one set per arithmetic variant. Each returns the number of
// kernels it launched. `dt` is used unless m.dtime is set.
namespace fp64 {
int launch_forces(const Mesh& m, cudaStream_t s);
int launch_forces_range(const Mesh& m, int first, int end, cudaStream_t s);  // elements [first, end)
int launch_nodes(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics_range(const Mesh& m, double dt, int first, int end, cudaStream_t s);  // elements
int launch_material(const Mesh& m, cudaStream_t s);
// matOrder positions [first, end); accumulate: fold the dt minima into m.result's
int launch_material_range(const Mesh& m, int first, int end, bool accumulate, cudaStream_t s);
// the resident loop's form: kinematics that also stores the element geometry
// of the updated coordinates (m.geo), forces that read it, and the pass that
// forms it from the current coordinates when it is stale
int launch_forces_geo(const Mesh& m, cudaStream_t s);
int launch_kinematics_geo(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics_geo_range(const Mesh& m, double dt, int first, int end, cudaStream_t s);
int launch_geometry(const Mesh& m, cudaStream_t s);
// lulesh_leapfrog's force phase, slab by slab: the check of the slab's nodes
// [first, end) (*flag = 1 when an uploaded coordinate sx, sy, sz differs from
// m.x, m.y, m.z), then forces of its elements [first, end) from the stored
// geometry unless *flag, and forces with the geometry formed from the
// uploaded coordinates when *flag (always when flag is null)
int launch_upload_check(const Mesh& m, const double* sx, const double* sy, const double* sz, int first, int end,
                        int32_t* flag, cudaStream_t s);
int launch_forces_geo_unless(const Mesh& m, int first, int end, const int32_t* flag, cudaStream_t s);
// and its node phase: positions advanced from the uploaded copies
int launch_nodes_upload(const Mesh& m, double dt, const double* sx, const double* sy, const double* sz,
                        cudaStream_t s);
int launch_forces_upload(const Mesh& m, const double* sx, const double* sy, const double* sz, int first, int end,
                         const int32_t* flag, cudaStream_t s);
}  // namespace fp64
namespace fp64x {
int launch_forces(const Mesh& m, cudaStream_t s);
int launch_forces_range(const Mesh& m, int first, int end, cudaStream_t s);  // elements [first, end)
int launch_nodes(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics_range(const Mesh& m, double dt, int first, int end, cudaStream_t s);  // elements
int launch_material(const Mesh& m, cudaStream_t s);
// matOrder positions [first, end); accumulate: fold the dt minima into m.result's
int launch_material_range(const Mesh& m, int first, int end, bool accumulate, cudaStream_t s);
}  // namespace fp64x
namespace mixed {
int launch_forces(const Mesh& m, cudaStream_t s);
int launch_forces_range(const Mesh& m, int first, int end, cudaStream_t s);  // elements [first, end)
int launch_nodes(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics(const Mesh& m, double dt, cudaStream_t s);
int launch_kinematics_range(const Mesh& m, double dt, int first, int end, cudaStream_t s);  // elements
int launch_material(const Mesh& m, cudaStream_t s);
// matOrder positions [first, end); accumulate: fold the dt minima into m.result's
int launch_material_range(const Mesh& m, int first, int end, bool accumulate, cudaStream_t s);
int launch_mirror(const Mesh& m, cudaStream_t s);
int launch_mirror_range(const Mesh& m, int first, int end, cudaStream_t s);  // nodes [first, end)
}  // namespace mixed

// Device-side TimeIncrement for the graph form (time_increment.cu).
int launch_time_increment(DevTime* t, StepResult* r, cudaStream_t s);
int launch_time_finish(DevTime* t, StepResult* r, cudaStream_t s);

// --- batched form -------------------------------------------------------------
// Many independent problems ("instances"), each with its own Mesh in a slot
// of a device pool. A phase is one persistent launch whose blocks pull
// (instance, tile) work items from a queue; each tile is a contiguous range
// of one instance's elements (or nodes, or positions in its matOrder).
struct BatchTile {
    int32_t inst;   // slot
    int32_t first;  // first element / node / matOrder position
    int32_t count;  // number of units
    int32_t cost;   // units x EOS passes (material tiles), for ordering
};

enum { TILES_ELEM = 0, TILES_NODE = 1, TILES_MAT = 2 };

struct BatchCtl {
    const Mesh* meshes;   // [slots]; dtime -> times[slot], result -> results[slot]
    DevTime* times;       // [slots]; max_cycles < 0 marks an empty slot
    StepResult* results;  // [slots]; dt minima as atomically lowered doubles
    const BatchTile* tiles[3];
    const int32_t* ntiles;  // [3], in device memory so tables change without re-capture
    unsigned* queue;        // [4] per-phase tile counters, cleared each cycle
    int32_t slots;
};

struct BatchLaunch {
    int32_t block;  // threads per block
    int32_t grid;   // persistent blocks
    int32_t grab;   // tiles taken per queue access
};

constexpr int kBatchMaxBlock = 256;

// Launch one batched phase; and the resident blocks per SM of a phase's
// kernel at a block size (occupancy).
namespace fp64 {
int launch_batch_phase(int phase, const BatchCtl& c, const BatchLaunch& l, cudaStream_t s);
int batch_occupancy(int phase, int block);
}
namespace fp64x {
int launch_batch_phase(int phase, const BatchCtl& c, const BatchLaunch& l, cudaStream_t s);
int batch_occupancy(int phase, int block);
}
namespace mixed {
int launch_batch_phase(int phase, const BatchCtl& c, const BatchLaunch& l, cudaStream_t s);
int batch_occupancy(int phase, int block);
}

// Per-slot TimeIncrement + dt reset, and the dt hand-off (time_increment.cu).
int launch_batch_time_increment(const BatchCtl& c, cudaStream_t s);
int launch_batch_time_finish(const BatchCtl& c, cudaStream_t s);

// Final report on the device (verify.cu): out[0..3] = e(0), MaxAbsDiff,
// TotalAbsDiff, MaxRelDiff of an nx^3 energy field; one block.
int launch_verify(const double* e, int nx, double* out, cudaStream_t s);

// --- problem set-up shared by the host Domain and the device build ---------------

// EOS repeat count of a 0-based region (lulesh.cc:2156-2170).
__host__ __device__ inline int region_rep(int reg, int numReg, int cost) {
    if (reg < numReg / 2) return 1;
    if (reg < (numReg - (numReg + 15) / 20)) return 1 + cost;
    return 10 * (1 + cost);
}

// A run of consecutive elements of one region; reg is 1-based.
struct RegionRun {
    int32_t first, count, reg;
};

// The reference's region assignment (CreateRegionIndexSets,
// lulesh-init.cc:341-445) as runs in element order: srand(0) and the
// reference's sequence of rand() draws (domain.cpp).
void region_runs(int numElem, int numReg, int balance, std::vector<RegionRun>& runs);
// Physics constants of Domain::Domain (lulesh-init.cc:18-41).
void default_params(lulesh_params& P);
// Initial time state of an s^3 Sedov problem and its origin energy
// (lulesh-init.cc:133-183); energy_scale multiplies the deposit.
void initial_time_state(int s, double energy_scale, lulesh_time_state& ts, double& einit);

// Device build of the initial state of problem s (device_init.cu): every
// array of a carved mesh from the analytic cube but matOrder, the region
// runs (element order, device memory) expanded into elemRep.
int launch_build(const Mesh& m, int s, double einit, const RegionRun* runs, int nruns, int numReg, int cost,
                 cudaStream_t st);
// Expands (first, count) element ranges with prefix offsets `off` (n + 1
// entries, device memory) into an element order out[numElem].
int launch_build_order(int32_t* out, int numElem, const int2* ranges, const int32_t* off, int n, cudaStream_t st);

// Handle-independent instance set-up shared by the single-problem handle and
// the batch pool (capi.cu).
size_t mesh_bytes(int precision, int numElem, int numNode);
int validate_view(const lulesh_domain_view* v);
// Carves the mesh arrays out of base (mesh_bytes long), uploads topology and
// the full state of v on stream s and waits for the copies; leaves
// partials/result/dtime/matGrid to the caller.
int mesh_init(Mesh& m, char* base, const lulesh_domain_view* v, int precision, cudaStream_t s);
// Checks a problem description (sizes that fit the int32 indices).
int check_problem(const lulesh_problem* p);
// Builds problem p on the device into an already carved mesh with numElem
// and numNode set (the build kernels, then a wait); fills *ts and, when
// given, *classes as mesh_init_problem does. With slab_order and slabs > 1
// it also writes the material order split into that many slabs of whole
// element planes (repeat-count order within a slab) to slab_order[N_e],
// for a material phase run slab by slab.
int mesh_fill_problem(Mesh& m, const lulesh_problem* p, int precision, cudaStream_t s, lulesh_time_state* ts,
                      std::vector<int2>* classes, int slabs, int32_t* slab_order);
// The same for problem p built on the device (no host Domain): fills *ts
// with the problem's initial time state and *classes with (repeat count,
// elements) pairs, largest repeat count first; waits for the build.
int mesh_init_problem(Mesh& m, char* base, const lulesh_problem* p, int precision, cudaStream_t s,
                      lulesh_time_state* ts, std::vector<int2>* classes);
// Copies the LULESH_F_* field groups of mask between m and v (either way)
// on stream s and waits.
int copy_fields(const Mesh& m, const lulesh_domain_view* v, uint32_t mask, bool to_device, cudaStream_t s);

}  // namespace lulesh
