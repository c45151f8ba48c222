/* lulesh_gb300.h - C ABI of the GB300-native LULESH Lagrange-leapfrog step.
 *
 * Drop-in for the hot path of esa-tu-darmstadt/lulesh-task-based-hpx: the
 * per-cycle LagrangeLeapFrogWithTasks(Domain&) (reference lulesh.cc:1977-2240)
 * and the host TimeIncrement (lulesh.cc:182-229) that precedes it in the time
 * loop of hpx_main (lulesh.cc:2374-2386).
 *
 * Conventions
 *  - Plain C types and pointers only. Every entry point returns a status:
 *    LULESH_OK or a negative code; LULESH_EVOLUME is the reference's
 *    VolumeError (lulesh.h:30), the condition on which the reference calls
 *    exit(VolumeError) (lulesh.cc:821, 908, 1262).
 *  - A lulesh_dev handle owns one CUDA stream (lulesh_leapfrog creates five
 *    more on its first call) and device copies of every Domain array the
 *    step touches. Use a handle from one host thread at a
 *    time. Host arrays stay owned by the caller.
 *  - All arithmetic of LULESH_FP64 and LULESH_FP64_EXACT is IEEE double, as
 *    the reference (Real_t = double, lulesh.h:27). LULESH_MIXED runs the
 *    element force, kinematic and Q-gradient temporaries in float and keeps
 *    positions, velocities, e, p, q, v and the dt minima in double.
 */
#ifndef LULESH_GB300_H
#define LULESH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define LULESH_OK 0
#define LULESH_EVOLUME (-1)   /* VolumeError, lulesh.h:30 */
#define LULESH_EQSTOP (-2)    /* QStopError, lulesh.h:30 (never raised: the reference never checks qstop) */
#define LULESH_EINVAL (-10)   /* bad argument or size */
#define LULESH_ECUDA (-11)    /* CUDA runtime error */
#define LULESH_ENOMEM (-12)   /* device or host allocation failed */
#define LULESH_ENODEV (-13)   /* no CUDA device */
#define LULESH_ETIMEOUT (-14) /* a bounded device-side wait gave up */

/* Arithmetic of a device handle. */
#define LULESH_FP64 0       /* double, FMA contraction allowed (the fast double path) */
#define LULESH_FP64_EXACT 1 /* double, every operation separately rounded as the reference
                               source is written; reproduces the CPU oracle bit for bit when
                               the oracle uses the same cube root (lulesh_cbrt_portable) */
#define LULESH_MIXED 2      /* float element temporaries, double state (see above) */

/* Physics constants of Domain (lulesh.h:538-560, values lulesh-init.cc:18-36). */
typedef struct lulesh_params {
    double e_cut, p_cut, q_cut, v_cut, u_cut;
    double hgcoef, ss4o3, qstop, monoq_max_slope, monoq_limiter_mult;
    double qlc_monoq, qqc_monoq, qqc;
    double eosvmax, eosvmin, pmin, emin, dvovmax, refdens;
} lulesh_params;

/* Time-control state of Domain (lulesh.h:563-572). */
typedef struct lulesh_time_state {
    double time, deltatime, dtcourant, dthydro, dtfixed;
    double deltatimemultlb, deltatimemultub, dtmax, stoptime;
    int32_t cycle;
    int32_t pad_;
} lulesh_time_state;

/* A view of a host Domain (lulesh.h:130-606): raw pointers to its SoA arrays,
 * as the Domain accessors *_begin(), nodelist(0), nodeElemCornerList(0) and
 * regNumList() return them (lulesh.h:281-392). Index arrays are int32
 * (Index_t, lulesh.h:26), reals double (Real_t, lulesh.h:27). */
typedef struct lulesh_domain_view {
    int32_t numElem, numNode;
    int32_t sizeX;     /* elements along one cube edge (Domain::sizeX) */
    int32_t numReg;    /* regions (Domain::numReg) */
    int32_t cost;      /* extra cost of expensive regions (Domain::cost) */
    int32_t numSymmX, numSymmY, numSymmZ; /* sizes of the symmetry node sets (0 = empty) */
    /* node-centred, numNode each */
    double *x, *y, *z, *xd, *yd, *zd, *xdd, *ydd, *zdd, *fx, *fy, *fz;
    const double* nodalMass;
    const int32_t *symmX, *symmY, *symmZ;
    /* element-centred, numElem each unless noted */
    const int32_t* nodelist; /* 8 * numElem, corners 0..7 of each element */
    const int32_t *lxim, *lxip, *letam, *letap, *lzetam, *lzetap;
    const int32_t* elemBC;
    double *e, *p, *q, *ql, *qq, *v, *vnew, *delv, *vdov, *arealg, *ss;
    const double *volo, *elemMass;
    const int32_t* nodeElemStart;      /* numNode + 1 */
    const int32_t* nodeElemCornerList; /* nodeElemStart[numNode] entries of 8*elem+corner */
    const int32_t* regNumList;         /* region number 1..numReg of each element */
    lulesh_params params;
    lulesh_time_state* time; /* may be NULL except for lulesh_leapfrog */
} lulesh_domain_view;

/* One Sedov problem of the reference's command line (--s --r --b --c), for the
 * device build and the batch. */
typedef struct lulesh_problem {
    int32_t s, nr, balance, cost; /* --s --r --b --c */
    double energy_scale;          /* deposited energy multiplier (1.0 = the reference) */
    double stoptime;              /* <= 0: the reference's 1e-2 */
    int32_t max_cycles;           /* <= 0: no cycle limit (the reference's --i default) */
    int32_t pad_;
} lulesh_problem;

/* Field groups for lulesh_dev_upload / lulesh_dev_download. */
#define LULESH_F_POS 0x001u   /* x y z */
#define LULESH_F_VEL 0x002u   /* xd yd zd */
#define LULESH_F_ACC 0x004u   /* xdd ydd zdd */
#define LULESH_F_FORCE 0x008u /* fx fy fz */
#define LULESH_F_EPQ 0x010u   /* e p q */
#define LULESH_F_V 0x020u     /* v */
#define LULESH_F_QLQQ 0x040u  /* ql qq */
#define LULESH_F_KIN 0x080u   /* vnew delv vdov arealg */
#define LULESH_F_SS 0x100u    /* ss */
/* What one step reads from the mutable state, and everything it writes. */
#define LULESH_F_STEP_IN (LULESH_F_POS | LULESH_F_VEL | LULESH_F_EPQ | LULESH_F_V | LULESH_F_SS)
#define LULESH_F_STEP_OUT                                                                \
    (LULESH_F_POS | LULESH_F_VEL | LULESH_F_ACC | LULESH_F_FORCE | LULESH_F_EPQ |          \
     LULESH_F_V | LULESH_F_QLQQ | LULESH_F_KIN | LULESH_F_SS)
#define LULESH_F_ALL 0x1ffu
/* The constant mesh, download only: nodalMass volo elemMass nodelist
 * lxim..lzetap elemBC nodeElemStart nodeElemCornerList (the upload calls
 * refuse it with LULESH_EINVAL: the mesh is fixed when a handle or slot is
 * created). */
#define LULESH_F_MESH 0x200u

typedef struct lulesh_dev lulesh_dev;
typedef struct lulesh_domain lulesh_domain;

/* ---------------- host Domain (replaces Domain::Domain, lulesh-init.cc:10-183) ------- */

/* Builds the Sedov problem of Domain::Domain for an s^3 mesh with nr regions,
 * load balance `balance` and region cost `cost` (the reference's --s --r --b
 * --c, lulesh.cc:2421-2432), including the srand(0)/rand() region sets
 * (lulesh-init.cc:341-445). energy_scale multiplies the deposited energy
 * (1.0 = the reference); the initial dt follows lulesh-init.cc:181. */
int lulesh_domain_create(int32_t s, int32_t nr, int32_t balance, int32_t cost, double energy_scale,
                         lulesh_domain** out);
/* The view stays valid until lulesh_domain_destroy. */
lulesh_domain_view* lulesh_domain_get_view(lulesh_domain* d);
void lulesh_domain_destroy(lulesh_domain* d);

/* TimeIncrement (lulesh.cc:182-229) on a host time state. */
int lulesh_time_increment(lulesh_time_state* ts);

/* Plane-0 energy symmetry of VerifyAndWriteFinalOutput (lulesh-util.cc:77-103):
 * out[0] MaxAbsDiff, out[1] TotalAbsDiff, out[2] MaxRelDiff. */
int lulesh_symmetry(const lulesh_domain_view* v, double out[3]);

/* Final report of a run (VerifyAndWriteFinalOutput, lulesh-util.cc:60-115)
 * as computed on the device by lulesh_dev_verify / lulesh_batch_verify:
 * e(0) and the plane-0 symmetry diffs, bit for bit what lulesh_symmetry
 * gives on the downloaded energy field. */
typedef struct lulesh_verify_result {
    double e0;                      /* final origin energy */
    double maxabs, totabs, maxrel;  /* MaxAbsDiff, TotalAbsDiff, MaxRelDiff */
    int32_t cycle, nx;              /* cycles run, problem edge s */
} lulesh_verify_result;

/* ---------------- device handle ------------------------------------------------------ */

/* Allocates device mirrors of the Domain arrays the step touches and uploads
 * all of them (constant topology and the full mutable state). Replaces the
 * reference's per-cycle malloc/free of temporaries (lulesh.cc:2017-2022,
 * lulesh.h:203-214): scratch is allocated once here. A LULESH_FP64 handle
 * also keeps each element's geometry between the kinematics and the next
 * force phase (48 doubles per element) and copies of the node coordinates
 * for lulesh_leapfrog: lulesh_batch_footprint(LULESH_FP64, s) plus
 * 24 (s + 1)^3 bytes in all. */
int lulesh_dev_create(const lulesh_domain_view* host, int32_t precision, lulesh_dev** out);
void lulesh_dev_destroy(lulesh_dev* dev);

/* Builds problem `p` (as Domain::Domain, lulesh-init.cc:10-183) directly in
 * device memory: no host Domain and no upload. Every array equals the host
 * build's bit for bit; the region sets are drawn on the host (the reference's
 * rand() sequence) and expanded on the device. *ts receives the initial time
 * state (with p->stoptime when > 0); pass it to lulesh_dev_run. Download
 * fields into the view of a host Domain of the same problem when needed. */
int lulesh_dev_create_problem(const lulesh_problem* p, int32_t precision, lulesh_time_state* ts,
                              lulesh_dev** out);

/* Copies field groups host -> device / device -> host (LULESH_F_* masks). */
int lulesh_dev_upload(lulesh_dev* dev, const lulesh_domain_view* host, uint32_t mask);
int lulesh_dev_download(lulesh_dev* dev, lulesh_domain_view* host, uint32_t mask);

/* The final report of the device-resident state (e(0), plane-0 symmetry)
 * without downloading any field; `cycle` is the caller's count of cycles run
 * (copied into the result, as the reference prints it). Blocks until done.
 * LULESH_EINVAL unless the mesh is a cube of edge nx (numElem = nx^3). */
int lulesh_dev_verify(lulesh_dev* dev, int32_t cycle, lulesh_verify_result* out);

/* One LagrangeLeapFrog cycle (lulesh.cc:1977-2240) on the device-resident
 * state with time step `deltatime`; returns the new Courant and hydro
 * constraints (Domain::dtcourant/dthydro, lulesh.cc:2229-2236). Blocks until
 * the cycle is done. LULESH_EVOLUME where the reference exits with VolumeError. */
int lulesh_dev_step(lulesh_dev* dev, double deltatime, double* dtcourant, double* dthydro);

/* The literal drop-in for LagrangeLeapFrogWithTasks(Domain&): uploads the
 * state a step reads from the host Domain view, runs one cycle with
 * view->time->deltatime, downloads every field the step writes and stores
 * dtcourant/dthydro into view->time. The cycle runs in slabs of element
 * planes and the copies overlap it: each slab's inputs upload ahead of its
 * force kernel, node fields go back behind the node update of each pair of
 * slabs, element fields behind each kinematics and material slab. With
 * LULESH_FP64, slabs whose node coordinates all equal those the previous
 * call left on the device reuse the element geometry it stored; the others
 * form it from the uploaded coordinates (same results either way). The
 * host arrays must stay untouched until the call returns; pin them
 * (lulesh_domain_pin) for full link bandwidth. On LULESH_EVOLUME (where the
 * reference exits) the host fields hold the partly advanced state and
 * view->time's dt constraints are unchanged. */
int lulesh_leapfrog(lulesh_dev* dev, lulesh_domain_view* host);

/* The time loop of hpx_main (lulesh.cc:2374-2386) on device-resident state:
 * while (time < stoptime && cycle < max_cycles) { TimeIncrement; step }.
 * TimeIncrement runs on the host between cycles; while it waits for a
 * cycle's dt minima, the next cycle's force phase (which reads neither dt
 * nor the time) is already queued when another cycle follows. *cycles_run
 * counts the cycles this call ran. On LULESH_EVOLUME that queued force phase
 * may still run on the handle's stream after the call returns; it writes
 * only scratch arrays, and later calls on the handle wait for it. */
int lulesh_dev_run(lulesh_dev* dev, lulesh_time_state* ts, int32_t max_cycles, int32_t* cycles_run);

/* The same time loop with TimeIncrement on the device and each cycle's
 * kernels replayed from one CUDA graph; the host reads the state back only
 * every `sync_every` cycles (>= 1). Results equal lulesh_dev_run's. */
int lulesh_dev_run_graph(lulesh_dev* dev, lulesh_time_state* ts, int32_t max_cycles,
                         int32_t sync_every, int32_t* cycles_run);

/* ---------------- batched ensembles ---------------------------------------------------
 * No counterpart in the reference, which runs one problem per process. A
 * batch keeps many independent Sedov problems resident in one device pool;
 * each cycle of every active problem runs in one CUDA graph: a device-side
 * TimeIncrement per problem, then the four phases as persistent launches
 * over an (instance, tile) work queue, then the dt hand-off. Each problem
 * keeps its own dt, stoptime and cycle limit; problems join (admit) and
 * leave (retire) between graph replays without re-capturing the graph. */
typedef struct lulesh_batch lulesh_batch;

typedef struct lulesh_slot_status {
    int32_t in_use, active, cycle, err; /* err: 0 or LULESH_EVOLUME */
    int32_t err_elem, numElem, s, pad_;
    double time, deltatime, dtcourant, dthydro;
} lulesh_slot_status;

/* Per-phase launch shapes of the persistent kernels (forces, nodes,
 * kinematics, material), the tiles a block takes per queue access, and the
 * tile size in units. */
typedef struct lulesh_batch_tuning {
    int32_t block[4];
    int32_t blocks_per_sm[4];
    int32_t grab[4]; /* tiles a block takes per queue access (1..64) */
    int32_t tile;
    int32_t pad_;
    double ms_per_cycle; /* measured by lulesh_batch_autotune */
} lulesh_batch_tuning;

/* pool_bytes of device memory hold the problems' arrays; at most max_slots
 * problems at once. */
int lulesh_batch_create(int32_t precision, uint64_t pool_bytes, int32_t max_slots, lulesh_batch** out);
void lulesh_batch_destroy(lulesh_batch* b);
/* Device bytes one s^3 problem takes in a pool of this precision (for
 * LULESH_FP64 including its element geometry, 384 bytes per element). */
int lulesh_batch_footprint(int32_t precision, int32_t s, uint64_t* bytes);
/* Builds the problem on the device in its pool block (the state
 * Domain::Domain makes, bit for bit; the region runs of the reference's
 * rand() sequence are drawn on the host) and makes it active. LULESH_ENOMEM
 * when the pool or the slots are full. */
int lulesh_batch_admit(lulesh_batch* b, const lulesh_problem* p, int32_t* slot);
/* Admits an existing host Domain (a view as for lulesh_dev_create, with
 * view->time set): its whole state is copied into the pool. stoptime > 0 and
 * max_cycles > 0 override the view's stoptime and the unlimited cycle count. */
int lulesh_batch_admit_view(lulesh_batch* b, const lulesh_domain_view* v, double stoptime,
                            int32_t max_cycles, int32_t* slot);
/* Origin energy e(0) of a slot (the reference's reported result). */
int lulesh_batch_origin_energy(lulesh_batch* b, int32_t slot, double* e0);
/* Frees a slot (finished or not) and its pool memory. */
int lulesh_batch_retire(lulesh_batch* b, int32_t slot);
/* Replays the cycle graph `cycles` times, then refreshes the slot status.
 * *active_slots (optional) = slots still running; *device_ms (optional) =
 * device time of the replays. */
int lulesh_batch_run(lulesh_batch* b, int32_t cycles, int32_t* active_slots, double* device_ms);
int lulesh_batch_status(const lulesh_batch* b, lulesh_slot_status* out, int32_t n);
/* Copies fields of one slot into a host view of the same problem size. */
int lulesh_batch_download(lulesh_batch* b, int32_t slot, lulesh_domain_view* host, uint32_t mask);
/* The final report of one slot, computed on the device (as lulesh_dev_verify). */
int lulesh_batch_verify(lulesh_batch* b, int32_t slot, lulesh_verify_result* out);
/* Times candidate launch shapes and tile sizes on the resident problems
 * (their state is saved first and restored after, so tuning does not
 * advance them), keeps the fastest and reports it. */
int lulesh_batch_autotune(lulesh_batch* b, int32_t cycles_per_candidate, lulesh_batch_tuning* chosen);
int lulesh_batch_get_tuning(const lulesh_batch* b, lulesh_batch_tuning* out);
int lulesh_batch_set_tuning(lulesh_batch* b, const lulesh_batch_tuning* t);
/* Kernel launches issued so far (graph replays count every kernel node). */
int64_t lulesh_batch_launch_count(const lulesh_batch* b);

/* ---------------- serving loop ---------------------------------------------------------
 * No counterpart in the reference. Serves a stream of requests with
 * continuous batching: a worker thread builds each request's Domain on the
 * host once it has arrived (arrival_s after the call starts, wall clock),
 * the loop admits built requests into the resident batch whenever a slot and
 * enough of the hbm_budget pool are free (in arrival order, later requests
 * may pass one that does not fit yet), replays cycles of all resident
 * problems in chunks of about sync_ms of device time, and retires each
 * problem when it reaches its stoptime or cycle limit. Results and
 * time-to-solution (finish - arrival) per request, p50/p99 and aggregate
 * zone-cycles/s in stats. */
typedef struct lulesh_request {
    lulesh_problem problem;
    double arrival_s;
} lulesh_request;

typedef struct lulesh_request_result {
    int32_t cycles, err, s, pad_;
    double arrival_s, admitted_s, finished_s, time_to_solution_s;
    double e0; /* final origin energy */
    double maxabs, totabs, maxrel; /* plane-0 symmetry, computed on the device at retire */
    int64_t zone_cycles;
} lulesh_request_result;

typedef struct lulesh_serve_stats {
    double wall_s;             /* start to the last finish */
    double device_s;           /* device time of the cycle replays */
    double zone_cycles_per_s;  /* all requests' zone-cycles / wall_s */
    double p50_s, p99_s, mean_s; /* time to solution (quantiles interpolated between order statistics) */
    int64_t zone_cycles, launches;
    int32_t served, max_resident; /* requests served; most problems resident at once */
    int64_t peak_resident_bytes;  /* most pool bytes the resident problems held at once
                                     (lulesh_batch_footprint each), against hbm_budget */
    double p50_queue_s, p99_queue_s; /* admission delay (admitted - arrival) */
} lulesh_serve_stats;

int lulesh_serve(int32_t precision, uint64_t hbm_budget, int32_t max_slots, const lulesh_request* reqs,
                 int32_t n, double sync_ms, lulesh_request_result* results, lulesh_serve_stats* stats);

/* Test hooks (no counterpart in the reference; they expose the step's
 * intermediate arrays so each kernel can be checked on its own). */
#define LULESH_PHASE_FORCES 0     /* stress + hourglass corner forces */
#define LULESH_PHASE_NODES 1      /* gather, acceleration, BC, velocity, position */
#define LULESH_PHASE_KINEMATICS 2 /* kinematics + monotonic-Q gradients */
#define LULESH_PHASE_MATERIAL 3   /* Q limiter, EOS x rep, sound speed, dt minima */
int lulesh_dev_phase(lulesh_dev* dev, int32_t phase, double deltatime);
/* Corner forces of the last force phase, stress + hourglass, element-major
 * (index 8*elem + corner), double. */
int lulesh_dev_corner_forces(lulesh_dev* dev, double* fx8, double* fy8, double* fz8);
/* Monotonic-Q gradients of the last kinematics phase, 6 arrays of numElem:
 * delv_xi delv_eta delv_zeta delx_xi delx_eta delx_zeta, as double. */
int lulesh_dev_gradients(lulesh_dev* dev, double* out6);
/* Element index that raised the last LULESH_EVOLUME (or -1). */
int32_t lulesh_dev_error_elem(const lulesh_dev* dev);
/* Number of kernel launches issued by this handle so far. */
int64_t lulesh_dev_launch_count(const lulesh_dev* dev);

/* Device-side timing (no counterpart in the reference, which wall-clocks
 * its whole time loop, lulesh.cc:2368-2395). Between begin and end the
 * handle records CUDA events on its stream: total_ms spans the whole
 * interval on the device timeline; kernel_ms[k] sums the durations of the
 * forces, nodes, kinematics and material kernels of lulesh_dev_step cycles
 * (the graph form contributes to total_ms only). */
typedef struct lulesh_profile {
    double total_ms;
    double kernel_ms[4];
    int64_t cycles;   /* lulesh_dev_step cycles timed per kernel */
    int64_t launches; /* kernels launched between begin and end */
} lulesh_profile;
int lulesh_dev_profile_begin(lulesh_dev* dev);
int lulesh_dev_profile_end(lulesh_dev* dev, lulesh_profile* out);

/* Stage timeline of lulesh_leapfrog (no counterpart in the reference). With
 * the timeline on, each call records a CUDA event, on the stream that does
 * the work, at every stage boundary of its slab pipeline;
 * lulesh_leapfrog_timeline_read returns the last call's marks: ms[k] is the
 * time of mark k after the call's first device work, stage[k] its kind
 * (LULESH_TL_*), index[k] its slab, node range or kinematics group, and
 * wall_ms the call's wall time on the host. Off (the default) it costs
 * nothing. */
#define LULESH_TL_UPLOAD 1     /* a slab's inputs are on the device */
#define LULESH_TL_FORCES 2     /* a slab's corner forces are formed */
#define LULESH_TL_ENERGY_UP 3  /* the energy is on the device */
#define LULESH_TL_NODES 4      /* a node range is updated */
#define LULESH_TL_NODES_DOWN 5 /* its node fields are in host memory */
#define LULESH_TL_KIN 6        /* a kinematics group is done */
#define LULESH_TL_KIN_DOWN 7   /* its element fields are in host memory */
#define LULESH_TL_MAT 8        /* a material slab is done */
#define LULESH_TL_MAT_DOWN 9   /* its element fields are in host memory */
#define LULESH_TL_END 10       /* the dt minima and error word are back */
#define LULESH_TL_MAX 96
typedef struct lulesh_timeline {
    int32_t n;
    int32_t stage[LULESH_TL_MAX], index[LULESH_TL_MAX];
    float ms[LULESH_TL_MAX];
    double wall_ms;
} lulesh_timeline;
int lulesh_leapfrog_timeline(lulesh_dev* dev, int32_t on);
int lulesh_leapfrog_timeline_read(const lulesh_dev* dev, lulesh_timeline* out);

/* Courant and hydro time-step constraints without allocating device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc, such as a host framework that owns every device allocation
 * through its own pool or budget, or a loop that cannot afford cudaMalloc's
 * possible device-wide synchronization. From the caller's device arrays ss,
 * vdov and arealg (numElem each) it writes out_dt[0] = dtcourant and
 * out_dt[1] = dthydro (out_dt: 2 doubles of device memory), using qqc and
 * dvovmax of lulesh_params: the minima lulesh_dev_step returns for the same
 * arrays on a LULESH_FP64 or LULESH_MIXED handle, bit for bit (the same
 * arithmetic), and within about one ulp of a LULESH_FP64_EXACT handle's
 * (whose divide and square root are IEEE). Values are folded with fmin, so
 * any finite input works and NaN candidates are ignored.
 * Asynchronous on `stream` (a cudaStream_t; NULL = the legacy default stream).
 * Working memory is one file-scope device array of 256 KiB that every GPU
 * loading this library keeps until exit; it bounds numElem to
 * LULESH_NOALLOC_MAX_ELEMS and larger sizes return LULESH_EINVAL. Each call
 * whose stream is not capturing looks up that array's device address (so it
 * follows a device reset); a call during stream capture reuses the last
 * address, so the first call on a device must come before any capture
 * (LULESH_EINVAL otherwise). Calls share the array: calls whose kernels
 * overlap on the GPU race and must be serialized by the caller. */
#define LULESH_NOALLOC_MAX_ELEMS 4194304
int lulesh_dt_constraints_noalloc(const double* ss, const double* vdov, const double* arealg,
                                  int32_t numElem, double qqc, double dvovmax, double* out_dt,
                                  void* stream);

/* Page-locks (pin = 1) or releases (pin = 0) the host arrays of a Domain so
 * lulesh_leapfrog's per-cycle copies run at full link bandwidth. */
int lulesh_domain_pin(lulesh_domain* d, int32_t pin);

/* Selects the CUDA device used by handles created afterwards on this thread. */
int lulesh_set_device(int32_t device);

/* The cube root used by LULESH_FP64_EXACT for the hourglass coefficient
 * (lulesh.cc:1068 uses cbrt): built from IEEE add/mul/fma/div only, so the
 * GPU and a CPU build of the same steps round identically. */
double lulesh_cbrt_portable(double x);

const char* lulesh_strerror(int32_t status);

#ifdef __cplusplus
}
#endif
#endif
