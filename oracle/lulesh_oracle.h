/* CPU oracle for the LULESH Lagrange-leapfrog step (test infrastructure).
 *
 * A plain-C restatement of the reference algorithm of
 * esa-tu-darmstadt/lulesh-task-based-hpx (lulesh.cc, lulesh-init.cc,
 * lulesh-util.cc). It is the oracle the GPU path's results are compared
 * with, and the timed CPU baseline where the reference sources are absent.
 * Built with -ffp-contract=off it reproduces the reference, compiled the
 * same way, bit for bit (tests/test_oracle.py pins this).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 */
#ifndef LULESH_ORACLE_H
#define LULESH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes, as the reference's exit codes (lulesh.h:30). */
#define LO_OK 0
#define LO_VOLUME_ERROR (-1)

typedef struct lo_domain lo_domain;

/* Builds the Sedov problem of Domain::Domain (lulesh-init.cc:10-183) for an
 * s^3 mesh with nr regions. energy_scale multiplies the deposited origin
 * energy (1.0 reproduces the reference); deltatime is then derived from the
 * scaled energy with the formula of lulesh-init.cc:181. */
lo_domain* lo_create(int s, int nr, int balance, int cost, double energy_scale);
void lo_destroy(lo_domain* d);

/* Cube root used for the hourglass coefficient: 0 = libm cbrt (the
 * reference), 1 = the portable IEEE-only cube root of the GPU's exact path. */
void lo_set_cbrt_mode(int mode);
double lo_portable_cbrt(double x);

/* Worker threads for the element/node loops (OpenMP builds only). */
void lo_set_threads(int n);
int lo_get_threads(void);

/* TimeIncrement (lulesh.cc:182-229). */
void lo_time_increment(lo_domain* d);
/* One LagrangeLeapFrog cycle (lulesh.cc:1977-2240). Returns LO_OK or
 * LO_VOLUME_ERROR where the reference would exit(VolumeError). */
int lo_leapfrog(lo_domain* d);
/* The time loop of hpx_main (lulesh.cc:2374-2386): TimeIncrement + step
 * until stoptime or max_cycles. Returns LO_OK or LO_VOLUME_ERROR. */
int lo_run(lo_domain* d, int max_cycles);

/* Plane-0 energy symmetry statistics (lulesh-util.cc:77-103):
 * out[0]=MaxAbsDiff, out[1]=TotalAbsDiff, out[2]=MaxRelDiff. */
void lo_symmetry(const lo_domain* d, double out[3]);

/* Writes the state in the "LULESHD1" field-dump layout (see ref_report.cc).
 * Returns 0 on success. */
int lo_dump(const lo_domain* d, const char* path);

/* Field access by name. Returns a pointer to the array (double or int32, as
 * *is_int says) and its length, or NULL for an unknown name. Names follow the
 * Domain accessors: x y z xd yd zd xdd ydd zdd fx fy fz nodalMass e p q ql qq
 * v volo vnew delv vdov arealg ss elemMass delv_xi delv_eta delv_zeta delx_xi
 * delx_eta delx_zeta fx_elem fy_elem fz_elem (8 corner forces per element,
 * stress + hourglass of the last cycle), nodelist lxim lxip letam letap
 * lzetam lzetap elemBC nodeElemStart nodeElemCornerList regNumList symmX
 * symmY symmZ regElemSize. */
void* lo_field(lo_domain* d, const char* name, long* len, int* is_int);

/* Scalars: 0 time, 1 deltatime, 2 dtcourant, 3 dthydro, 4 stoptime,
 * 5 dtmax, 6 dtfixed, 7 cycle. lo_set_scalar writes 0-7 likewise. */
double lo_get_scalar(const lo_domain* d, int which);
void lo_set_scalar(lo_domain* d, int which, double v);
int lo_num_elem(const lo_domain* d);
int lo_num_node(const lo_domain* d);
int lo_num_reg(const lo_domain* d);
/* Region list r (0-based) and its size. */
const int* lo_region(const lo_domain* d, int r, int* size);

#ifdef __cplusplus
}
#endif
#endif
