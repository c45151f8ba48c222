/* CPU oracle for the LULESH Lagrange-leapfrog step: a plain-C restatement of
 * the reference algorithm (esa-tu-darmstadt/lulesh-task-based-hpx).
 *
 * TEST INFRASTRUCTURE. The GPU product never links this file; tests/,
 * __graft_entry__.smoke() and bench.py's CPU baseline do.
 *
 * Structure. The reference splits each cycle into HPX chunk tasks
 * (lulesh.cc:1977-2240). Every one of those tasks is element-wise or
 * node-wise (each output location is written by one iteration from inputs no
 * other iteration of the same phase writes), the nodal gather walks the
 * node->corner CSR in order, and the two dt reductions are exact minima. So
 * the same results come from one parallel loop per phase, which is how this
 * file is organised:
 *   phase_forces   stress + FB hourglass corner forces   lulesh.cc:787-836, 864-1113
 *   phase_nodes    CSR gather, a=f/m, symmetry BC, v, x    lulesh.cc:838-862, 1115-1158, 566-588
 *   phase_kinematics  volume, arealg, vdov, v<-vnew       lulesh.cc:1169-1275
 *   phase_qgrad    monotonic-Q gradients                  lulesh.cc:1277-1418
 *   phase_material Q limiter, EOS x rep, sound speed      lulesh.cc:1420-1924, 2144-2206
 *   phase_dt       Courant and hydro dt minima            lulesh.cc:1938-1974, 2207-2237
 * Each arithmetic expression keeps the reference's operand order and
 * parenthesisation, because with -ffp-contract=off that fixes the rounding
 * of every operation and makes this port bit-identical to the reference.
 *
 * Errors: where the reference calls exit(VolumeError) the phase records
 * LO_VOLUME_ERROR and lo_leapfrog returns it.
 */
#include "lulesh_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Boundary-condition bit masks of an element face (lulesh.h:46-74). */
#define XI_M 0x00007
#define XI_M_SYMM 0x00001
#define XI_M_FREE 0x00002
#define XI_M_COMM 0x00004
#define XI_P 0x00038
#define XI_P_SYMM 0x00008
#define XI_P_FREE 0x00010
#define XI_P_COMM 0x00020
#define ETA_M 0x001c0
#define ETA_M_SYMM 0x00040
#define ETA_M_FREE 0x00080
#define ETA_M_COMM 0x00100
#define ETA_P 0x00e00
#define ETA_P_SYMM 0x00200
#define ETA_P_FREE 0x00400
#define ETA_P_COMM 0x00800
#define ZETA_M 0x07000
#define ZETA_M_SYMM 0x01000
#define ZETA_M_FREE 0x02000
#define ZETA_M_COMM 0x04000
#define ZETA_P 0x38000
#define ZETA_P_SYMM 0x08000
#define ZETA_P_FREE 0x10000
#define ZETA_P_COMM 0x20000

struct lo_domain {
    int s, numElem, numNode, numReg, cost, balance, numSymm;
    /* node-centred */
    double *x, *y, *z, *xd, *yd, *zd, *xdd, *ydd, *zdd, *fx, *fy, *fz, *nodalMass;
    int *symmX, *symmY, *symmZ;
    unsigned char* nodeSymm; /* bit 0/1/2: node lies in the x/y/z symmetry set */
    /* element-centred */
    int *nodelist, *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elemBC;
    double *e, *p, *q, *ql, *qq, *v, *volo, *vnew, *delv, *vdov, *arealg, *ss, *elemMass;
    double *delv_xi, *delv_eta, *delv_zeta, *delx_xi, *delx_eta, *delx_zeta;
    double *fx_stress, *fy_stress, *fz_stress, *fx_hg, *fy_hg, *fz_hg; /* 8 per element */
    double *fx_elem, *fy_elem, *fz_elem; /* stress + hourglass, for inspection */
    int *nodeElemStart, *nodeElemCornerList;
    int *regElemSize, *regNumList, **regElemlist;
    /* constants (lulesh-init.cc:18-36) */
    double e_cut, p_cut, q_cut, v_cut, u_cut, hgcoef, ss4o3, qstop, monoq_max_slope,
        monoq_limiter_mult, qlc_monoq, qqc_monoq, qqc, eosvmax, eosvmin, pmin, emin, dvovmax,
        refdens;
    /* time control (lulesh-init.cc:135-145) */
    double dtcourant, dthydro, dtfixed, time, deltatime, deltatimemultlb, deltatimemultub,
        dtmax, stoptime;
    int cycle;
};

static int g_threads = 0;
static int g_cbrt_mode = 0;

/* Cube root of the hourglass coefficient. Mode 0 is libm cbrt, as the
 * reference (lulesh.cc:1068). Mode 1 is a cube root built from IEEE add,
 * multiply and divide only (exponent split x = m 2^(3k), m in [1,8);
 * least-squares quadratic start on [1,8]; four Halley steps
 * y <- y (y^3 + 2m) / (2y^3 + m); exact rescale by 2^k), the same steps the
 * GPU's LULESH_FP64_EXACT path takes, so the two agree bit for bit. */
static double portable_cbrt(double x) {
    if (!(x > 0.0)) {
        if (x < 0.0) return -portable_cbrt(-x);
        return x;
    }
    uint64_t bits;
    memcpy(&bits, &x, sizeof bits);
    int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0x7ff) return x;
    if (ex == 0) return portable_cbrt(x * 18014398509481984.0) * 3.814697265625e-06;
    int e = ex - 1023;
    int k = (e >= 0) ? e / 3 : -((2 - e) / 3);
    int r = e - 3 * k;
    uint64_t mb = (bits & 0x000fffffffffffffULL) | ((uint64_t)(1023 + r) << 52);
    double m;
    memcpy(&m, &mb, sizeof m);
    double y = 0.8209 + m * (0.2374 - m * 0.01159);
    for (int it = 0; it < 4; ++it) {
        double y3 = y * y * y;
        y = y * (y3 + 2.0 * m) / (2.0 * y3 + m);
    }
    /* Newton correction with an error-free residual y^3 - m */
    double t = y * y;
    double e1 = fma(y, y, -t);
    double u = t * y;
    double e2 = fma(t, y, -u);
    double res = (u - m) + (e2 + e1 * y);
    y = y - res / (3.0 * t);
    uint64_t sb = (uint64_t)(1023 + k) << 52;
    double scale;
    memcpy(&scale, &sb, sizeof scale);
    return y * scale;
}

void lo_set_cbrt_mode(int mode) { g_cbrt_mode = mode; }
double lo_portable_cbrt(double x) { return portable_cbrt(x); }

static inline double hg_cbrt(double x) { return g_cbrt_mode ? portable_cbrt(x) : cbrt(x); }

void lo_set_threads(int n) {
    g_threads = n;
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}

int lo_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) {
        fprintf(stderr, "lulesh_oracle: out of memory\n");
        abort();
    }
    return p;
}
#define DALLOC(n) ((double*)xcalloc((size_t)(n), sizeof(double)))
#define IALLOC(n) ((int*)xcalloc((size_t)(n), sizeof(int)))

/* ------------------------------------------------------------------ */
/* Element geometry kernels                                            */
/* ------------------------------------------------------------------ */

/* Triple product of the three vectors (a1,a2,a3) (b1,b2,b3) (c1,c2,c3) as the
 * TRIPLE_PRODUCT macro of lulesh.cc:649-651 evaluates it. The arguments are
 * passed in the macro's order: (x1,y1,z1,x2,y2,z2,x3,y3,z3). */
static inline double triple(double x1, double y1, double z1, double x2, double y2, double z2,
                            double x3, double y3, double z3) {
    return x1 * (y2 * z3 - z2 * y3) + x2 * (z1 * y3 - y1 * z3) + x3 * (y1 * z2 - z1 * y2);
}

/* Hexahedron volume (lulesh.cc:592-665). */
static double hex_volume(const double x[8], const double y[8], const double z[8]) {
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
    double vol = triple(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
                 triple(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
                 triple(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
    vol *= twelveth;
    return vol;
}

/* Jacobian of the trilinear map at the element centre, its cofactors, the
 * shape-function derivatives b[3][8] and 8*det (lulesh.cc:277-374). b may be
 * NULL when only the determinant is wanted. */
static double shape_derivs(const double x[8], const double y[8], const double z[8], double b[3][8]) {
    double fjxxi = .125 * ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    double fjxet = .125 * ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    double fjxze = .125 * ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    double fjyxi = .125 * ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    double fjyet = .125 * ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    double fjyze = .125 * ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    double fjzxi = .125 * ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    double fjzet = .125 * ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    double fjzze = .125 * ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));

    double cjxxi = (fjyet * fjzze) - (fjzet * fjyze);
    double cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    double cjxze = (fjyxi * fjzet) - (fjzxi * fjyet);
    double cjyxi = -(fjxet * fjzze) + (fjzet * fjxze);
    double cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    double cjyze = -(fjxxi * fjzet) + (fjzxi * fjxet);
    double cjzxi = (fjxet * fjyze) - (fjyet * fjxze);
    double cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    double cjzze = (fjxxi * fjyet) - (fjyxi * fjxet);

    if (b) {
        b[0][0] = -cjxxi - cjxet - cjxze;
        b[0][1] = cjxxi - cjxet - cjxze;
        b[0][2] = cjxxi + cjxet - cjxze;
        b[0][3] = -cjxxi + cjxet - cjxze;
        b[0][4] = -b[0][2];
        b[0][5] = -b[0][3];
        b[0][6] = -b[0][0];
        b[0][7] = -b[0][1];
        b[1][0] = -cjyxi - cjyet - cjyze;
        b[1][1] = cjyxi - cjyet - cjyze;
        b[1][2] = cjyxi + cjyet - cjyze;
        b[1][3] = -cjyxi + cjyet - cjyze;
        b[1][4] = -b[1][2];
        b[1][5] = -b[1][3];
        b[1][6] = -b[1][0];
        b[1][7] = -b[1][1];
        b[2][0] = -cjzxi - cjzet - cjzze;
        b[2][1] = cjzxi - cjzet - cjzze;
        b[2][2] = cjzxi + cjzet - cjzze;
        b[2][3] = -cjzxi + cjzet - cjzze;
        b[2][4] = -b[2][2];
        b[2][5] = -b[2][3];
        b[2][6] = -b[2][0];
        b[2][7] = -b[2][1];
    }
    return 8. * (fjxet * cjxet + fjyet * cjyet + fjzet * cjzet);
}

/* Area-weighted normal of one quadrilateral face, added to its 4 corners
 * (lulesh.cc:378-409). c[] are the face's corner indices in face order. */
static inline void face_normal_add(double nx[8], double ny[8], double nz[8], const int c[4],
                                   const double x[8], const double y[8], const double z[8]) {
    double x0 = x[c[0]], x1 = x[c[1]], x2 = x[c[2]], x3 = x[c[3]];
    double y0 = y[c[0]], y1 = y[c[1]], y2 = y[c[2]], y3 = y[c[3]];
    double z0 = z[c[0]], z1 = z[c[1]], z2 = z[c[2]], z3 = z[c[3]];
    double bisX0 = 0.5 * (x3 + x2 - x1 - x0);
    double bisY0 = 0.5 * (y3 + y2 - y1 - y0);
    double bisZ0 = 0.5 * (z3 + z2 - z1 - z0);
    double bisX1 = 0.5 * (x2 + x1 - x3 - x0);
    double bisY1 = 0.5 * (y2 + y1 - y3 - y0);
    double bisZ1 = 0.5 * (z2 + z1 - z3 - z0);
    double ax = 0.25 * (bisY0 * bisZ1 - bisZ0 * bisY1);
    double ay = 0.25 * (bisZ0 * bisX1 - bisX0 * bisZ1);
    double az = 0.25 * (bisX0 * bisY1 - bisY0 * bisX1);
    for (int k = 0; k < 4; ++k) {
        nx[c[k]] += ax;
        ny[c[k]] += ay;
        nz[c[k]] += az;
    }
}

/* The six faces in the order CalcElemNodeNormals visits them
 * (lulesh.cc:421-450). */
static const int kFaceNormalOrder[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2},
                                           {2, 6, 7, 3}, {3, 7, 4, 0}, {4, 7, 6, 5}};

static void node_normals(double nx[8], double ny[8], double nz[8], const double x[8],
                         const double y[8], const double z[8]) {
    for (int i = 0; i < 8; ++i) nx[i] = ny[i] = nz[i] = 0.0;
    for (int f = 0; f < 6; ++f) face_normal_add(nx, ny, nz, kFaceNormalOrder[f], x, y, z);
}

/* Volume derivative with respect to one corner from the six neighbouring
 * corner coordinates a[0..5] (lulesh.cc:468-491). */
static inline void volu_der(const double xa[6], const double ya[6], const double za[6],
                            double* dvdx, double* dvdy, double* dvdz) {
    const double twelfth = 1.0 / 12.0;
    double x0 = xa[0], x1 = xa[1], x2 = xa[2], x3 = xa[3], x4 = xa[4], x5 = xa[5];
    double y0 = ya[0], y1 = ya[1], y2 = ya[2], y3 = ya[3], y4 = ya[4], y5 = ya[5];
    double z0 = za[0], z1 = za[1], z2 = za[2], z3 = za[3], z4 = za[4], z5 = za[5];
    *dvdx = (y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2) + (y0 + y4) * (z3 + z4) -
            (y3 + y4) * (z0 + z4) - (y2 + y5) * (z3 + z5) + (y3 + y5) * (z2 + z5);
    *dvdy = -(x1 + x2) * (z0 + z1) + (x0 + x1) * (z1 + z2) - (x0 + x4) * (z3 + z4) +
            (x3 + x4) * (z0 + z4) + (x2 + x5) * (z3 + z5) - (x3 + x5) * (z2 + z5);
    *dvdz = -(y1 + y2) * (x0 + x1) + (y0 + y1) * (x1 + x2) - (y0 + y4) * (x3 + x4) +
            (y3 + y4) * (x0 + x4) + (y2 + y5) * (x3 + x5) - (y3 + y5) * (x2 + x5);
    *dvdx *= twelfth;
    *dvdy *= twelfth;
    *dvdz *= twelfth;
}

/* Neighbour corners used for each corner's volume derivative
 * (lulesh.cc:499-522): row k lists the six corners for corner kVoluDerCorner[k]. */
static const int kVoluDerCorner[8] = {0, 3, 2, 1, 4, 5, 6, 7};
static const int kVoluDerArgs[8][6] = {{1, 2, 3, 4, 5, 7}, {0, 1, 2, 7, 4, 6}, {3, 0, 1, 6, 7, 5},
                                       {2, 3, 0, 5, 6, 4}, {7, 6, 5, 0, 3, 1}, {4, 7, 6, 1, 0, 2},
                                       {5, 4, 7, 2, 1, 3}, {6, 5, 4, 3, 2, 0}};

static void volume_derivs(double dvdx[8], double dvdy[8], double dvdz[8], const double x[8],
                          const double y[8], const double z[8]) {
    for (int k = 0; k < 8; ++k) {
        double xa[6], ya[6], za[6];
        for (int j = 0; j < 6; ++j) {
            xa[j] = x[kVoluDerArgs[k][j]];
            ya[j] = y[kVoluDerArgs[k][j]];
            za[j] = z[kVoluDerArgs[k][j]];
        }
        int c = kVoluDerCorner[k];
        volu_der(xa, ya, za, &dvdx[c], &dvdy[c], &dvdz[c]);
    }
}

/* Flanagan-Belytschko hourglass base vectors (lulesh.cc:921-954). */
static const double kGamma[4][8] = {{1., 1., -1., -1., -1., -1., 1., 1.},
                                    {1., -1., -1., 1., -1., 1., 1., -1.},
                                    {1., -1., 1., -1., 1., -1., 1., -1.},
                                    {-1., 1., -1., 1., 1., -1., 1., -1.}};

/* Face area measure used by the characteristic length (lulesh.cc:678-692). */
static inline double face_area(double x0, double x1, double x2, double x3, double y0, double y1,
                               double y2, double y3, double z0, double z1, double z2, double z3) {
    double fx = (x2 - x0) - (x3 - x1);
    double fy = (y2 - y0) - (y3 - y1);
    double fz = (z2 - z0) - (z3 - z1);
    double gx = (x2 - x0) + (x3 - x1);
    double gy = (y2 - y0) + (y3 - y1);
    double gz = (z2 - z0) + (z3 - z1);
    return (fx * fx + fy * fy + fz * fz) * (gx * gx + gy * gy + gz * gz) -
           (fx * gx + fy * gy + fz * gz) * (fx * gx + fy * gy + fz * gz);
}

static const int kCharFaces[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                     {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};

/* 4 V / sqrt(largest face measure) (lulesh.cc:696-729). */
static double char_length(const double x[8], const double y[8], const double z[8], double volume) {
    double cl = 0.0;
    for (int f = 0; f < 6; ++f) {
        const int* c = kCharFaces[f];
        double a = face_area(x[c[0]], x[c[1]], x[c[2]], x[c[3]], y[c[0]], y[c[1]], y[c[2]],
                             y[c[3]], z[c[0]], z[c[1]], z[c[2]], z[c[3]]);
        cl = (a < cl) ? cl : a; /* std::max(a, cl) */
    }
    return 4.0 * volume / sqrt(cl);
}

static void gather8(const double* f, const int* nl, double out[8]) {
    for (int k = 0; k < 8; ++k) out[k] = f[nl[k]];
}

/* ------------------------------------------------------------------ */
/* Phases                                                              */
/* ------------------------------------------------------------------ */

/* Stress and hourglass corner forces of every element
 * (InitIntegrateStressForElemsTask lulesh.cc:787-836,
 *  CalcHourglassForElemsTask lulesh.cc:864-1113). */
static int phase_forces(lo_domain* d) {
    int err = 0;
    const double hgcoef = d->hgcoef;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int i = 0; i < d->numElem; ++i) {
        const int* nl = &d->nodelist[8 * i];
        double x[8], y[8], z[8];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);

        /* stress: sigma = -p - q on the diagonal */
        double sig = -d->p[i] - d->q[i];
        double det = shape_derivs(x, y, z, NULL);
        if (det == 0) err |= 1;
        double nx[8], ny[8], nz[8];
        node_normals(nx, ny, nz, x, y, z);
        for (int k = 0; k < 8; ++k) {
            d->fx_stress[8 * i + k] = -(sig * nx[k]);
            d->fy_stress[8 * i + k] = -(sig * ny[k]);
            d->fz_stress[8 * i + k] = -(sig * nz[k]);
        }

        /* hourglass */
        double dvdx[8], dvdy[8], dvdz[8];
        volume_derivs(dvdx, dvdy, dvdz, x, y, z);
        double determ = d->volo[i] * d->v[i];
        if (determ <= 0.0) {
            err |= 1;
            continue;
        }
        double volinv = 1.0 / determ;
        double hg[8][4];
        for (int m = 0; m < 4; ++m) {
            const double* g = kGamma[m];
            double hx = x[0] * g[0] + x[1] * g[1] + x[2] * g[2] + x[3] * g[3] + x[4] * g[4] +
                        x[5] * g[5] + x[6] * g[6] + x[7] * g[7];
            double hy = y[0] * g[0] + y[1] * g[1] + y[2] * g[2] + y[3] * g[3] + y[4] * g[4] +
                        y[5] * g[5] + y[6] * g[6] + y[7] * g[7];
            double hz = z[0] * g[0] + z[1] * g[1] + z[2] * g[2] + z[3] * g[3] + z[4] * g[4] +
                        z[5] * g[5] + z[6] * g[6] + z[7] * g[7];
            for (int k = 0; k < 8; ++k)
                hg[k][m] = g[k] - volinv * (dvdx[k] * hx + dvdy[k] * hy + dvdz[k] * hz);
        }
        double coefficient = -hgcoef * 0.01 * d->ss[i] * d->elemMass[i] / hg_cbrt(determ);
        double vel[8];
        double* outs[3] = {d->fx_hg, d->fy_hg, d->fz_hg};
        const double* vsrc[3] = {d->xd, d->yd, d->zd};
        for (int a = 0; a < 3; ++a) {
            gather8(vsrc[a], nl, vel);
            double h[4];
            for (int m = 0; m < 4; ++m)
                h[m] = hg[0][m] * vel[0] + hg[1][m] * vel[1] + hg[2][m] * vel[2] +
                       hg[3][m] * vel[3] + hg[4][m] * vel[4] + hg[5][m] * vel[5] +
                       hg[6][m] * vel[6] + hg[7][m] * vel[7];
            for (int k = 0; k < 8; ++k)
                outs[a][8 * i + k] = coefficient * (hg[k][0] * h[0] + hg[k][1] * h[1] +
                                                    hg[k][2] * h[2] + hg[k][3] * h[3]);
        }
    }
#pragma omp parallel for schedule(static)
    for (long c = 0; c < 8L * d->numElem; ++c) {
        d->fx_elem[c] = d->fx_stress[c] + d->fx_hg[c];
        d->fy_elem[c] = d->fy_stress[c] + d->fy_hg[c];
        d->fz_elem[c] = d->fz_stress[c] + d->fz_hg[c];
    }
    return err ? LO_VOLUME_ERROR : LO_OK;
}

/* Node phase: force gather in CSR order adding the stress then the
 * hourglass corner force (lulesh.cc:838-862), acceleration (1115-1123),
 * symmetry-plane zeroing (566-588), velocity with u_cut and position
 * (1125-1158). */
static void phase_nodes(lo_domain* d) {
    const double dt = d->deltatime, u_cut = d->u_cut;
#pragma omp parallel for schedule(static)
    for (int n = 0; n < d->numNode; ++n) {
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int j = d->nodeElemStart[n]; j < d->nodeElemStart[n + 1]; ++j) {
            int c = d->nodeElemCornerList[j];
            fx += d->fx_stress[c];
            fx += d->fx_hg[c];
            fy += d->fy_stress[c];
            fy += d->fy_hg[c];
            fz += d->fz_stress[c];
            fz += d->fz_hg[c];
        }
        d->fx[n] = fx;
        d->fy[n] = fy;
        d->fz[n] = fz;
        double m = d->nodalMass[n];
        double ax = fx / m, ay = fy / m, az = fz / m;
        unsigned char sym = d->nodeSymm[n];
        if (sym & 1) ax = 0.0;
        if (sym & 2) ay = 0.0;
        if (sym & 4) az = 0.0;
        d->xdd[n] = ax;
        d->ydd[n] = ay;
        d->zdd[n] = az;
        double vx = d->xd[n] + ax * dt;
        if (fabs(vx) < u_cut) vx = 0.0;
        double vy = d->yd[n] + ay * dt;
        if (fabs(vy) < u_cut) vy = 0.0;
        double vz = d->zd[n] + az * dt;
        if (fabs(vz) < u_cut) vz = 0.0;
        d->xd[n] = vx;
        d->yd[n] = vy;
        d->zd[n] = vz;
        d->x[n] = d->x[n] + vx * dt;
        d->y[n] = d->y[n] + vy * dt;
        d->z[n] = d->z[n] + vz * dt;
    }
}

/* Kinematics (lulesh.cc:1169-1275): new relative volume, its change,
 * characteristic length, vdov = trace of the velocity gradient at the
 * half-step geometry, the relative-volume check, and v <- vnew snapped
 * to 1 within v_cut. */
static int phase_kinematics(lo_domain* d) {
    int err = 0;
    const double dt = d->deltatime;
    const double eosvmin = d->eosvmin, eosvmax = d->eosvmax, v_cut = d->v_cut;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int i = 0; i < d->numElem; ++i) {
        const int* nl = &d->nodelist[8 * i];
        double x[8], y[8], z[8], xv[8], yv[8], zv[8];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        double volume = hex_volume(x, y, z);
        double relv = volume / d->volo[i];
        double vold = d->v[i];
        d->vnew[i] = relv;
        d->delv[i] = relv - vold;
        d->arealg[i] = char_length(x, y, z, volume);
        gather8(d->xd, nl, xv);
        gather8(d->yd, nl, yv);
        gather8(d->zd, nl, zv);
        double dt2 = 0.5 * dt;
        for (int k = 0; k < 8; ++k) {
            x[k] -= dt2 * xv[k];
            y[k] -= dt2 * yv[k];
            z[k] -= dt2 * zv[k];
        }
        double b[3][8];
        double detJ = shape_derivs(x, y, z, b);
        double inv = 1.0 / detJ;
        double dxx = inv * (b[0][0] * (xv[0] - xv[6]) + b[0][1] * (xv[1] - xv[7]) +
                            b[0][2] * (xv[2] - xv[4]) + b[0][3] * (xv[3] - xv[5]));
        double dyy = inv * (b[1][0] * (yv[0] - yv[6]) + b[1][1] * (yv[1] - yv[7]) +
                            b[1][2] * (yv[2] - yv[4]) + b[1][3] * (yv[3] - yv[5]));
        double dzz = inv * (b[2][0] * (zv[0] - zv[6]) + b[2][1] * (zv[1] - zv[7]) +
                            b[2][2] * (zv[2] - zv[4]) + b[2][3] * (zv[3] - zv[5]));
        d->vdov[i] = dxx + dyy + dzz;
        /* CheckAndUpdateVolumeForElems: the check reads the old v */
        double vc = vold;
        if (eosvmin != 0.0 && vc < eosvmin) vc = eosvmin;
        if (eosvmax != 0.0 && vc > eosvmax) vc = eosvmax;
        if (vc < 0.0) err |= 1;
        double vn = relv;
        if (fabs(vn - 1.0) < v_cut) vn = 1.0;
        d->v[i] = vn;
    }
    return err ? LO_VOLUME_ERROR : LO_OK;
}

/* Monotonic-Q position and velocity gradients (lulesh.cc:1277-1418). */
static void phase_qgrad(lo_domain* d) {
    const double ptiny = 1.e-36;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < d->numElem; ++i) {
        const int* nl = &d->nodelist[8 * i];
        double x[8], y[8], z[8], xv[8], yv[8], zv[8];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        gather8(d->xd, nl, xv);
        gather8(d->yd, nl, yv);
        gather8(d->zd, nl, zv);
        double vol = d->volo[i] * d->vnew[i];
        double norm = 1.0 / (vol + ptiny);

        double dxj = -0.25 * ((x[0] + x[1] + x[5] + x[4]) - (x[3] + x[2] + x[6] + x[7]));
        double dyj = -0.25 * ((y[0] + y[1] + y[5] + y[4]) - (y[3] + y[2] + y[6] + y[7]));
        double dzj = -0.25 * ((z[0] + z[1] + z[5] + z[4]) - (z[3] + z[2] + z[6] + z[7]));
        double dxi = 0.25 * ((x[1] + x[2] + x[6] + x[5]) - (x[0] + x[3] + x[7] + x[4]));
        double dyi = 0.25 * ((y[1] + y[2] + y[6] + y[5]) - (y[0] + y[3] + y[7] + y[4]));
        double dzi = 0.25 * ((z[1] + z[2] + z[6] + z[5]) - (z[0] + z[3] + z[7] + z[4]));
        double dxk = 0.25 * ((x[4] + x[5] + x[6] + x[7]) - (x[0] + x[1] + x[2] + x[3]));
        double dyk = 0.25 * ((y[4] + y[5] + y[6] + y[7]) - (y[0] + y[1] + y[2] + y[3]));
        double dzk = 0.25 * ((z[4] + z[5] + z[6] + z[7]) - (z[0] + z[1] + z[2] + z[3]));
        double ax, ay, az, dxv, dyv, dzv;

        /* zeta: i cross j */
        ax = dyi * dzj - dzi * dyj;
        ay = dzi * dxj - dxi * dzj;
        az = dxi * dyj - dyi * dxj;
        d->delx_zeta[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm;
        ay *= norm;
        az *= norm;
        dxv = 0.25 * ((xv[4] + xv[5] + xv[6] + xv[7]) - (xv[0] + xv[1] + xv[2] + xv[3]));
        dyv = 0.25 * ((yv[4] + yv[5] + yv[6] + yv[7]) - (yv[0] + yv[1] + yv[2] + yv[3]));
        dzv = 0.25 * ((zv[4] + zv[5] + zv[6] + zv[7]) - (zv[0] + zv[1] + zv[2] + zv[3]));
        d->delv_zeta[i] = ax * dxv + ay * dyv + az * dzv;

        /* xi: j cross k */
        ax = dyj * dzk - dzj * dyk;
        ay = dzj * dxk - dxj * dzk;
        az = dxj * dyk - dyj * dxk;
        d->delx_xi[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm;
        ay *= norm;
        az *= norm;
        dxv = 0.25 * ((xv[1] + xv[2] + xv[6] + xv[5]) - (xv[0] + xv[3] + xv[7] + xv[4]));
        dyv = 0.25 * ((yv[1] + yv[2] + yv[6] + yv[5]) - (yv[0] + yv[3] + yv[7] + yv[4]));
        dzv = 0.25 * ((zv[1] + zv[2] + zv[6] + zv[5]) - (zv[0] + zv[3] + zv[7] + zv[4]));
        d->delv_xi[i] = ax * dxv + ay * dyv + az * dzv;

        /* eta: k cross i */
        ax = dyk * dzi - dzk * dyi;
        ay = dzk * dxi - dxk * dzi;
        az = dxk * dyi - dyk * dxi;
        d->delx_eta[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm;
        ay *= norm;
        az *= norm;
        dxv = -0.25 * ((xv[0] + xv[1] + xv[5] + xv[4]) - (xv[3] + xv[2] + xv[6] + xv[7]));
        dyv = -0.25 * ((yv[0] + yv[1] + yv[5] + yv[4]) - (yv[3] + yv[2] + yv[6] + yv[7]));
        dzv = -0.25 * ((zv[0] + zv[1] + zv[5] + zv[4]) - (zv[3] + zv[2] + zv[6] + zv[7]));
        d->delv_eta[i] = ax * dxv + ay * dyv + az * dzv;
    }
}

/* Limiter phi for one direction (lulesh.cc:1464-1531 for xi; eta and zeta
 * repeat it). mask_m/mask_p select the face's BC bits, nm/np the neighbours. */
static inline double limiter(const double* delv_dir, int i, int bc, int mask_m, int symm_m,
                             int free_m, int comm_m, int nm, int mask_p, int symm_p, int free_p,
                             int comm_p, int np, double ptiny, double mult, double max_slope) {
    double norm = 1. / (delv_dir[i] + ptiny);
    double delvm, delvp;
    int bm = bc & mask_m, bp = bc & mask_p;
    if (bm == comm_m || bm == 0) delvm = delv_dir[nm];
    else if (bm == symm_m) delvm = delv_dir[i];
    else if (bm == free_m) delvm = 0.0;
    else delvm = 0; /* unreachable for well-formed masks (lulesh.cc:1477-1480) */
    if (bp == comm_p || bp == 0) delvp = delv_dir[np];
    else if (bp == symm_p) delvp = delv_dir[i];
    else if (bp == free_p) delvp = 0.0;
    else delvp = 0;
    delvm = delvm * norm;
    delvp = delvp * norm;
    double phi = .5 * (delvm + delvp);
    delvm *= mult;
    delvp *= mult;
    if (delvm < phi) phi = delvm;
    if (delvp < phi) phi = delvp;
    if (phi < 0.) phi = 0.;
    if (phi > max_slope) phi = max_slope;
    return phi;
}

/* Pressure from the gamma-law EOS for one element
 * (CalcPressureForElemsTask lulesh.cc:1671-1690). */
static inline void eos_pressure(double* p_new, double* bvc, double* pbvc, double e, double comp,
                                double vnewc, double pmin, double p_cut, double eosvmax) {
    const double cls = 2.0 / 3.0;
    *bvc = cls * (comp + 1.0);
    *pbvc = cls;
    double nv = *bvc * e;
    if (fabs(nv) < p_cut || vnewc >= eosvmax) nv = 0.0;
    if (nv < pmin) nv = pmin;
    *p_new = nv;
}

static inline double sound_speed_sq_guard(double ssc) {
    return (ssc <= .1111111e-36) ? .3333333e-18 : sqrt(ssc);
}

/* Number of EOS evaluations for region reg (lulesh.cc:2156-2170). */
static int region_rep(const lo_domain* d, int reg) {
    if (reg < d->numReg / 2) return 1;
    if (reg < (d->numReg - (d->numReg + 15) / 20)) return 1 + d->cost;
    return 10 * (1 + d->cost);
}

/* Material phase for every element: monotonic-Q limiter and q terms
 * (lulesh.cc:1420-1669), rep evaluations of the EOS (EvalEOSAllInOneTask
 * lulesh.cc:1692-1871, each from the same saved state), sound speed and the
 * save of p, e, q (lulesh.cc:1873-1924). */
static void phase_material(lo_domain* d) {
    const double ptiny = 1.e-36;
    const double mult = d->monoq_limiter_mult, max_slope = d->monoq_max_slope;
    const double qlc = d->qlc_monoq, qqc = d->qqc_monoq;
    const double eosvmin = d->eosvmin, eosvmax = d->eosvmax;
    const double emin = d->emin, pmin = d->pmin, p_cut = d->p_cut, e_cut = d->e_cut,
                 q_cut = d->q_cut, rho0 = d->refdens;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < d->numElem; ++i) {
        int bc = d->elemBC[i];
        double phixi = limiter(d->delv_xi, i, bc, XI_M, XI_M_SYMM, XI_M_FREE, XI_M_COMM,
                               d->lxim[i], XI_P, XI_P_SYMM, XI_P_FREE, XI_P_COMM, d->lxip[i],
                               ptiny, mult, max_slope);
        double phieta = limiter(d->delv_eta, i, bc, ETA_M, ETA_M_SYMM, ETA_M_FREE, ETA_M_COMM,
                                d->letam[i], ETA_P, ETA_P_SYMM, ETA_P_FREE, ETA_P_COMM,
                                d->letap[i], ptiny, mult, max_slope);
        double phizeta = limiter(d->delv_zeta, i, bc, ZETA_M, ZETA_M_SYMM, ZETA_M_FREE,
                                 ZETA_M_COMM, d->lzetam[i], ZETA_P, ZETA_P_SYMM, ZETA_P_FREE,
                                 ZETA_P_COMM, d->lzetap[i], ptiny, mult, max_slope);
        double qlin, qquad;
        if (d->vdov[i] > 0.) {
            qlin = 0.;
            qquad = 0.;
        } else {
            double dxi = d->delv_xi[i] * d->delx_xi[i];
            double deta = d->delv_eta[i] * d->delx_eta[i];
            double dzeta = d->delv_zeta[i] * d->delx_zeta[i];
            if (dxi > 0.) dxi = 0.;
            if (deta > 0.) deta = 0.;
            if (dzeta > 0.) dzeta = 0.;
            double rho = d->elemMass[i] / (d->volo[i] * d->vnew[i]);
            qlin = -qlc * rho *
                   (dxi * (1. - phixi) + deta * (1. - phieta) + dzeta * (1. - phizeta));
            qquad = qqc * rho *
                    (dxi * dxi * (1. - phixi * phixi) + deta * deta * (1. - phieta * phieta) +
                     dzeta * dzeta * (1. - phizeta * phizeta));
        }
        d->qq[i] = qquad;
        d->ql[i] = qlin;

        double vnewc = d->vnew[i];
        if (eosvmin != 0.0 && vnewc < eosvmin) vnewc = eosvmin;
        if (eosvmax != 0.0 && vnewc > eosvmax) vnewc = eosvmax;

        int rep = region_rep(d, d->regNumList[i] - 1);
        double e_new = 0, p_new = 0, q_new = 0, bvc = 0, pbvc = 0;
        for (int r = 0; r < rep; ++r) {
            /* EvalEOSInit (lulesh.cc:1718-1749) */
            double e_old = d->e[i], delvc = d->delv[i], p_old = d->p[i], q_old = d->q[i];
            double qq_old = d->qq[i], ql_old = d->ql[i];
            double comp = 1. / vnewc - 1.;
            double vchalf = vnewc - delvc * .5;
            double compHalf = 1. / vchalf - 1.;
            double work = 0;
            if (eosvmin != 0. && vnewc <= eosvmin) compHalf = comp;
            if (eosvmax != 0.0 && vnewc >= eosvmax) {
                p_old = 0.;
                comp = 0.;
                compHalf = 0.;
            }
            /* CalcEnergyForElems, predictor (lulesh.cc:1754-1789) */
            e_new = e_old - 0.5 * delvc * (p_old + q_old) + 0.5 * work;
            if (e_new < emin) e_new = emin;
            double pHalf;
            eos_pressure(&pHalf, &bvc, &pbvc, e_new, compHalf, vnewc, pmin, p_cut, eosvmax);
            double vhalf = 1. / (1. + compHalf);
            if (delvc > 0.) {
                q_new = 0.;
            } else {
                double ssc = (pbvc * e_new + vhalf * vhalf * bvc * pHalf) / rho0;
                ssc = sound_speed_sq_guard(ssc);
                q_new = (ssc * ql_old + qq_old);
            }
            e_new = e_new + 0.5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (pHalf + q_new));
            /* lulesh.cc:1793-1804 */
            e_new = e_new + 0.5 * work;
            if (fabs(e_new) < e_cut) e_new = 0.0;
            if (e_new < emin) e_new = emin;
            eos_pressure(&p_new, &bvc, &pbvc, e_new, comp, vnewc, pmin, p_cut, eosvmax);
            /* corrector (lulesh.cc:1812-1841) */
            {
                const double sixth = 1.0 / 6.0;
                double q_tilde;
                if (delvc > 0.) {
                    q_tilde = 0.;
                } else {
                    double ssc = (pbvc * e_new + vnewc * vnewc * bvc * p_new) / rho0;
                    ssc = sound_speed_sq_guard(ssc);
                    q_tilde = (ssc * ql_old + qq_old);
                }
                e_new = e_new - (7.0 * (p_old + q_old) - 8.0 * (pHalf + q_new) + (p_new + q_tilde)) *
                                    delvc * sixth;
                if (fabs(e_new) < e_cut) e_new = 0.;
                if (e_new < emin) e_new = emin;
            }
            eos_pressure(&p_new, &bvc, &pbvc, e_new, comp, vnewc, pmin, p_cut, eosvmax);
            /* final q (lulesh.cc:1850-1868) */
            if (delvc <= 0.) {
                double ssc = (pbvc * e_new + vnewc * vnewc * bvc * p_new) / rho0;
                ssc = sound_speed_sq_guard(ssc);
                q_new = (ssc * ql_old + qq_old);
                if (fabs(q_new) < q_cut) q_new = 0.;
            }
        }
        /* CalcSoundSpeedForElemsAndSaveTask (lulesh.cc:1873-1904) */
        double sst = (pbvc * e_new + vnewc * vnewc * bvc * p_new) / rho0;
        d->ss[i] = sound_speed_sq_guard(sst);
        d->p[i] = p_new;
        d->e[i] = e_new;
        d->q[i] = q_new;
    }
}

/* Courant and hydro constraints (lulesh.cc:1938-1974; both start from
 * 1e20 each cycle, lulesh.cc:2214-2215; exact minima). */
static void phase_dt(lo_domain* d) {
    const double qqc2 = 64.0 * d->qqc * d->qqc;
    const double dvovmax = d->dvovmax;
    double dtc = 1.0e+20, dth = 1.0e+20;
#pragma omp parallel for schedule(static) reduction(min : dtc, dth)
    for (int i = 0; i < d->numElem; ++i) {
        double vd = d->vdov[i];
        double c, h;
        if (vd == 0.0) {
            c = DBL_MAX;
            h = DBL_MAX;
        } else {
            double dtf = d->ss[i] * d->ss[i];
            if (vd < 0.0) dtf += qqc2 * d->arealg[i] * d->arealg[i] * vd * vd;
            dtf = sqrt(dtf);
            c = d->arealg[i] / dtf;
            h = dvovmax / (fabs(vd) + 1.e-20);
        }
        if (c < dtc) dtc = c;
        if (h < dth) dth = h;
    }
    d->dtcourant = dtc;
    d->dthydro = dth;
}

int lo_leapfrog(lo_domain* d) {
    int st = phase_forces(d);
    if (st != LO_OK) return st;
    phase_nodes(d);
    st = phase_kinematics(d);
    if (st != LO_OK) return st;
    phase_qgrad(d);
    phase_material(d);
    phase_dt(d);
    return LO_OK;
}

void lo_time_increment(lo_domain* d) {
    double targetdt = d->stoptime - d->time;
    if ((d->dtfixed <= 0.0) && (d->cycle != 0)) {
        double olddt = d->deltatime;
        double gnewdt = 1.0e+20;
        if (d->dtcourant < gnewdt) gnewdt = d->dtcourant / 2.0;
        if (d->dthydro < gnewdt) gnewdt = d->dthydro * 2.0 / 3.0;
        double newdt = gnewdt;
        double ratio = newdt / olddt;
        if (ratio >= 1.0) {
            if (ratio < d->deltatimemultlb) newdt = olddt;
            else if (ratio > d->deltatimemultub) newdt = olddt * d->deltatimemultub;
        }
        if (newdt > d->dtmax) newdt = d->dtmax;
        d->deltatime = newdt;
    }
    if ((targetdt > d->deltatime) && (targetdt < (4.0 * d->deltatime / 3.0)))
        targetdt = 2.0 * d->deltatime / 3.0;
    if (targetdt < d->deltatime) d->deltatime = targetdt;
    d->time += d->deltatime;
    ++d->cycle;
}

int lo_run(lo_domain* d, int max_cycles) {
    while (d->time < d->stoptime && d->cycle < max_cycles) {
        lo_time_increment(d);
        int st = lo_leapfrog(d);
        if (st != LO_OK) return st;
    }
    return LO_OK;
}

/* ------------------------------------------------------------------ */
/* Problem set-up (lulesh-init.cc)                                     */
/* ------------------------------------------------------------------ */

/* Node coordinates and element connectivity of the uniform cube
 * (BuildMesh, lulesh-init.cc:202-252; one domain, so all offsets are 0). */
static void build_mesh(lo_domain* d) {
    const int s = d->s, en = s + 1;
    int n = 0;
    for (int pl = 0; pl < en; ++pl) {
        double tz = 1.125 * (double)pl / (double)s;
        for (int row = 0; row < en; ++row) {
            double ty = 1.125 * (double)row / (double)s;
            for (int col = 0; col < en; ++col) {
                d->x[n] = 1.125 * (double)col / (double)s;
                d->y[n] = ty;
                d->z[n] = tz;
                ++n;
            }
        }
    }
    int e = 0, nb = 0;
    for (int pl = 0; pl < s; ++pl) {
        for (int row = 0; row < s; ++row) {
            for (int col = 0; col < s; ++col) {
                int* ln = &d->nodelist[8 * e];
                ln[0] = nb;
                ln[1] = nb + 1;
                ln[2] = nb + en + 1;
                ln[3] = nb + en;
                ln[4] = nb + en * en;
                ln[5] = nb + en * en + 1;
                ln[6] = nb + en * en + en + 1;
                ln[7] = nb + en * en + en;
                ++e;
                ++nb;
            }
            ++nb;
        }
        nb += en;
    }
}

/* Node -> (8*element + corner) CSR, corners in ascending element order
 * (SetupThreadSupportStructures, lulesh-init.cc:256-310). */
static void build_corner_csr(lo_domain* d) {
    int* count = IALLOC(d->numNode);
    for (int i = 0; i < d->numElem; ++i)
        for (int k = 0; k < 8; ++k) ++count[d->nodelist[8 * i + k]];
    d->nodeElemStart[0] = 0;
    for (int n = 1; n <= d->numNode; ++n) d->nodeElemStart[n] = d->nodeElemStart[n - 1] + count[n - 1];
    memset(count, 0, sizeof(int) * (size_t)d->numNode);
    for (int i = 0; i < d->numElem; ++i)
        for (int k = 0; k < 8; ++k) {
            int m = d->nodelist[8 * i + k];
            d->nodeElemCornerList[d->nodeElemStart[m] + count[m]++] = 8 * i + k;
        }
    free(count);
}

/* Random region assignment (CreateRegionIndexSets, lulesh-init.cc:341-445):
 * runs of elements drawn from glibc rand() after srand(0), region weights
 * (i+1)^balance, never the same region twice in a row. */
static void build_regions(lo_domain* d) {
    const int nr = d->numReg, ne = d->numElem;
    d->regElemSize = IALLOC(nr);
    d->regElemlist = (int**)xcalloc((size_t)nr, sizeof(int*));
    srand(0);
    if (nr == 1) {
        for (int i = 0; i < ne; ++i) d->regNumList[i] = 1;
    } else {
        int* binEnd = IALLOC(nr);
        int costDen = 0;
        for (int i = 0; i < nr; ++i) {
            costDen += pow((i + 1), d->balance);
            binEnd[i] = costDen;
        }
        int next = 0, last = -1;
        while (next < ne) {
            int var = rand() % costDen, i = 0;
            while (var >= binEnd[i]) i++;
            int regionNum = (i % nr) + 1;
            while (regionNum == last) {
                var = rand() % costDen;
                i = 0;
                while (var >= binEnd[i]) i++;
                regionNum = (i % nr) + 1;
            }
            int bin = rand() % 1000, elems;
            if (bin < 773) elems = rand() % 15 + 1;
            else if (bin < 937) elems = rand() % 16 + 16;
            else if (bin < 970) elems = rand() % 32 + 32;
            else if (bin < 974) elems = rand() % 64 + 64;
            else if (bin < 978) elems = rand() % 128 + 128;
            else if (bin < 981) elems = rand() % 256 + 256;
            else elems = rand() % 1537 + 512;
            int runto = elems + next;
            while (next < runto && next < ne) d->regNumList[next++] = regionNum;
            last = regionNum;
        }
        free(binEnd);
    }
    for (int i = 0; i < ne; ++i) d->regElemSize[d->regNumList[i] - 1]++;
    for (int r = 0; r < nr; ++r) {
        d->regElemlist[r] = IALLOC(d->regElemSize[r]);
        d->regElemSize[r] = 0;
    }
    for (int i = 0; i < ne; ++i) {
        int r = d->regNumList[i] - 1;
        d->regElemlist[r][d->regElemSize[r]++] = i;
    }
}

/* Symmetry node sets on the x=0, y=0, z=0 planes (lulesh-init.cc:448-468). */
static void build_symmetry(lo_domain* d) {
    const int en = d->s + 1;
    int n = 0;
    for (int i = 0; i < en; ++i) {
        int planeInc = i * en * en, rowInc = i * en;
        for (int j = 0; j < en; ++j) {
            d->symmZ[n] = rowInc + j;
            d->symmY[n] = planeInc + j;
            d->symmX[n] = planeInc + j * en;
            ++n;
        }
    }
    for (int k = 0; k < d->numSymm; ++k) {
        d->nodeSymm[d->symmX[k]] |= 1;
        d->nodeSymm[d->symmY[k]] |= 2;
        d->nodeSymm[d->symmZ[k]] |= 4;
    }
}

/* Face neighbours (lulesh-init.cc:473-500) and face BCs for a single domain:
 * symmetry on the minus faces, free surface on the plus faces
 * (lulesh-init.cc:503-608). */
static void build_connectivity(lo_domain* d) {
    const int s = d->s, ne = d->numElem;
    d->lxim[0] = 0;
    for (int i = 1; i < ne; ++i) {
        d->lxim[i] = i - 1;
        d->lxip[i - 1] = i;
    }
    d->lxip[ne - 1] = ne - 1;
    for (int i = 0; i < s; ++i) {
        d->letam[i] = i;
        d->letap[ne - s + i] = ne - s + i;
    }
    for (int i = s; i < ne; ++i) {
        d->letam[i] = i - s;
        d->letap[i - s] = i;
    }
    for (int i = 0; i < s * s; ++i) {
        d->lzetam[i] = i;
        d->lzetap[ne - s * s + i] = ne - s * s + i;
    }
    for (int i = s * s; i < ne; ++i) {
        d->lzetam[i] = i - s * s;
        d->lzetap[i - s * s] = i;
    }
    for (int i = 0; i < ne; ++i) d->elemBC[i] = 0;
    for (int i = 0; i < s; ++i) {
        int planeInc = i * s * s, rowInc = i * s;
        for (int j = 0; j < s; ++j) {
            d->elemBC[rowInc + j] |= ZETA_M_SYMM;
            d->elemBC[rowInc + j + ne - s * s] |= ZETA_P_FREE;
            d->elemBC[planeInc + j] |= ETA_M_SYMM;
            d->elemBC[planeInc + j + s * s - s] |= ETA_P_FREE;
            d->elemBC[planeInc + j * s] |= XI_M_SYMM;
            d->elemBC[planeInc + j * s + s - 1] |= XI_P_FREE;
        }
    }
}

lo_domain* lo_create(int s, int nr, int balance, int cost, double energy_scale) {
    if (s < 1 || nr < 1) return NULL;
    lo_domain* d = (lo_domain*)xcalloc(1, sizeof(lo_domain));
    d->s = s;
    d->numElem = s * s * s;
    d->numNode = (s + 1) * (s + 1) * (s + 1);
    d->numReg = nr;
    d->cost = cost;
    d->balance = balance;
    d->numSymm = (s + 1) * (s + 1);
    const int ne = d->numElem, nn = d->numNode;

    d->e_cut = 1.0e-7;
    d->p_cut = 1.0e-7;
    d->q_cut = 1.0e-7;
    d->v_cut = 1.0e-10;
    d->u_cut = 1.0e-7;
    d->hgcoef = 3.0;
    d->ss4o3 = 4.0 / 3.0;
    d->qstop = 1.0e+12;
    d->monoq_max_slope = 1.0;
    d->monoq_limiter_mult = 2.0;
    d->qlc_monoq = 0.5;
    d->qqc_monoq = 2.0 / 3.0;
    d->qqc = 2.0;
    d->eosvmax = 1.0e+9;
    d->eosvmin = 1.0e-9;
    d->pmin = 0.;
    d->emin = -1.0e+15;
    d->dvovmax = 0.1;
    d->refdens = 1.0;

    d->x = DALLOC(nn); d->y = DALLOC(nn); d->z = DALLOC(nn);
    d->xd = DALLOC(nn); d->yd = DALLOC(nn); d->zd = DALLOC(nn);
    d->xdd = DALLOC(nn); d->ydd = DALLOC(nn); d->zdd = DALLOC(nn);
    d->fx = DALLOC(nn); d->fy = DALLOC(nn); d->fz = DALLOC(nn);
    d->nodalMass = DALLOC(nn);
    d->symmX = IALLOC(d->numSymm); d->symmY = IALLOC(d->numSymm); d->symmZ = IALLOC(d->numSymm);
    d->nodeSymm = (unsigned char*)xcalloc((size_t)nn, 1);

    d->nodelist = IALLOC(8L * ne);
    d->lxim = IALLOC(ne); d->lxip = IALLOC(ne); d->letam = IALLOC(ne);
    d->letap = IALLOC(ne); d->lzetam = IALLOC(ne); d->lzetap = IALLOC(ne);
    d->elemBC = IALLOC(ne);
    d->e = DALLOC(ne); d->p = DALLOC(ne); d->q = DALLOC(ne); d->ql = DALLOC(ne);
    d->qq = DALLOC(ne); d->v = DALLOC(ne); d->volo = DALLOC(ne); d->vnew = DALLOC(ne);
    d->delv = DALLOC(ne); d->vdov = DALLOC(ne); d->arealg = DALLOC(ne); d->ss = DALLOC(ne);
    d->elemMass = DALLOC(ne);
    d->delv_xi = DALLOC(ne); d->delv_eta = DALLOC(ne); d->delv_zeta = DALLOC(ne);
    d->delx_xi = DALLOC(ne); d->delx_eta = DALLOC(ne); d->delx_zeta = DALLOC(ne);
    d->fx_stress = DALLOC(8L * ne); d->fy_stress = DALLOC(8L * ne); d->fz_stress = DALLOC(8L * ne);
    d->fx_hg = DALLOC(8L * ne); d->fy_hg = DALLOC(8L * ne); d->fz_hg = DALLOC(8L * ne);
    d->fx_elem = DALLOC(8L * ne); d->fy_elem = DALLOC(8L * ne); d->fz_elem = DALLOC(8L * ne);
    d->nodeElemStart = IALLOC(nn + 1);
    d->nodeElemCornerList = IALLOC(8L * ne);
    d->regNumList = IALLOC(ne);

    for (int i = 0; i < ne; ++i) d->v[i] = 1.0;

    build_mesh(d);
    build_corner_csr(d);
    build_regions(d);
    build_symmetry(d);
    build_connectivity(d);

    d->dtfixed = -1.0e-6;
    d->stoptime = 1.0e-2;
    d->deltatimemultlb = 1.1;
    d->deltatimemultub = 1.2;
    d->dtcourant = 1.0e+20;
    d->dthydro = 1.0e+20;
    d->dtmax = 1.0e-2;
    d->time = 0.;
    d->cycle = 0;

    /* volumes and masses (lulesh-init.cc:148-168) */
    for (int i = 0; i < ne; ++i) {
        double x[8], y[8], z[8];
        const int* nl = &d->nodelist[8 * i];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        double vol = hex_volume(x, y, z);
        d->volo[i] = vol;
        d->elemMass[i] = vol;
        for (int k = 0; k < 8; ++k) d->nodalMass[nl[k]] += vol / 8.0;
    }
    /* energy deposit and initial dt (lulesh-init.cc:170-181) */
    const double ebase = 3.948746e+7;
    double scale = (s * 1) / 45.0;
    double einit = ebase * scale * scale * scale;
    if (energy_scale != 1.0) einit = einit * energy_scale;
    d->e[0] = einit;
    d->deltatime = (.5 * cbrt(d->volo[0])) / sqrt(2.0 * einit);
    return d;
}

void lo_destroy(lo_domain* d) {
    if (!d) return;
    double* dd[] = {d->x, d->y, d->z, d->xd, d->yd, d->zd, d->xdd, d->ydd, d->zdd, d->fx, d->fy,
                    d->fz, d->nodalMass, d->e, d->p, d->q, d->ql, d->qq, d->v, d->volo, d->vnew,
                    d->delv, d->vdov, d->arealg, d->ss, d->elemMass, d->delv_xi, d->delv_eta,
                    d->delv_zeta, d->delx_xi, d->delx_eta, d->delx_zeta, d->fx_stress,
                    d->fy_stress, d->fz_stress, d->fx_hg, d->fy_hg, d->fz_hg, d->fx_elem,
                    d->fy_elem, d->fz_elem};
    for (size_t k = 0; k < sizeof(dd) / sizeof(dd[0]); ++k) free(dd[k]);
    int* ii[] = {d->symmX, d->symmY, d->symmZ, d->nodelist, d->lxim, d->lxip, d->letam,
                 d->letap, d->lzetam, d->lzetap, d->elemBC, d->nodeElemStart,
                 d->nodeElemCornerList, d->regNumList, d->regElemSize};
    for (size_t k = 0; k < sizeof(ii) / sizeof(ii[0]); ++k) free(ii[k]);
    if (d->regElemlist)
        for (int r = 0; r < d->numReg; ++r) free(d->regElemlist[r]);
    free(d->regElemlist);
    free(d->nodeSymm);
    free(d);
}

/* ------------------------------------------------------------------ */
/* Reporting and access                                                */
/* ------------------------------------------------------------------ */

void lo_symmetry(const lo_domain* d, double out[3]) {
    const int nx = d->s;
    double maxAbs = 0.0, totAbs = 0.0, maxRel = 0.0;
    for (int j = 0; j < nx; ++j)
        for (int k = j + 1; k < nx; ++k) {
            double a = fabs(d->e[j * nx + k] - d->e[k * nx + j]);
            totAbs += a;
            if (maxAbs < a) maxAbs = a;
            double r = fabs(d->e[k * nx + j]) > 1e-8 ? a / d->e[k * nx + j] : 0.0;
            if (maxRel < r) maxRel = r;
        }
    out[0] = maxAbs;
    out[1] = totAbs;
    out[2] = maxRel;
}

int lo_dump(const lo_domain* d, const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    const char magic[8] = {'L', 'U', 'L', 'E', 'S', 'H', 'D', '1'};
    fwrite(magic, 1, 8, f);
    int hdr[6] = {d->s, d->numElem, d->numNode, d->cycle, d->numReg, 0};
    fwrite(hdr, sizeof(int), 6, f);
    double t[4] = {d->time, d->deltatime, d->dtcourant, d->dthydro};
    fwrite(t, sizeof(double), 4, f);
    const double* na[] = {d->x, d->y, d->z, d->xd, d->yd, d->zd, d->xdd, d->ydd, d->zdd,
                          d->fx, d->fy, d->fz};
    for (int k = 0; k < 12; ++k) fwrite(na[k], sizeof(double), (size_t)d->numNode, f);
    const double* ea[] = {d->e, d->p, d->q, d->ql, d->qq, d->v, d->vnew, d->delv, d->vdov,
                          d->arealg, d->ss};
    for (int k = 0; k < 11; ++k) fwrite(ea[k], sizeof(double), (size_t)d->numElem, f);
    return fclose(f) == 0 ? 0 : -1;
}

void* lo_field(lo_domain* d, const char* name, long* len, int* is_int) {
    const long nn = d->numNode, ne = d->numElem;
    struct {
        const char* n;
        void* p;
        long len;
        int is_int;
    } t[] = {
        {"x", d->x, nn, 0}, {"y", d->y, nn, 0}, {"z", d->z, nn, 0},
        {"xd", d->xd, nn, 0}, {"yd", d->yd, nn, 0}, {"zd", d->zd, nn, 0},
        {"xdd", d->xdd, nn, 0}, {"ydd", d->ydd, nn, 0}, {"zdd", d->zdd, nn, 0},
        {"fx", d->fx, nn, 0}, {"fy", d->fy, nn, 0}, {"fz", d->fz, nn, 0},
        {"nodalMass", d->nodalMass, nn, 0},
        {"e", d->e, ne, 0}, {"p", d->p, ne, 0}, {"q", d->q, ne, 0},
        {"ql", d->ql, ne, 0}, {"qq", d->qq, ne, 0}, {"v", d->v, ne, 0},
        {"volo", d->volo, ne, 0}, {"vnew", d->vnew, ne, 0}, {"delv", d->delv, ne, 0},
        {"vdov", d->vdov, ne, 0}, {"arealg", d->arealg, ne, 0}, {"ss", d->ss, ne, 0},
        {"elemMass", d->elemMass, ne, 0},
        {"delv_xi", d->delv_xi, ne, 0}, {"delv_eta", d->delv_eta, ne, 0},
        {"delv_zeta", d->delv_zeta, ne, 0}, {"delx_xi", d->delx_xi, ne, 0},
        {"delx_eta", d->delx_eta, ne, 0}, {"delx_zeta", d->delx_zeta, ne, 0},
        {"fx_elem", d->fx_elem, 8 * ne, 0}, {"fy_elem", d->fy_elem, 8 * ne, 0},
        {"fz_elem", d->fz_elem, 8 * ne, 0},
        {"nodelist", d->nodelist, 8 * ne, 1}, {"lxim", d->lxim, ne, 1},
        {"lxip", d->lxip, ne, 1}, {"letam", d->letam, ne, 1}, {"letap", d->letap, ne, 1},
        {"lzetam", d->lzetam, ne, 1}, {"lzetap", d->lzetap, ne, 1},
        {"elemBC", d->elemBC, ne, 1}, {"nodeElemStart", d->nodeElemStart, nn + 1, 1},
        {"nodeElemCornerList", d->nodeElemCornerList, 8 * ne, 1},
        {"regNumList", d->regNumList, ne, 1}, {"symmX", d->symmX, d->numSymm, 1},
        {"symmY", d->symmY, d->numSymm, 1}, {"symmZ", d->symmZ, d->numSymm, 1},
        {"regElemSize", d->regElemSize, d->numReg, 1},
    };
    for (size_t k = 0; k < sizeof(t) / sizeof(t[0]); ++k)
        if (strcmp(t[k].n, name) == 0) {
            if (len) *len = t[k].len;
            if (is_int) *is_int = t[k].is_int;
            return t[k].p;
        }
    return NULL;
}

double lo_get_scalar(const lo_domain* d, int which) {
    switch (which) {
        case 0: return d->time;
        case 1: return d->deltatime;
        case 2: return d->dtcourant;
        case 3: return d->dthydro;
        case 4: return d->stoptime;
        case 5: return d->dtmax;
        case 6: return d->dtfixed;
        case 7: return (double)d->cycle;
        default: return NAN;
    }
}

void lo_set_scalar(lo_domain* d, int which, double v) {
    switch (which) {
        case 0: d->time = v; break;
        case 1: d->deltatime = v; break;
        case 2: d->dtcourant = v; break;
        case 3: d->dthydro = v; break;
        case 4: d->stoptime = v; break;
        case 5: d->dtmax = v; break;
        case 6: d->dtfixed = v; break;
        case 7: d->cycle = (int)v; break;
        default: break;
    }
}

int lo_num_elem(const lo_domain* d) { return d->numElem; }
int lo_num_node(const lo_domain* d) { return d->numNode; }
int lo_num_reg(const lo_domain* d) { return d->numReg; }

const int* lo_region(const lo_domain* d, int r, int* size) {
    if (r < 0 || r >= d->numReg) return NULL;
    if (size) *size = d->regElemSize[r];
    return d->regElemlist[r];
}
