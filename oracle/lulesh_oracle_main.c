/* Command-line front end of the CPU oracle (test infrastructure).
 *
 * Accepts the reference's flags (lulesh.cc:2421-2432): --s --r --i --b --c
 * --q --p, plus --threads N (the reference's --hpx:threads=N is accepted as
 * well). Without --q it prints the same full-precision RESULT line as the
 * reference oracle binary (oracle/ref_report.cc); with --q it prints the
 * reference's CSV line "s,regions,cycles,threads,elapsed,e0"
 * (lulesh.cc:2405-2407). LULESH_DUMP=<file> writes the final field dump.
 */
#define _POSIX_C_SOURCE 199309L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "lulesh_oracle.h"

static double now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char** argv) {
    int its = 9999999, s = 30, nr = 11, b = 1, c = 1, quiet = 0, prog = 0, threads = 0;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        const char* val = NULL;
        if (strncmp(a, "--hpx:threads=", 14) == 0) {
            threads = atoi(a + 14);
            continue;
        }
        if (!strcmp(a, "--q")) { quiet = 1; continue; }
        if (!strcmp(a, "--p")) { prog = 1; continue; }
        if (i + 1 < argc) val = argv[i + 1];
        if (!val) { fprintf(stderr, "missing value for %s\n", a); return 1; }
        if (!strcmp(a, "--s")) s = atoi(val);
        else if (!strcmp(a, "--r")) nr = atoi(val);
        else if (!strcmp(a, "--i")) its = atoi(val);
        else if (!strcmp(a, "--b")) b = atoi(val);
        else if (!strcmp(a, "--c")) c = atoi(val);
        else if (!strcmp(a, "--threads")) threads = atoi(val);
        else { fprintf(stderr, "unknown option %s\n", a); return 1; }
        ++i;
    }
    if (threads > 0) lo_set_threads(threads);
    lo_domain* d = lo_create(s, nr, b, c, 1.0);
    if (!d) { fprintf(stderr, "bad problem size\n"); return 1; }
    double t0 = now();
    int st = LO_OK;
    while (lo_get_scalar(d, 0) < lo_get_scalar(d, 4) && (int)lo_get_scalar(d, 7) < its) {
        lo_time_increment(d);
        st = lo_leapfrog(d);
        if (st != LO_OK) break;
        int cyc = (int)lo_get_scalar(d, 7);
        if (prog && !quiet && cyc % 100 == 0)
            printf("cycle = %d, time = %e, dt=%e\n", cyc, lo_get_scalar(d, 0), lo_get_scalar(d, 1));
    }
    double elapsed = now() - t0;
    if (st != LO_OK) {
        fprintf(stderr, "VolumeError\n");
        lo_destroy(d);
        return -1 & 0xff;
    }
    long ne = lo_num_elem(d);
    int cycles = (int)lo_get_scalar(d, 7);
    long ecount = 0;
    int is_int = 0;
    double* e = (double*)lo_field(d, "e", &ecount, &is_int);
    if (quiet) {
        printf("%d,%d,%d,%d,%g,%.6e\n", s, nr, cycles, lo_get_threads(), elapsed, e[0]);
    } else {
        double sym[3];
        lo_symmetry(d, sym);
        double grind = cycles ? (elapsed * 1e6 / cycles) / (double)ne : 0.0;
        printf("RESULT s=%d cycles=%d e0=%.17e maxabs=%.17e totabs=%.17e maxrel=%.17e "
               "elapsed=%.6f grind_us=%.6f time=%.17e dt=%.17e\n",
               s, cycles, e[0], sym[0], sym[1], sym[2], elapsed, grind, lo_get_scalar(d, 0),
               lo_get_scalar(d, 1));
    }
    const char* dump = getenv("LULESH_DUMP");
    if (dump && lo_dump(d, dump) != 0) fprintf(stderr, "dump failed: %s\n", dump);
    lo_destroy(d);
    return 0;
}
