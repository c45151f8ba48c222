/* lulesh_probe.h - measurement probes of the GB300 LULESH library.
 *
 * Not part of the step's C ABI (include/lulesh_gb300.h): these entry points
 * live in their own library, liblulesh_probe.so, which only the benchmark
 * and the accuracy tests load. The product library does not contain them.
 */
#ifndef LULESH_PROBE_H
#define LULESH_PROBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Measures the current GPU's pipe rates: out[0] double FMA/s, out[1] double
 * add/s, out[2] double divide/s, out[3] double square root/s, out[4] float
 * FMA/s, out[5] double multiplies/s on the FP64 pipe, out[6] the same on the
 * integer pipes (the step's dmul_ipipe), out[7] both at once (half of the
 * chains each), out[8] double adds/s on the integer pipes (dadd_ipipe),
 * out[9] adds on both at once; per-thread operations. The double path is
 * bound by out[0]; takes about 80 ms. Returns 0 or a LULESH_* status. */
int lulesh_probe_pipe_rates(double out[10]);

/* Evaluates one arithmetic helper of the fast variants on the device for n
 * inputs (accuracy tests compare the results with correctly rounded host
 * values): fn 0 reciprocal, 1 reciprocal cube root, 2 square root, 3
 * reciprocal square root (inputs positive and normal for 1-3), 4 the
 * hardware seed of the reciprocal; 5 the mixed variant's double-to-float
 * rounding, 6 and 7 the high and low floats of its float-pair split (results
 * returned as doubles). n <= 2^26. */
int lulesh_probe_math(int32_t fn, const double* in, double* out, int64_t n);

/* The double product of a[i] and b[i] for n pairs, by the FP64 pipe's
 * multiply (native) and by the step's integer-pipe multiply (ipipe, which
 * must give the same bits). n <= 2^26. */
int lulesh_probe_dmul(const double* a, const double* b, double* native, double* ipipe, int64_t n);

/* The double sum of a[i] and b[i] for n pairs, by the FP64 pipe's add
 * (native) and by an integer-pipe add (dadd_ipipe, which must give the same
 * bits; measured slower than the FP64 pipe's, so no step kernel uses it).
 * n <= 2^26. */
int lulesh_probe_dadd(const double* a, const double* b, double* native, double* ipipe, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
