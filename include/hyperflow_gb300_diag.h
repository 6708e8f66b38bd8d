/* HyperFlow-GB300 -- self-test entry points of the device arithmetic.  No counterpart in the
 * reference; they check that the kernels' own arithmetic reproduces IEEE results, which is
 * what keeps the GPU path bit-identical to the reference. */
#ifndef HYPERFLOW_GB300_DIAG_H
#define HYPERFLOW_GB300_DIAG_H

#include <stdint.h>

#include "hyperflow_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Compares the kernels' integer-pipe FP64 division and square root with the hardware IEEE
 * operations on n generated operands: division modes 0 raw bit patterns, 1 normal operands,
 * 2 near-halfway quotients, 3 short mantissas, 4 operands near the range limits; square-root
 * modes 5 raw bit patterns, 6 every normal exponent, 7 near-squares.  Writes the number of
 * bitwise mismatches and the first mismatching (a, b, got, want). */
int hf_diag_div_check(uint64_t seed, int64_t n, int mode, int64_t* mismatches, double* first4);

#ifdef __cplusplus
}
#endif
#endif
