/*
 * gbfir_oracle.c — CPU oracle for the direct-FIR path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of MatX's HostExecutor
 * algorithms (conv1d/corr direct, resample_poly, channelize_poly), used by the
 * tests as the checker and by bench.py as the timed CPU baseline.  The CUDA
 * product never links or calls this file.
 *
 * Built with -ffp-contract=off so that x86-64 and aarch64 hosts round every
 * product and sum the same way (no fused multiply-add contraction).
 * The double instantiation is the FP64 oracle; the float one follows the
 * reference's FP32 host arithmetic step by step.
 * Parity pins: tests/test_oracle.py checks both against the reference's own
 * golden vectors (tests/golden/) and, where MatX compiles here, against MatX's
 * HostExecutor run on the same inputs.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define T double
#define SUF _d
#include "oracle_impl.h"
#undef T
#undef SUF

#define T float
#define SUF _f
#include "oracle_impl.h"
#undef T
#undef SUF

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
