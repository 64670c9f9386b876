/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of the reference's finite-difference ERNN cell
 * (Parameter_inversion/Inversion_adam.py:44-307 and
 * Damage_inversion/Inversion_adam.py:100-393) and of the gradient that the
 * reference obtains from autograd (Inversion_adam.py:447).  Only the test
 * suite, the smoke check and bench.py's CPU-baseline leg load it; the CUDA
 * library never links or calls it.
 *
 * Parity status: pinned.  tests/golden/ holds forward histories and autograd
 * gradients produced by importing the reference module itself
 * (tests/golden/make_golden.py), and tests/test_oracle_golden.py checks this
 * file against them in FP32 and FP64.
 *
 * Build: oracle/build_oracle.py (gcc -O2 -fopenmp -shared -fPIC).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MODE_SCALAR 0
#define ORACLE_MODE_DFIELD 1
#define ORACLE_MODE_FIELDS 2
#define ORACLE_RECORD_FIELDS 0
#define ORACLE_RECORD_RECEIVERS 1
#define ORACLE_ERR_INVALID 1
#define ORACLE_ERR_ALLOC 2
/* fixed chunks of the imaging sums (order independent of the thread count) */
#define ORACLE_CHUNKS 64

/* Problem description; mirrors the fields of ErnnProblem that the oracle needs. */
typedef struct {
  int32_t nshots, nx, ny, nt;
  int32_t stride, mode, record, nrec;
  int32_t src_comp, src_bx, src_by;
  int32_t ref_f32_sum; /* 1: form C12 + C66 in float32 as the reference does */
  double h, dt;
} OracleProblem;

static int oracle_check(const OracleProblem* p) {
  if (!p) return ORACLE_ERR_INVALID;
  if (p->nshots < 1 || p->nx < 1 || p->ny < 1 || p->nt < 1 || p->stride < 1)
    return ORACLE_ERR_INVALID;
  if (p->mode < 0 || p->mode > 2 || p->record < 0 || p->record > 1) return ORACLE_ERR_INVALID;
  if (p->record == ORACLE_RECORD_RECEIVERS && p->nrec < 1) return ORACLE_ERR_INVALID;
  if (p->src_comp < 0 || p->src_comp > 1 || p->src_bx < 0 || p->src_by < 0)
    return ORACLE_ERR_INVALID;
  if (!(p->h > 0.0) || !(p->dt > 0.0)) return ORACLE_ERR_INVALID;
  return 0;
}

#define REAL float
#define FN(x) x##_f32
#include "ernn_oracle_impl.h"
#undef REAL
#undef FN

#define REAL double
#define FN(x) x##_f64
#include "ernn_oracle_impl.h"
#undef REAL
#undef FN

int oracle_abi_version(void) { return 1; }
