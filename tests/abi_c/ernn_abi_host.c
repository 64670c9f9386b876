/* Host-side use of the C ABI from plain C99 (no CUDA headers, no device
 * calls): the header compiles as C, the library links, and validation, size
 * queries, the stability check and the error strings behave as ernn.h
 * documents.  Prints "ok" and exits 0, or names the first failed check. */
#include <stdio.h>
#include <string.h>

#include "ernn.h"

#define CHECK(cond)                                          \
  do {                                                       \
    if (!(cond)) {                                           \
      fprintf(stderr, "failed: %s (line %d)\n", #cond, __LINE__); \
      return 1;                                              \
    }                                                        \
  } while (0)

int main(void) {
  CHECK(ernn_abi_version() == ERNN_ABI_VERSION);

  /* the calling sequence's problem: rot256 with 64 receivers, checkpoint 100 */
  ErnnProblem p;
  memset(&p, 0, sizeof(p));
  p.nshots = 1; p.nx = 256; p.ny = 256; p.nt = 2000; p.stride = 1;
  p.mode = ERNN_MODE_SCALAR; p.record = ERNN_RECORD_RECEIVERS; p.nrec = 64;
  p.src_comp = 1; p.src_bx = 9; p.src_by = 9; p.ckpt_k = 100;
  p.path = ERNN_PATH_AUTO; p.flags = 0; p.h = 1e-4; p.dt = 5e-9;
  CHECK(ernn_validate(&p) == ERNN_OK);
  const size_t state = (size_t)2 * 256 * 256 * sizeof(float);
  const size_t tape = ernn_tape_bytes(&p, 1), notape = ernn_tape_bytes(&p, 0);
  CHECK(notape >= 2 * state);                  /* two working levels */
  CHECK(tape >= notape + (size_t)(2000 / 100 - 1) * 2 * state);  /* checkpoint pairs */
  CHECK(ernn_adjoint_scratch_bytes(&p) >= 2 * state);

  /* refused problems: an error code and size queries of 0 */
  ErnnProblem bad = p;
  bad.stride = 0;
  CHECK(ernn_validate(&bad) == ERNN_ERR_INVALID);
  CHECK(ernn_tape_bytes(&bad, 1) == 0 && ernn_adjoint_scratch_bytes(&bad) == 0);
  bad = p;
  bad.nshots = 65535; bad.nx = 46340; bad.ny = 46340; bad.nt = 1 << 30; bad.ckpt_k = 1 << 30;
  CHECK(ernn_validate(&bad) == ERNN_ERR_INVALID);  /* sizes past 64 bits */
  CHECK(ernn_tape_bytes(&bad, 1) == 0);
  CHECK(ernn_validate(NULL) == ERNN_ERR_INVALID);

  /* leapfrog stability, host pointers: an orthotropic plate at dt = 5 ns is
   * stable, the same at 50 ns is not */
  const double C6[6] = {130e9, 12e9, 6e9, 0.0, 0.0, 5.5e9};
  double courant = -1.0;
  CHECK(ernn_check_stability(C6, 1560.0, 1e-4, 5e-9, &courant) == ERNN_OK);
  CHECK(courant > 0.0 && courant <= 1.0);
  CHECK(ernn_check_stability(C6, 1560.0, 1e-4, 5e-8, &courant) == ERNN_ERR_UNSTABLE);
  CHECK(courant > 1.0);

  for (int code = ERNN_OK; code <= ERNN_ERR_UNSUPPORTED; ++code) {
    const char* s = ernn_error_string(code);
    CHECK(s != NULL && s[0] != '\0');
  }
  printf("ok\n");
  return 0;
}
