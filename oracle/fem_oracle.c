/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of the reference's FEM data generator time loop
 * (Parameter_inversion/FEM_generate_data.py), the step before the ERNN path:
 *   :117-185  structured triangular mesh, checkerboard diagonals, node id
 *             j*nx + i (x index fastest), boundary = the four edges
 *   :330-342  lumped mass: every element adds rho * (dx dy / 2) / 3 to each
 *             of its three nodes
 *   :345-384  per-element Jacobian J = [[x1-x0, x2-x0], [y1-y0, y2-y0]],
 *             |det J|, J^-1 (constant-strain triangles)
 *   :417-457  internal force: three Gauss points of weight 1/6 (all with the
 *             same constant B), strain, anisotropic stress, element forces
 *             scattered to the nodes
 *   :474-499  central differences with the lumped mass, external load
 *             (Ricker(t_n) * gaussian / rho) * M on the y component, edge
 *             nodes forced to zero after every step
 * Output frames are scaled by `out_scale` (0.7 at :525-526) and laid out as
 * the generator saves them, (frame, i, j) with j (y) fastest; frame k holds
 * time level k * stride (u^0 = u^1 = 0).
 *
 * REAL = float restates the reference's float32 run; REAL = double is the
 * FP64 run of the same scheme.  Parity pinned by tests/golden/fem_*.npz,
 * produced by running the reference function itself (tests/golden/make_golden.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int32_t nx, ny, nt, stride;
  double dx, dy, dt, rho;
  double C[6];      /* C11, C22, C12, C16, C26, C66 */
  double out_scale; /* factor applied to the saved frames */
} OracleFemProblem;

#define FEM_ERR_INVALID 1
#define FEM_ERR_ALLOC 2

#define REAL float
#define FN(x) x##_f32
#include "fem_oracle_impl.h"
#undef REAL
#undef FN

#define REAL double
#define FN(x) x##_f64
#include "fem_oracle_impl.h"
#undef REAL
#undef FN
