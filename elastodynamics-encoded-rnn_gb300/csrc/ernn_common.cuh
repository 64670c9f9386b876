// Shared device-side definitions of the ERNN propagation library.
//
// Notation used across the kernels (cell (i, j) = row i along x, column j
// along y; y is contiguous in memory, as in the reference's (1, nx, ny)
// tensors):
//   sxx(u) = u[i-1,j] - 2u[i,j] + u[i+1,j]                    (h^2 d2/dx2)
//   syy(u) = u[i,j-1] - 2u[i,j] + u[i,j+1]                    (h^2 d2/dy2)
//   sxy(u) = u[i+1,j+1] + u[i-1,j-1] - u[i+1,j-1] - u[i-1,j+1] (4h^2 d2/dxdy)
// with u = 0 outside the grid (the zero-padded convolutions of
// Parameter_inversion/Inversion_adam.py:44-51).  With q = dt^2 / (rho h^2)
// one leapfrog step of Inversion_adam.py:86-104, 286-287 is
//   u^{n+1} = 2u^n - u^{n-1} + Lq(u^n) + (dt^2/rho) f^n
//   Lq_x = k11 sxx(ux) + k66 syy(ux) + kq12 sxy(uy) + k16h sxy(ux) + k16 sxx(uy) + k26 syy(uy)
//   Lq_y = k66 sxx(uy) + k22 syy(uy) + kq12 sxy(ux) + k16 sxx(ux) + k26 syy(ux) + k26h sxy(uy)
// where k_t = C_t q, k16h = C16 q/2, k26h = C26 q/2, kq12 = (C12 + C66) q/4.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ernn {

constexpr int kModeScalar = 0;
constexpr int kModeDField = 1;
constexpr int kModeFields = 2;
constexpr int kRecordFields = 0;
constexpr int kRecordReceivers = 1;

// Coefficients computed once per call on the device (no host round trip).
struct Coef {
  float k11, k22, kq12, k16, k26, k66, k16h, k26h;  // scalar (or C0) constants times q
  float kappa;   // dt^2 / rho, multiplies the force
  float q;       // dt^2 / (rho h^2)
  float gscale;  // power-of-two scale applied to the adjoint source
  float pad0;
  double qd;         // q in double
  double inv_gscale; // 1 / gscale in double
  uint32_t gmax_bits; // max |g| (non-negative float bits, atomicMax-able)
  int err;            // device-side error word (ERNN_ERR_TIMEOUT from a bounded wait)
  double pad2;
};

// Spin limit of every device-side wait on an mbarrier (about a second at the
// part's clocks).  A wait that runs out records kDeviceTimeout in the call's
// error word and returns; later waits of the launch return at once.
constexpr long long kWaitLimitCycles = 1ll << 31;
constexpr int kDeviceTimeout = 5;  // ERNN_ERR_TIMEOUT

// Programmatic dependent launch.  A step kernel launched with the
// programmatic-serialisation attribute may be scheduled while the previous
// kernel of its stream still runs.  Every step kernel lets its dependents
// launch as it starts (grid_dep_trigger: they are only scheduled once every
// block of this grid has started, so they never take the place of one), loads
// what no step kernel writes (coefficients, constant planes, source maps,
// receiver tables, tensor maps), and then waits in grid_dep_wait until the
// previous grid has completed and its writes are visible, before it reads or
// writes any state.  Without the attribute both are no-ops.
__device__ __forceinline__ void grid_dep_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Tile geometry of the per-step kernels: 32 rows (x) by 32 columns (y),
// 256 threads as 8 row groups of one warp each; a thread owns 4 cells of
// one column.
constexpr int TX = 32;
constexpr int TY = 32;
constexpr int HX = TX + 2;
constexpr int HY = TY + 2;
constexpr int NTHR = 256;
constexpr int RPT = TX / (NTHR / TY);  // rows per thread = 4

}  // namespace ernn
