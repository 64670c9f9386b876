// Device kernels of the ERNN propagation library (sm_103a).
//
// fwd_step_kernel  one fused leapfrog step: stencils, constants, force
//                  injection, update, history/checkpoint stores and the
//                  receiver gather, one pass over the state.
// adj_step_kernel  one reverse-time adjoint step fused with the imaging
//                  condition (gradient of the constants) and the adjoint
//                  source injection.
// The notation (sxx, syy, sxy, k11 ... kq12, q, kappa) is defined in
// ernn_common.cuh.
#include <atomic>
#include <functional>
#include <utility>
#include <vector>

#include "ernn_launch.h"

namespace ernn {

static std::atomic<uint64_t> g_launches{0};
uint64_t launches() { return g_launches.load(std::memory_order_relaxed); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Diagnostic timing: CUDA events recorded on the launch stream around every
// launch of a kernel class while enabled.  Host-side, single-threaded use.
namespace {
struct Profiler {
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool[kProfClasses];
  size_t used[kProfClasses] = {0, 0, 0};
  double alg_bytes[kProfClasses] = {0.0, 0.0, 0.0};
};
Profiler g_prof;
}  // namespace

static std::atomic<bool> g_overlap{true};
bool launch_overlap() { return g_overlap.load(std::memory_order_relaxed) && !g_prof.on; }
bool launch_overlap_setting() { return g_overlap.load(std::memory_order_relaxed); }
void set_launch_overlap(bool on) { g_overlap.store(on, std::memory_order_relaxed); }

void profile_enable(bool on) {
  g_prof.on = on;
  for (int c = 0; c < kProfClasses; ++c) {
    g_prof.used[c] = 0;
    g_prof.alg_bytes[c] = 0.0;
  }
}

cudaError_t profile_read(double* ms, uint64_t* count, double* alg_bytes) {
  for (int c = 0; c < kProfClasses; ++c) {
    double total = 0.0;
    for (size_t i = 0; i < g_prof.used[c]; ++i) {
      float t = 0.f;
      cudaError_t e = cudaEventSynchronize(g_prof.pool[c][i].second);
      if (e != cudaSuccess) return e;
      e = cudaEventElapsedTime(&t, g_prof.pool[c][i].first, g_prof.pool[c][i].second);
      if (e != cudaSuccess) return e;
      total += t;
    }
    if (ms) ms[c] = total;
    if (count) count[c] = g_prof.used[c];
    if (alg_bytes) alg_bytes[c] = g_prof.alg_bytes[c];
  }
  return cudaSuccess;
}

// Launch `fn` (which enqueues one kernel on st), counting it and, while the
// profiler is on, bracketing it with events of class `cls`.
template <class Fn>
static cudaError_t tracked(int cls, cudaStream_t st, Fn&& fn, double alg_bytes = 0.0) {
  if (g_prof.on) {
    g_prof.alg_bytes[cls] += alg_bytes;
    auto& pool = g_prof.pool[cls];
    if (g_prof.used[cls] == pool.size()) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
        return cudaGetLastError();
      pool.emplace_back(a, b);
    }
    auto& ev = pool[g_prof.used[cls]++];
    cudaEventRecord(ev.first, st);
    fn();
    cudaEventRecord(ev.second, st);
  } else {
    fn();
  }
  count_launch();
  return cudaGetLastError();
}

// Tile height of the plain per-step kernels: 32 rows (4 per thread), or 8
// rows (1 per thread) when a step has fewer than 512 tiles of 32 x 32 — four
// times the warps for small grids, whose steps are latency bound.
int step_rows(int nx, int ny, int S) {
  const long long tiles32 = (long long)S * ((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
  return tiles32 < 512 ? 8 : TX;
}

dim3 step_grid(int nx, int ny, int S) {
  const int rows = step_rows(nx, ny, S);
  return dim3((unsigned)((ny + TY - 1) / TY), (unsigned)((nx + rows - 1) / rows), (unsigned)S);
}

cudaError_t tracked_launch(int cls, cudaStream_t st, const std::function<void()>& fn,
                           double alg_bytes) {
  return tracked(cls, st, fn, alg_bytes);
}

// --------------------------------------------------------------------------
// Coefficients.  The constants arrive as float32 device scalars (the
// reference's clamped exp(log C) tensors); C12 + C66 is formed in float32 as
// the reference forms it from float32 tensors (Inversion_adam.py:88).
// One block per coefficient block: block b reads C[6b..6b+5] and rho[b]
// (one block, or one per shot with per-shot constants).
__global__ void coef_kernel(int mode, const float* __restrict__ C, const float* __restrict__ rho,
                            double h, double dt, Coef* __restrict__ out) {
  if (threadIdx.x != 0) return;
  const int b = blockIdx.x;
  C += 6 * b;
  Coef c;
  const double r = (double)rho[b];
  const double q = dt * dt / (r * h * h);
  c.k11 = c.k22 = c.kq12 = c.k16 = c.k26 = c.k66 = c.k16h = c.k26h = 0.f;
  if (mode != kModeFields) {
    const float c1266 = C[2] + C[5];
    c.k11 = (float)((double)C[0] * q);
    c.k22 = (float)((double)C[1] * q);
    c.kq12 = (float)((double)c1266 * q * 0.25);
    c.k16 = (float)((double)C[3] * q);
    c.k26 = (float)((double)C[4] * q);
    c.k66 = (float)((double)C[5] * q);
    c.k16h = (float)((double)C[3] * q * 0.5);
    c.k26h = (float)((double)C[4] * q * 0.5);
  }
  c.kappa = (float)(dt * dt / r);
  c.q = (float)q;
  c.gscale = 1.f;
  c.pad0 = 0.f;
  c.qd = q;
  c.inv_gscale = 1.0;
  c.gmax_bits = 0u;
  c.err = 0;
  c.pad2 = 0.0;
  out[b] = c;
}

// Scalar-constant operator on a staged tile, Lq of ernn_common.cuh.
struct KS {
  float k11, k22, kq12, k16, k26, k66, k16h, k26h;
};

__device__ __forceinline__ KS load_ks(const Coef* c) {
  KS k;
  k.k11 = c->k11; k.k22 = c->k22; k.kq12 = c->kq12; k.k16 = c->k16;
  k.k26 = c->k26; k.k66 = c->k66; k.k16h = c->k16h; k.k26h = c->k26h;
  return k;
}

// Per-cell constants of FIELDS mode (C11, C22, C12, C16, C26, C66 of one
// cell), scaled by q.
__device__ __forceinline__ KS cell_ks(const float c[6], float q) {
  const float C11 = c[0], C22 = c[1], C12 = c[2], C16 = c[3], C26 = c[4], C66 = c[5];
  KS k;
  k.k11 = C11 * q; k.k22 = C22 * q; k.k66 = C66 * q;
  k.k16 = C16 * q; k.k26 = C26 * q;
  k.k16h = 0.5f * k.k16; k.k26h = 0.5f * k.k26;
  k.kq12 = (C12 + C66) * q * 0.25f;
  return k;
}

struct Sten {
  float cx, cy;                          // centre values
  float xx_x, yy_x, xy_x, xx_y, yy_y, xy_y;  // sxx, syy, sxy of ux and uy
};

// The six stencil sums at tile position (r, c) (centre at s[r+1][c+1]).
__device__ __forceinline__ Sten stencils(const float (*sx)[HY], const float (*sy)[HY], int r, int c) {
  Sten s;
  s.cx = sx[r + 1][c + 1];
  s.cy = sy[r + 1][c + 1];
  s.xx_x = (sx[r][c + 1] + sx[r + 2][c + 1]) - 2.f * s.cx;
  s.yy_x = (sx[r + 1][c] + sx[r + 1][c + 2]) - 2.f * s.cx;
  s.xy_x = (sx[r + 2][c + 2] + sx[r][c]) - (sx[r + 2][c] + sx[r][c + 2]);
  s.xx_y = (sy[r][c + 1] + sy[r + 2][c + 1]) - 2.f * s.cy;
  s.yy_y = (sy[r + 1][c] + sy[r + 1][c + 2]) - 2.f * s.cy;
  s.xy_y = (sy[r + 2][c + 2] + sy[r][c]) - (sy[r + 2][c] + sy[r][c + 2]);
  return s;
}

__device__ __forceinline__ void apply_ks(const KS& k, const Sten& s, float& lx, float& ly) {
  lx = k.k11 * s.xx_x + k.k66 * s.yy_x + k.kq12 * s.xy_y + k.k16h * s.xy_x + k.k16 * s.xx_y +
       k.k26 * s.yy_y;
  ly = k.k66 * s.xx_y + k.k22 * s.yy_y + k.kq12 * s.xy_x + k.k16 * s.xx_x + k.k26 * s.yy_x +
       k.k26h * s.xy_y;
}

// Stage rows x0-1 .. x0+T and columns y0-1 .. y0+TY of both components of
// a [comp][cell] state into shared memory, zero outside the grid.
template <int T>
__device__ __forceinline__ void stage_pair(float (*sx)[HY], float (*sy)[HY],
                                           const float* __restrict__ base, int nx, int ny,
                                           size_t N, int x0, int y0, int tid) {
  for (int e = tid; e < (T + 2) * HY; e += NTHR) {
    const int r = e / HY, c = e - r * HY;
    const int gi = x0 + r - 1, gj = y0 + c - 1;
    float vx = 0.f, vy = 0.f;
    if (base != nullptr && gi >= 0 && gi < nx && gj >= 0 && gj < ny) {
      const size_t o = (size_t)gi * ny + gj;
      vx = base[o];
      vy = base[N + o];
    }
    sx[r][c] = vx;
    sy[r][c] = vy;
  }
}

// --------------------------------------------------------------------------
template <int MODE, int T>
__global__ void __launch_bounds__(NTHR) fwd_step_kernel(const FwdStep a) {
  constexpr int RPT_ = T / (NTHR / TY);  // rows per thread
  __shared__ float sx[T + 2][HY];
  __shared__ float sy[T + 2][HY];
  grid_dep_trigger();
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TY + tx;
  const int y0 = blockIdx.x * TY, x0 = blockIdx.y * T, s = blockIdx.z;
  const int nx = a.nx, ny = a.ny;
  const size_t N = (size_t)nx * ny;

  // Inputs no step writes, loaded before the wait (a chained launch loads
  // them while the previous step runs): coefficients, source, and the
  // per-cell constants of the thread's cells (FIELDS: the six planes;
  // DFIELD: 1 - D).
  const Coef* K = a.coef + (size_t)s * a.coef_stride;
  const float amp = a.src_signal[(size_t)s * a.nt + a.i] * K->kappa;
  const bool has_src = a.bx > 0 && a.by > 0;
  const int ox = has_src ? a.src_origin[2 * s] : 0, oy = has_src ? a.src_origin[2 * s + 1] : 0;
  KS ks;
  if (MODE != kModeFields) ks = load_ks(K);
  const float q = K->q;
  const int gj = y0 + tx;
  float cf[RPT_][MODE == kModeFields ? 6 : 1];
  if (MODE != kModeScalar) {
#pragma unroll
    for (int k = 0; k < RPT_; ++k) {
      const int gi = x0 + ty + (NTHR / TY) * k;
      const bool in = gi < nx && gj < ny;
      const size_t o = in ? (size_t)gi * ny + gj : 0;
      if (MODE == kModeFields) {
#pragma unroll
        for (int c = 0; c < 6; ++c) cf[k][c] = in ? a.field[c * N + o] : 0.f;
      } else {
        cf[k][0] = in ? 1.f - a.field[o] : 0.f;
      }
    }
  }
  grid_dep_wait();

  // the own cells of u^{i-1}, issued with the staging loads (one memory
  // round before the barrier instead of a second one after it)
  const float* prev = a.prev ? a.prev + (size_t)s * 2 * N : nullptr;
  float pxv[RPT_], pyv[RPT_];
#pragma unroll
  for (int k = 0; k < RPT_; ++k) {
    const int gi = x0 + ty + (NTHR / TY) * k;
    const bool in = prev != nullptr && gi < nx && gj < ny;
    const size_t o = in ? (size_t)gi * ny + gj : 0;
    pxv[k] = in ? prev[o] : 0.f;
    pyv[k] = in ? prev[N + o] : 0.f;
  }
  const float* cur = a.cur ? a.cur + (size_t)s * 2 * N : nullptr;
  stage_pair<T>(sx, sy, cur, nx, ny, N, x0, y0, tid);

  // Receiver gather of the input state u^i, folded into this launch.
  if (a.gframe >= 0 && blockIdx.x == 0 && blockIdx.y == 0) {
    for (int r = tid; r < a.nrec; r += NTHR) {
      const int32_t idx = a.rec_idx[(size_t)s * a.nrec + r];
      const size_t o = ((size_t)s * a.nt_out + a.gframe) * a.nrec + r;
      const bool ok = cur != nullptr && idx >= 0 && (size_t)idx < N;  // out of range: 0
      a.tr_x[o] = ok ? cur[idx] : 0.f;
      a.tr_y[o] = ok ? cur[N + idx] : 0.f;
    }
  }
  __syncthreads();

  float* out = a.out + (size_t)s * 2 * N;
#pragma unroll
  for (int k = 0; k < RPT_; ++k) {
    const int r = ty + (NTHR / TY) * k;
    const int gi = x0 + r;
    if (gi >= nx || gj >= ny) continue;
    const size_t o = (size_t)gi * ny + gj;
    const Sten st = stencils(sx, sy, r, tx);
    float lx, ly;
    if (MODE == kModeFields) {
      const KS kc = cell_ks(cf[k], q);
      apply_ks(kc, st, lx, ly);
    } else {
      apply_ks(ks, st, lx, ly);
      if (MODE == kModeDField) {
        lx *= cf[k][0];
        ly *= cf[k][0];
      }
    }
    // the load joins the operator sum before the update, as in the
    // reference's (A u + f) / rho: one rounding of the increment into 2 c - p
    const int sa = gi - ox, sb = gj - oy;
    if (has_src && sa >= 0 && sa < a.bx && sb >= 0 && sb < a.by) {
      const float f = a.src_map[((size_t)s * a.bx + sa) * a.by + sb];  // L + amp f, one rounding
      if (a.src_comp == 0) lx = fmaf(amp, f, lx); else ly = fmaf(amp, f, ly);
    }
    const float vx = (2.f * st.cx - pxv[k]) + lx;
    const float vy = (2.f * st.cy - pyv[k]) + ly;
    out[o] = vx;
    out[N + o] = vy;
    if (a.copy0) {
      a.copy0[(size_t)s * 2 * N + o] = vx;
      a.copy0[(size_t)s * 2 * N + N + o] = vy;
    }
    if (a.copy1) {
      a.copy1[(size_t)s * 2 * N + o] = vx;
      a.copy1[(size_t)s * 2 * N + N + o] = vy;
    }
    if (a.frame >= 0) {
      const size_t ho = ((size_t)s * a.nt_out + a.frame) * N + o;
      a.hist_x[ho] = vx;
      a.hist_y[ho] = vy;
    }
  }
}

// --------------------------------------------------------------------------
template <int MODE, int T>
__global__ void __launch_bounds__(NTHR) adj_step_kernel(const AdjStep a) {
  constexpr int NL = (MODE == kModeFields) ? 6 : 2;
  constexpr int RPT_ = T / (NTHR / TY);  // rows per thread
  __shared__ float sl[NL][T + 2][HY];
  __shared__ float su[2][T + 2][HY];
  __shared__ double red[NTHR / 32][6];
  grid_dep_trigger();
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TY + tx;
  const int y0 = blockIdx.x * TY, x0 = blockIdx.y * T, s = blockIdx.z;
  const int nx = a.nx, ny = a.ny;
  const size_t N = (size_t)nx * ny;
  const float* cur = a.cur + (size_t)s * 2 * N;
  const float* um = a.u ? a.u + (size_t)s * 2 * N : nullptr;
  const Coef* K = a.coef + (size_t)s * a.coef_stride;
  const float q = K->q;

  // Stage lam^{m+1} (weighted as A^T needs it) and u^m with a one-cell halo.
  // The per-cell constants of the staged cells are loaded before the wait on
  // 8-row tiles (two staged cells per thread; a chained launch loads them
  // while the previous step runs), inside the staging loop on 32-row tiles.
  constexpr int kStaged = (T + 2) * HY;
  constexpr int kIt = (kStaged + NTHR - 1) / NTHR;
  constexpr bool kPre = MODE != kModeScalar && T == 8;
  constexpr int kNF = MODE == kModeFields ? 6 : 1;
  float fpre[kPre ? kIt : 1][kNF];
  auto staged_field = [&](int e, float f[kNF]) {
    const int r = e / HY, c = e - r * HY;
    const int gi = x0 + r - 1, gj = y0 + c - 1;
    const bool in = e < kStaged && gi >= 0 && gi < nx && gj >= 0 && gj < ny;
    const size_t o = in ? (size_t)gi * ny + gj : 0;
#pragma unroll
    for (int k = 0; k < kNF; ++k) f[k] = in ? a.field[k * N + o] : 0.f;
  };
  if (kPre) {
#pragma unroll
    for (int it = 0; it < kIt; ++it) staged_field(tid + it * NTHR, fpre[kPre ? it : 0]);
  }
  // The own cells' dense adjoint source (written before the step loop, so
  // loaded before the wait) and, after it, their lam^{m+1} and lam^{m+2},
  // issued with the staging loads: one memory round before the barrier.
  const int gj = y0 + tx;
  const bool dense_src = a.frame >= 0 && a.record == kRecordFields;
  float gvx[RPT_], gvy[RPT_];
#pragma unroll
  for (int k = 0; k < RPT_; ++k) {
    const int gi = x0 + ty + (NTHR / TY) * k;
    const bool in = dense_src && gi < nx && gj < ny;
    const size_t go = in ? ((size_t)s * a.nt_out + a.frame) * N + (size_t)gi * ny + gj : 0;
    gvx[k] = in ? a.g_x[go] : 0.f;
    gvy[k] = in ? a.g_y[go] : 0.f;
  }
  grid_dep_wait();
  const float* prev = a.prev + (size_t)s * 2 * N;
  float l1x_[RPT_], l1y_[RPT_], pvx[RPT_], pvy[RPT_];
#pragma unroll
  for (int k = 0; k < RPT_; ++k) {
    const int gi = x0 + ty + (NTHR / TY) * k;
    const bool in = gi < nx && gj < ny;
    const size_t o = in ? (size_t)gi * ny + gj : 0;
    l1x_[k] = in ? cur[o] : 0.f;
    l1y_[k] = in ? cur[N + o] : 0.f;
    pvx[k] = in ? prev[o] : 0.f;
    pvy[k] = in ? prev[N + o] : 0.f;
  }
#pragma unroll
  for (int it = 0; it < kIt; ++it) {
    const int e = tid + it * NTHR;
    if (e >= kStaged) break;
    const int r = e / HY, c = e - r * HY;
    const int gi = x0 + r - 1, gj = y0 + c - 1;
    const bool in = gi >= 0 && gi < nx && gj >= 0 && gj < ny;
    const size_t o = in ? (size_t)gi * ny + gj : 0;
    const float lx = in ? cur[o] : 0.f;
    const float ly = in ? cur[N + o] : 0.f;
    float fv[kNF];
    if (MODE != kModeScalar) {
      if (kPre) {
#pragma unroll
        for (int k = 0; k < kNF; ++k) fv[k] = fpre[kPre ? it : 0][k];
      } else {
        staged_field(e, fv);
      }
    }
    if (MODE == kModeScalar) {
      sl[0][r][c] = lx;
      sl[1][r][c] = ly;
    } else if (MODE == kModeDField) {
      const float w = in ? 1.f - fv[0] : 0.f;
      sl[0][r][c] = w * lx;
      sl[1][r][c] = w * ly;
    } else {
      const float C11 = fv[0], C22 = fv[1], C12 = fv[2], C16 = fv[3], C26 = fv[4], C66 = fv[5];
      const float c1266 = C12 + C66;
      sl[0][r][c] = C11 * lx + C16 * ly;
      sl[1][r][c] = C66 * lx + C26 * ly;
      sl[2][r][c] = 2.f * C16 * lx + c1266 * ly;
      sl[3][r][c] = C16 * lx + C66 * ly;
      sl[4][r][c] = C26 * lx + C22 * ly;
      sl[5][r][c] = c1266 * lx + 2.f * C26 * ly;
    }
    float vx = 0.f, vy = 0.f;
    if (um != nullptr && in) {
      vx = um[o];
      vy = um[N + o];
    }
    su[0][r][c] = vx;
    su[1][r][c] = vy;
  }
  __syncthreads();

  KS ks;
  if (MODE != kModeFields) ks = load_ks(K);
  const float gs = K->gscale;
  float* out = a.out + (size_t)s * 2 * N;
  float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // this thread's cells, one step
  float nvx[RPT_], nvy[RPT_];
#pragma unroll
  for (int k = 0; k < RPT_; ++k) {
    nvx[k] = 0.f;
    nvy[k] = 0.f;
    const int r = ty + (NTHR / TY) * k;
    const int gi = x0 + r;
    if (gi >= nx || gj >= ny) continue;
    const size_t o = (size_t)gi * ny + gj;
    const float l1x = l1x_[k], l1y = l1y_[k];
    float ax, ay;
    if (MODE == kModeFields) {
      const float xx0 = (sl[0][r][tx + 1] + sl[0][r + 2][tx + 1]) - 2.f * sl[0][r + 1][tx + 1];
      const float yy1 = (sl[1][r + 1][tx] + sl[1][r + 1][tx + 2]) - 2.f * sl[1][r + 1][tx + 1];
      const float xy2 = (sl[2][r + 2][tx + 2] + sl[2][r][tx]) - (sl[2][r + 2][tx] + sl[2][r][tx + 2]);
      const float xx3 = (sl[3][r][tx + 1] + sl[3][r + 2][tx + 1]) - 2.f * sl[3][r + 1][tx + 1];
      const float yy4 = (sl[4][r + 1][tx] + sl[4][r + 1][tx + 2]) - 2.f * sl[4][r + 1][tx + 1];
      const float xy5 = (sl[5][r + 2][tx + 2] + sl[5][r][tx]) - (sl[5][r + 2][tx] + sl[5][r][tx + 2]);
      ax = q * (xx0 + yy1 + 0.25f * xy2);
      ay = q * (xx3 + yy4 + 0.25f * xy5);
    } else {
      const Sten sw = stencils(sl[0], sl[1], r, tx);
      apply_ks(ks, sw, ax, ay);
    }
    float vx = (2.f * l1x - pvx[k]) + ax;
    float vy = (2.f * l1y - pvy[k]) + ay;
    if (dense_src) {
      vx += gs * gvx[k];
      vy += gs * gvy[k];
    }
    nvx[k] = vx;
    nvy[k] = vy;
    if (um != nullptr) {
      const Sten su_ = stencils(su[0], su[1], r, tx);
      if (MODE == kModeDField) {
        float Lx, Ly;
        apply_ks(ks, su_, Lx, Ly);
        a.gacc[(size_t)s * N + o] += l1x * Lx + l1y * Ly;
      } else {
        const float g0 = l1x * su_.xx_x;
        const float g1 = l1y * su_.yy_y;
        const float g2 = l1x * su_.xy_y + l1y * su_.xy_x;
        const float g3 = l1x * (0.5f * su_.xy_x + su_.xx_y) + l1y * su_.xx_x;
        const float g4 = l1x * su_.yy_y + l1y * (su_.yy_x + 0.5f * su_.xy_y);
        const float g5 = l1x * su_.yy_x + l1y * su_.xx_y;
        if (MODE == kModeScalar) {
          acc[0] += g0; acc[1] += g1; acc[2] += g2;
          acc[3] += g3; acc[4] += g4; acc[5] += g5;
        } else {
          float* ga = a.gacc + (size_t)s * 6 * N + o;
          ga[0] += g0; ga[N] += g1; ga[2 * N] += g2;
          ga[3 * N] += g3; ga[4 * N] += g4; ga[5 * N] += g5;
        }
      }
    }
  }

  // Adjoint source at receiver cells: add into a shared copy of the output
  // tile (several receivers may share a cell), then store.
  const bool inject = (a.frame >= 0 && a.record == kRecordReceivers);
  if (inject) {
    __syncthreads();  // everyone is done reading su
#pragma unroll
    for (int k = 0; k < RPT_; ++k) {
      const int r = ty + (NTHR / TY) * k;
      su[0][r][tx] = nvx[k];
      su[1][r][tx] = nvy[k];
    }
    __syncthreads();
    for (int rr = tid; rr < a.nrec; rr += NTHR) {
      const int32_t idx = a.rec_idx[(size_t)s * a.nrec + rr];
      if (idx < 0 || (size_t)idx >= N) continue;  // out of range: ignored
      const int gi = idx / ny, gjj = idx - gi * ny;
      if (gi >= x0 && gi < x0 + T && gjj >= y0 && gjj < y0 + TY) {
        const size_t go = ((size_t)s * a.nt_out + a.frame) * a.nrec + rr;
        atomicAdd(&su[0][gi - x0][gjj - y0], gs * a.g_x[go]);
        atomicAdd(&su[1][gi - x0][gjj - y0], gs * a.g_y[go]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RPT_; ++k) {
      const int r = ty + (NTHR / TY) * k;
      nvx[k] = su[0][r][tx];
      nvy[k] = su[1][r][tx];
    }
  }
#pragma unroll
  for (int k = 0; k < RPT_; ++k) {
    const int gi = x0 + ty + (NTHR / TY) * k;
    if (gi >= nx || gj >= ny) continue;
    const size_t o = (size_t)gi * ny + gj;
    out[o] = nvx[k];
    out[N + o] = nvy[k];
  }

  if (MODE == kModeScalar && um != nullptr) {
    // Imaging sums: FP32 over one warp's 128 cells (the FP64 pipe of this part
    // is far narrower than FP32), FP64 across warps, tiles and steps.
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      float v = acc[t];
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (tx == 0) red[ty][t] = (double)v;
    }
    __syncthreads();
    if (tid < 6) {
      double v = 0.0;
      for (int w = 0; w < NTHR / 32; ++w) v += red[w][tid];
      const size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
      a.partials[blk * 8 + tid] += v;
    }
  }
}

// --------------------------------------------------------------------------
// With instances (inst_box != nullptr) every shot reads the one canvas
// plane, and an instance whose step count is below `step` (the state index
// recorded) gets zeros: its frames end earlier.
__global__ void gather_kernel(const float* __restrict__ state, int N, int S,
                              const int32_t* __restrict__ rec_idx, int nrec, int frame,
                              int nt_out, float* __restrict__ tr_x, float* __restrict__ tr_y,
                              const int4* __restrict__ inst_box, int step) {
  const int total = S * nrec;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int s = e / nrec, r = e - s * nrec;
    const int32_t idx = rec_idx[e];
    const size_t o = ((size_t)s * nt_out + frame) * nrec + r;
    const size_t plane = inst_box ? 0 : (size_t)s * 2 * N;
    const bool ok = idx >= 0 && idx < N && (inst_box == nullptr || step <= inst_box[2 * s + 1].z);
    tr_x[o] = ok ? state[plane + idx] : 0.f;
    tr_y[o] = ok ? state[plane + N + idx] : 0.f;
  }
}

// max |g| over both adjoint sources into coef->gmax_bits (non-negative float
// bits order like the floats, so an unsigned atomicMax is a float max).
__global__ void gmax_kernel(const float* __restrict__ gx, const float* __restrict__ gy, size_t n,
                            Coef* coef) {
  float m = 0.f;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    m = fmaxf(m, fmaxf(fabsf(gx[e]), fabsf(gy[e])));
  }
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(&coef->gmax_bits, __float_as_uint(m));
}

// Power-of-two scale that brings max |g| into [1, 2): keeps the adjoint
// field away from FP32 denormals; undone exactly in FP64 at the end.
__global__ void gscale_kernel(Coef* coef, int ncoef) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint32_t bits = coef->gmax_bits;
  int e = (int)((bits >> 23) & 0xffu) - 127;  // unbiased exponent of max |g|
  if (bits == 0u || e > 126) e = 0;           // zero, inf or nan: no scaling
  if (e < -126) e = -126;
  for (int b = 0; b < ncoef; ++b) {            // one scale for every shot's block
    coef[b].gscale = __uint_as_float((uint32_t)(127 - e) << 23);               // 2^-e
    coef[b].inv_gscale = __longlong_as_double((long long)(1023 + e) << 52);    // 2^e
  }
}

// Deterministic FP64 sum of the per-block partials, then the chain from the
// six imaging sums to dL/dC.  Block s of the grid finalises gradient s from
// rows [s * rows, (s + 1) * rows) with coefficient block s * coef_stride
// (one gradient, or one per shot with per-shot constants).
__global__ void finalize_scalar_kernel(const double* __restrict__ partials, int nblocks,
                                       const Coef* coef, int coef_stride, double* __restrict__ grad) {
  __shared__ double sh[6][256];
  const int tid = threadIdx.x;
  partials += (size_t)blockIdx.x * nblocks * 8;
  coef += (size_t)blockIdx.x * coef_stride;
  grad += 6 * (size_t)blockIdx.x;
  for (int t = 0; t < 6; ++t) {
    double v = 0.0;
    for (int b = tid; b < nblocks; b += 256) v += partials[(size_t)b * 8 + t];
    sh[t][tid] = v;
  }
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (tid < w)
      for (int t = 0; t < 6; ++t) sh[t][tid] += sh[t][tid + w];
    __syncthreads();
  }
  if (tid == 0) {
    const double f = coef->qd * coef->inv_gscale;
    const double A11 = sh[0][0], A22 = sh[1][0], A12 = sh[2][0], A16 = sh[3][0];
    const double A26 = sh[4][0], B66 = sh[5][0];
    grad[0] = f * A11;
    grad[1] = f * A22;
    grad[2] = f * 0.25 * A12;
    grad[3] = f * A16;
    grad[4] = f * A26;
    grad[5] = f * (B66 + 0.25 * A12);
  }
}

__global__ void finalize_fields_kernel(int mode, const float* __restrict__ gacc, int S, int N,
                                       const Coef* coef, float* __restrict__ out) {
  const double inv = coef->inv_gscale;
  const double f = coef->qd * inv;
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x) {
    if (mode == kModeDField) {
      double v = 0.0;
      for (int s = 0; s < S; ++s) v += (double)gacc[(size_t)s * N + o];
      out[o] = (float)(-inv * v);
    } else {
      double A[6] = {0, 0, 0, 0, 0, 0};
      for (int s = 0; s < S; ++s)
        for (int t = 0; t < 6; ++t) A[t] += (double)gacc[((size_t)s * 6 + t) * N + o];
      out[o] = (float)(f * A[0]);
      out[(size_t)N + o] = (float)(f * A[1]);
      out[2 * (size_t)N + o] = (float)(f * 0.25 * A[2]);
      out[3 * (size_t)N + o] = (float)(f * A[3]);
      out[4 * (size_t)N + o] = (float)(f * A[4]);
      out[5 * (size_t)N + o] = (float)(f * (A[5] + 0.25 * A[2]));
    }
  }
}

// One application of the operator in the reference's own form
// (Inversion_adam.py:54-106): float h^-2 weights, constants after the
// stencils, (L + f) / rho.
__global__ void operator_kernel(int S, int nx, int ny, int mode, float w1,
                                const float* __restrict__ C, const float* __restrict__ D,
                                const float* __restrict__ rho, const float* __restrict__ ux,
                                const float* __restrict__ uy, const float* __restrict__ fx,
                                const float* __restrict__ fy, float* __restrict__ Lux,
                                float* __restrict__ Luy) {
  const size_t N = (size_t)nx * ny;
  const float w2 = w1 * -2.f, wq = w1 * 0.25f;
  const float r = rho[0];
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)S * N;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t s = e / N, o = e - s * N;
    const int i = (int)(o / ny), j = (int)(o - (size_t)i * ny);
    const float* px = ux + s * N;
    const float* py = uy + s * N;
    auto at = [&](const float* u, int ii, int jj) -> float {
      return (ii < 0 || ii >= nx || jj < 0 || jj >= ny) ? 0.f : u[(size_t)ii * ny + jj];
    };
    const float xx_x = w1 * at(px, i - 1, j) + w2 * at(px, i, j) + w1 * at(px, i + 1, j);
    const float yy_x = w1 * at(px, i, j - 1) + w2 * at(px, i, j) + w1 * at(px, i, j + 1);
    const float xx_y = w1 * at(py, i - 1, j) + w2 * at(py, i, j) + w1 * at(py, i + 1, j);
    const float yy_y = w1 * at(py, i, j - 1) + w2 * at(py, i, j) + w1 * at(py, i, j + 1);
    const float xy_x = wq * at(px, i - 1, j - 1) - wq * at(px, i + 1, j - 1) -
                       wq * at(px, i - 1, j + 1) + wq * at(px, i + 1, j + 1);
    const float xy_y = wq * at(py, i - 1, j - 1) - wq * at(py, i + 1, j - 1) -
                       wq * at(py, i - 1, j + 1) + wq * at(py, i + 1, j + 1);
    float C11, C22, C12, C16, C26, C66;
    if (mode == kModeFields) {
      C11 = C[o]; C22 = C[N + o]; C12 = C[2 * N + o];
      C16 = C[3 * N + o]; C26 = C[4 * N + o]; C66 = C[5 * N + o];
    } else {
      const float w = (mode == kModeDField) ? 1.f - D[o] : 1.f;
      C11 = w * C[0]; C22 = w * C[1]; C12 = w * C[2];
      C16 = w * C[3]; C26 = w * C[4]; C66 = w * C[5];
    }
    const float lx = C11 * xx_x + C66 * yy_x + (C12 + C66) * xy_y + (2.f * C16) * xy_x +
                     C16 * xx_y + C26 * yy_y;
    const float ly = C66 * xx_y + C22 * yy_y + (C12 + C66) * xy_x + C16 * xx_x + C26 * yy_x +
                     (2.f * C26) * xy_y;
    Lux[e] = (lx + (fx ? fx[e] : 0.f)) / r;
    Luy[e] = (ly + (fy ? fy[e] : 0.f)) / r;
  }
}

// --------------------------------------------------------------------------
// Host launchers.
static int small_grid(size_t n, int threads) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 4096) b = 4096;
  return (int)b;
}

cudaError_t launch_coef(int mode, const float* C, const float* rho, double h, double dt,
                        Coef* coef, cudaStream_t st, int ncoef) {
  return tracked(kProfOther, st, [&] { coef_kernel<<<ncoef, 32, 0, st>>>(mode, C, rho, h, dt, coef); });
}

cudaError_t launch_fwd_step(int mode, const FwdStep& a, cudaStream_t st) {
  const dim3 grid = step_grid(a.nx, a.ny, a.S), block(TY, NTHR / TY);
  const bool small = step_rows(a.nx, a.ny, a.S) != TX;
  const double cells = (double)a.S * a.nx * a.ny;
  return tracked(kProfForward, st, [&] {
    switch (mode) {
      case kModeScalar:
        if (small) launch_step_kernel(fwd_step_kernel<kModeScalar, 8>, grid, block, 0, st, a.chained != 0, a);
        else launch_step_kernel(fwd_step_kernel<kModeScalar, TX>, grid, block, 0, st, a.chained != 0, a);
        break;
      case kModeDField:
        if (small) launch_step_kernel(fwd_step_kernel<kModeDField, 8>, grid, block, 0, st, a.chained != 0, a);
        else launch_step_kernel(fwd_step_kernel<kModeDField, TX>, grid, block, 0, st, a.chained != 0, a);
        break;
      default:
        if (small) launch_step_kernel(fwd_step_kernel<kModeFields, 8>, grid, block, 0, st, a.chained != 0, a);
        else launch_step_kernel(fwd_step_kernel<kModeFields, TX>, grid, block, 0, st, a.chained != 0, a);
        break;
    }
  }, cells * alg_bytes_forward(mode));
}

cudaError_t launch_adj_step(int mode, const AdjStep& a, cudaStream_t st) {
  const dim3 grid = step_grid(a.nx, a.ny, a.S), block(TY, NTHR / TY);
  const bool small = step_rows(a.nx, a.ny, a.S) != TX;
  const double cells = (double)a.S * a.nx * a.ny;
  return tracked(kProfAdjoint, st, [&] {
    switch (mode) {
      case kModeScalar:
        if (small) launch_step_kernel(adj_step_kernel<kModeScalar, 8>, grid, block, 0, st, a.chained != 0, a);
        else launch_step_kernel(adj_step_kernel<kModeScalar, TX>, grid, block, 0, st, a.chained != 0, a);
        break;
      case kModeDField:
        if (small) launch_step_kernel(adj_step_kernel<kModeDField, 8>, grid, block, 0, st, a.chained != 0, a);
        else launch_step_kernel(adj_step_kernel<kModeDField, TX>, grid, block, 0, st, a.chained != 0, a);
        break;
      default:
        if (small) launch_step_kernel(adj_step_kernel<kModeFields, 8>, grid, block, 0, st, a.chained != 0, a);
        else launch_step_kernel(adj_step_kernel<kModeFields, TX>, grid, block, 0, st, a.chained != 0, a);
        break;
    }
  }, cells * alg_bytes_adjoint(mode));
}

cudaError_t launch_gather(const float* state, int nx, int ny, int S, const int32_t* rec_idx,
                          int nrec, int frame, int nt_out, float* tr_x, float* tr_y,
                          cudaStream_t st, const int4* inst_box, int step) {
  return tracked(kProfOther, st, [&] {
    gather_kernel<<<small_grid((size_t)S * nrec, 256), 256, 0, st>>>(
        state, nx * ny, S, rec_idx, nrec, frame, nt_out, tr_x, tr_y, inst_box, step);
  });
}

cudaError_t launch_gscale(const float* gx, const float* gy, size_t n, Coef* coef,
                          cudaStream_t st, int ncoef) {
  cudaError_t e = tracked(kProfOther, st, [&] {
    gmax_kernel<<<small_grid(n, 256), 256, 0, st>>>(gx, gy, n, coef);
  });
  if (e != cudaSuccess) return e;
  return tracked(kProfOther, st, [&] { gscale_kernel<<<1, 32, 0, st>>>(coef, ncoef); });
}

cudaError_t launch_finalize_scalar(const double* partials, int nblocks, const Coef* coef,
                                   double* grad_C, cudaStream_t st, int ngrad, int coef_stride) {
  return tracked(kProfOther, st, [&] {
    finalize_scalar_kernel<<<ngrad, 256, 0, st>>>(partials, nblocks, coef, coef_stride, grad_C);
  });
}

cudaError_t launch_finalize_fields(int mode, const float* gacc, int S, int N, const Coef* coef,
                                   float* grad_field, cudaStream_t st) {
  return tracked(kProfOther, st, [&] {
    finalize_fields_kernel<<<small_grid((size_t)N, 256), 256, 0, st>>>(mode, gacc, S, N, coef,
                                                                       grad_field);
  });
}

cudaError_t launch_operator(int S, int nx, int ny, int mode, double h, const float* C,
                            const float* D, const float* rho, const float* ux, const float* uy,
                            const float* fx, const float* fy, float* Lux, float* Luy,
                            cudaStream_t st) {
  const float w1 = (float)(1.0 / (h * h));
  return tracked(kProfOther, st, [&] {
    operator_kernel<<<small_grid((size_t)S * nx * ny, 256), 256, 0, st>>>(
        S, nx, ny, mode, w1, C, D, rho, ux, uy, fx, fy, Lux, Luy);
  });
}

}  // namespace ernn
