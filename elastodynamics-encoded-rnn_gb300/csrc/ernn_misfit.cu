// Misfit of predicted against observed series and its gradient, the step
// between the forward and the adjoint of an inversion iteration:
//   loss = wx * sum((px - ox)^2) / count + wy * sum((py - oy)^2) / count
// over the counted frames (every frame_stride-th) of every series, and
//   gx = 2 (wx g0 + g1) (px - ox) / count on counted frames, 0 elsewhere
//   (likewise gy with wy g0 + g2)
// for upstream gradients (g0, g1, g2) of (loss, mean square x, mean square
// y).  The loss is the MSE of Parameter_inversion/Inversion_adam.py:389-391
// (wx = wy = 1) and the 5:1 weighted data term of
// Damage_inversion/Inversion_adam.py:441-463 on every
// secondary_time_stride-th frame (Inversion_adam.py:420-422).
//
// Layout: series x frames x n floats, y contiguous within a frame, as the
// library's traces (S, nt_out, nrec) and histories (S, nt_out, nx, ny).
// Differences and squares in FP32 (as the reference forms them), summed per
// thread with an error-compensated FP32 pair (TwoSum), across threads and
// blocks in FP64; the block partials are summed in a fixed order, so the
// loss is bitwise reproducible.  One pass over the counted frames for the
// loss, one over all frames for the gradient.
#include <cstdint>

#include "ernn.h"
#include "ernn_launch.h"

namespace ernn {
namespace {

constexpr int kMisfitThreads = 256;
constexpr int kMisfitMaxBlocks = 1024;

// Counted elements as rows of `len` floats: one row for the whole layout
// when every element counts, else one row per counted frame of a series
// holding its counted cells (i, j multiples of the space stride).
struct Rows {
  int64_t rows, len;        // rows x len counted floats in all
  int64_t frames, nf;       // frames per series; counted frames nf = ceil(frames / ts)
  int64_t frame_len;        // nx * ny
  int32_t ts, ss, ny, nys;  // strides, frame width, counted cells per frame row
  bool flat;
  __device__ __forceinline__ int64_t row_off(int64_t r) const {
    if (flat) return 0;
    const int64_t s = r / nf, f = r - s * nf;
    return (s * frames + f * ts) * frame_len;
  }
  __device__ __forceinline__ int64_t cell_off(int64_t e) const {
    if (ss == 1) return e;
    const int32_t a = (int32_t)(e / nys), b = (int32_t)(e - (int64_t)a * nys);
    return (int64_t)a * ss * ny + (int64_t)b * ss;
  }
};

Rows counted_rows(const ErnnSeries& s) {
  Rows R;
  R.frames = s.frames;
  R.ts = s.frame_stride;
  R.ss = s.space_stride;
  R.ny = s.ny;
  R.frame_len = (int64_t)s.nx * s.ny;
  R.nf = (s.frames + s.frame_stride - 1) / s.frame_stride;
  const int32_t nxs = (s.nx + s.space_stride - 1) / s.space_stride;
  R.nys = (s.ny + s.space_stride - 1) / s.space_stride;
  R.flat = s.frame_stride == 1 && s.space_stride == 1;
  R.rows = R.flat ? 1 : s.series * R.nf;
  R.len = R.flat ? s.series * s.frames * R.frame_len : (int64_t)nxs * R.nys;
  return R;
}

__device__ __forceinline__ void two_sum(float& s, float& c, float v) {
  const float t = s + v;
  const float bp = t - s;
  c += (s - (t - bp)) + (v - bp);
  s = t;
}

__global__ void __launch_bounds__(kMisfitThreads)
    misfit_partial_kernel(const float* __restrict__ px, const float* __restrict__ py,
                          const float* __restrict__ ox, const float* __restrict__ oy, Rows R,
                          double2* __restrict__ partials) {
  float sx = 0.f, cx = 0.f, sy = 0.f, cy = 0.f;
  const int64_t step = (int64_t)gridDim.x * kMisfitThreads;
  for (int64_t r = blockIdx.y; r < R.rows; r += gridDim.y) {
    const int64_t base = R.row_off(r);
    for (int64_t e = (int64_t)blockIdx.x * kMisfitThreads + threadIdx.x; e < R.len; e += step) {
      const int64_t o = base + R.cell_off(e);
      const float dx = px[o] - ox[o];
      const float dy = py[o] - oy[o];
      two_sum(sx, cx, dx * dx);
      two_sum(sy, cy, dy * dy);
    }
  }
  double vx = (double)sx + (double)cx, vy = (double)sy + (double)cy;
  for (int o = 16; o > 0; o >>= 1) {
    vx += __shfl_down_sync(0xffffffffu, vx, o);
    vy += __shfl_down_sync(0xffffffffu, vy, o);
  }
  __shared__ double red[2][kMisfitThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = vx;
    red[1][warp] = vy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ax = 0.0, ay = 0.0;
    for (int w = 0; w < kMisfitThreads / 32; ++w) {
      ax += red[0][w];
      ay += red[1][w];
    }
    partials[blockIdx.y * gridDim.x + blockIdx.x] = make_double2(ax, ay);
  }
}

// One block: the partials in a fixed order, then the weighted means.
__global__ void __launch_bounds__(kMisfitThreads)
    misfit_final_kernel(const double2* __restrict__ partials, int nparts, double wx, double wy,
                        double inv_count, double* __restrict__ loss) {
  __shared__ double red[2][kMisfitThreads];
  double ax = 0.0, ay = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kMisfitThreads) {
    ax += partials[i].x;
    ay += partials[i].y;
  }
  red[0][threadIdx.x] = ax;
  red[1][threadIdx.x] = ay;
  __syncthreads();
  for (int h = kMisfitThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      red[0][threadIdx.x] += red[0][threadIdx.x + h];
      red[1][threadIdx.x] += red[1][threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double sx = red[0][0] * inv_count, sy = red[1][0] * inv_count;
    loss[0] = wx * sx + wy * sy;
    loss[1] = sx;
    loss[2] = sy;
  }
}

// Gradient over the whole layout (series x frames rows of nx * ny, or one
// row when everything counts): counted cells of counted frames get the
// scaled residual, the others zero.
__global__ void __launch_bounds__(kMisfitThreads)
    misfit_grad_kernel(const float* __restrict__ px, const float* __restrict__ py,
                       const float* __restrict__ ox, const float* __restrict__ oy, int64_t rows,
                       int64_t len, int64_t frames, int32_t ts, int32_t ss, int32_t ny, double wx,
                       double wy, double two_over_count, const double* __restrict__ grad_loss,
                       float* __restrict__ gx, float* __restrict__ gy) {
  // upstream gradients of (loss, mean square x, mean square y)
  const double g0 = grad_loss ? grad_loss[0] : 1.0;
  const double g1 = grad_loss ? grad_loss[1] : 0.0, g2 = grad_loss ? grad_loss[2] : 0.0;
  const float ax = (float)(two_over_count * (wx * g0 + g1));
  const float ay = (float)(two_over_count * (wy * g0 + g2));
  const int64_t step = (int64_t)gridDim.x * kMisfitThreads;
  for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
    const bool frame_counted = ts == 1 || (r % frames) % ts == 0;
    const int64_t base = r * len;
    for (int64_t e = (int64_t)blockIdx.x * kMisfitThreads + threadIdx.x; e < len; e += step) {
      const int64_t o = base + e;
      bool counted = frame_counted;
      if (ss > 1) {
        const int32_t i = (int32_t)(e / ny), j = (int32_t)(e - (int64_t)i * ny);
        counted = counted && i % ss == 0 && j % ss == 0;
      }
      float vx = 0.f, vy = 0.f;
      if (counted) {
        vx = ax * (px[o] - ox[o]);
        vy = ay * (py[o] - oy[o]);
      }
      gx[o] = vx;
      gy[o] = vy;
    }
  }
}

int num_sms_cached() {
  static int sms = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 132;
    return v;
  }();
  return sms;
}

// Blocks along a row and over rows: about four blocks per SM in all.
dim3 grid_of(int64_t rows, int64_t len) {
  const int64_t want = 4LL * num_sms_cached();
  int64_t gx = (len + kMisfitThreads * 4 - 1) / (kMisfitThreads * 4);
  gx = gx < 1 ? 1 : (gx > want ? want : gx);
  int64_t gy = want / gx;
  gy = gy < 1 ? 1 : (gy > rows ? rows : gy);
  if (gx * gy > kMisfitMaxBlocks) gy = kMisfitMaxBlocks / gx;
  if (gy > 65535) gy = 65535;
  return dim3((unsigned)gx, (unsigned)(gy < 1 ? 1 : gy), 1);
}

int validate_series(const ErnnSeries* s) {
  if (s == nullptr || s->series < 1 || s->frames < 1 || s->nx < 1 || s->ny < 1 ||
      s->frame_stride < 1 || s->space_stride < 1)
    return ERNN_ERR_INVALID;
  if (!(s->wx >= 0.0) || !(s->wy >= 0.0)) return ERNN_ERR_INVALID;  // also rejects NaN
  // element counts are formed in 64-bit: refuse series that would wrap them
  if ((double)s->series * (double)s->frames * (double)s->nx * (double)s->ny >= 4.0e18) return ERNN_ERR_INVALID;
  return ERNN_OK;
}

}  // namespace
}  // namespace ernn

using namespace ernn;

extern "C" {

size_t ernn_misfit_workspace_bytes(void) { return (size_t)kMisfitMaxBlocks * sizeof(double2); }

int ernn_misfit(const ErnnSeries* s, const float* px, const float* py, const float* ox,
                const float* oy, double* loss, void* workspace, size_t workspace_bytes, void* stream) {
  int rc = validate_series(s);
  if (rc) return rc;
  if (!px || !py || !ox || !oy || !loss || !workspace) return ERNN_ERR_INVALID;
  if (workspace_bytes < ernn_misfit_workspace_bytes()) return ERNN_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const Rows R = counted_rows(*s);
  const dim3 grid = grid_of(R.rows, R.len);
  double2* parts = static_cast<double2*>(workspace);
  const double count = (double)R.rows * (double)R.len;
  if (tracked_launch(kProfOther, st, [&] {
        misfit_partial_kernel<<<grid, kMisfitThreads, 0, st>>>(px, py, ox, oy, R, parts);
      }) != cudaSuccess)
    return ERNN_ERR_CUDA;
  if (tracked_launch(kProfOther, st, [&] {
        misfit_final_kernel<<<1, kMisfitThreads, 0, st>>>(parts, (int)(grid.x * grid.y), s->wx, s->wy,
                                                           1.0 / count, loss);
      }) != cudaSuccess)
    return ERNN_ERR_CUDA;
  return ERNN_OK;
}

int ernn_misfit_grad(const ErnnSeries* s, const float* px, const float* py, const float* ox,
                     const float* oy, const double* grad_loss, float* gx, float* gy, void* stream) {
  int rc = validate_series(s);
  if (rc) return rc;
  if (!px || !py || !ox || !oy || !gx || !gy) return ERNN_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  const Rows R = counted_rows(*s);
  const double count = (double)R.rows * (double)R.len;
  const int64_t frame_len = (int64_t)s->nx * s->ny;
  const int64_t rows = R.flat ? 1 : s->series * s->frames;
  const int64_t len = R.flat ? s->series * s->frames * frame_len : frame_len;
  const dim3 grid = grid_of(rows, len);
  if (tracked_launch(kProfOther, st, [&] {
        misfit_grad_kernel<<<grid, kMisfitThreads, 0, st>>>(px, py, ox, oy, rows, len, s->frames,
                                                            s->frame_stride, s->space_stride, s->ny,
                                                            s->wx, s->wy, 2.0 / count, grad_loss, gx,
                                                            gy);
      }) != cudaSuccess)
    return ERNN_ERR_CUDA;
  return ERNN_OK;
}

}  // extern "C"
