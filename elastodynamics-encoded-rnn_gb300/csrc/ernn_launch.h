// Host-side launch interface between the C ABI driver (ernn_abi.cu) and the
// kernels (ernn_kernels.cu).  Internal to the library.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <utility>
#include <cuda_runtime.h>

#include "ernn_common.cuh"

namespace ernn {

// Instances on one canvas (ERNN_FLAG_INSTANCES): the tiled kernels walk a
// tile table instead of the grid's tiling.  Entry t of the table is
// (instance, x0, y0, 0) of one 64 x 16 tile; per instance k, box[2k] =
// (x0, y0, x1, y1) of its region and box[2k + 1] = (first table entry of its
// tiles, tiles per tile row, steps, 0).
struct InstTiles {
  const int4* tiles;   // the table, instances ordered by decreasing step count
  const int4* box;     // per instance (region, tiling and step count)
  int ntiles;          // entries of this launch: the prefix of running instances
};

// Per-step arguments of the forward kernel: computes u^{i+1} from u^i, u^{i-1}.
// State buffers are laid out [shot][component][cell] with N = nx*ny cells.
struct FwdStep {
  int nx, ny, S, nt, i;
  const float* cur;   // u^i (nullptr: zero state)
  const float* prev;  // u^{i-1} (nullptr: zero state)
  float* out;         // u^{i+1}
  float* out2;        // two-step launches: u^{i+2}; otherwise nullptr
  float* copy0;       // optional second destination of u^{i+1} (checkpoint), or nullptr
  float* copy1;       // optional third destination, or nullptr
  // dense history: frame index (>= 0 when this step records), bases of (S, nt_out, N)
  float* hist_x;
  float* hist_y;
  int frame, nt_out;
  // receiver gather of the INPUT state u^i into frame gframe (>= 0 when due)
  const int32_t* rec_idx;
  int nrec, gframe;
  float* tr_x;
  float* tr_y;
  const Coef* coef;
  int coef_stride;     // 0: one coefficient block; 1: one per shot (coef + shot)
  const float* field;  // FIELDS: 6 planes of C; DFIELD: D plane
  const float* src_signal;
  const float* src_map;
  const int32_t* src_origin;
  int bx, by, src_comp;
  int chained;  // previous launch on the stream is a step kernel of the same loop
  InstTiles inst;  // instances: tile table (inst.tiles == nullptr otherwise)
  int tile_rows;   // tiled kernels: 32 for 64 x 32 tiles, otherwise the default (16)
};

// Per-step arguments of the adjoint kernel: computes lam^m from lam^{m+1},
// lam^{m+2}, adds the adjoint source of frame `frame` and accumulates the
// imaging condition of lam^{m+1} against u^m.
struct AdjStep {
  int nx, ny, S, m;
  const float* cur;   // lam^{m+1}
  const float* prev;  // lam^{m+2}
  float* out;         // lam^m (may alias prev)
  const float* u;     // u^m, nullptr when the imaging term vanishes (m == nt)
  const Coef* coef;
  int coef_stride;    // 0: one coefficient block; 1: one per shot (coef + shot)
  const float* field;
  const float* g_x;   // adjoint source bases (S, nt_out, N or nrec)
  const float* g_y;
  int frame, nt_out, record, nrec;
  const int32_t* rec_idx;
  double* partials;   // SCALAR: [row][8] FP64 running sums (rows: see the kernels)
  float* gacc;        // DFIELD: [S][N]; FIELDS: [S][6][N] running sums
  // tiled kernels: non-zero for the 64 x 32 tiles (shot-major) holding a
  // receiver, or nullptr (every tile scans the receivers)
  const uint8_t* tile_flags;
  int chained;  // previous launch on the stream is a step kernel of the same loop
  InstTiles inst;  // instances: tile table (inst.tiles == nullptr otherwise)
  int tile_rows;   // tiled kernels: 32 for 64 x 32 tiles, otherwise the default (16)
};

dim3 step_grid(int nx, int ny, int S);

// ncoef coefficient blocks from C[6 ncoef] and rho[ncoef].
cudaError_t launch_coef(int mode, const float* C, const float* rho, double h, double dt,
                        Coef* coef, cudaStream_t st, int ncoef = 1);
cudaError_t launch_fwd_step(int mode, const FwdStep& a, cudaStream_t st);
cudaError_t launch_adj_step(int mode, const AdjStep& a, cudaStream_t st);
cudaError_t launch_gather(const float* state, int nx, int ny, int S, const int32_t* rec_idx,
                          int nrec, int frame, int nt_out, float* tr_x, float* tr_y,
                          cudaStream_t st, const int4* inst_box = nullptr, int step = 0);
cudaError_t launch_gscale(const float* gx, const float* gy, size_t n, Coef* coef,
                          cudaStream_t st, int ncoef = 1);
// ngrad gradients of 6: gradient s sums partial rows [s nblocks, (s+1) nblocks).
cudaError_t launch_finalize_scalar(const double* partials, int nblocks, const Coef* coef,
                                   double* grad_C, cudaStream_t st, int ngrad = 1,
                                   int coef_stride = 0);
cudaError_t launch_finalize_fields(int mode, const float* gacc, int S, int N,
                                   const Coef* coef, float* grad_field, cudaStream_t st);
cudaError_t launch_operator(int S, int nx, int ny, int mode, double h, const float* C,
                            const float* D, const float* rho, const float* ux, const float* uy,
                            const float* fx, const float* fy, float* Lux, float* Luy,
                            cudaStream_t st);

uint64_t launches();
void count_launch();

// Launch overlap of consecutive step kernels (programmatic dependent launch,
// see grid_dep_wait): on unless switched off, and off while the diagnostic
// profiler brackets launches with events.
bool launch_overlap();
bool launch_overlap_setting();  // the switch alone
void set_launch_overlap(bool on);

// Enqueue `kernel` on st; `chained`: as a programmatic dependent of the
// previous kernel on st (a step kernel that calls grid_dep_wait before it
// touches state).
template <class... KArgs, class... Args>
inline void launch_step_kernel(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                               cudaStream_t st, bool chained, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (chained && launch_overlap()) ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// kernel classes of the diagnostic profiler
constexpr int kProfForward = 0;
constexpr int kProfAdjoint = 1;
constexpr int kProfOther = 2;
constexpr int kProfClasses = 3;
void profile_enable(bool on);
cudaError_t profile_read(double* ms, uint64_t* count, double* alg_bytes);
// Enqueue one kernel through `fn`, counting it and, while profiling, timing it
// and adding its algorithmic DRAM bytes to its class.
cudaError_t tracked_launch(int cls, cudaStream_t st, const std::function<void()>& fn,
                           double alg_bytes = 0.0);

// Algorithmic bytes per cell-step (the minimum DRAM traffic of a step whose
// state does not fit on chip):
//   forward: read u^n and u^{n-1}, write u^{n+1}: 3 x 8 B, plus 4 B of D or
//            24 B of constant planes in the per-cell modes;
//   adjoint: read lam^{m+1}, lam^{m+2}, u^m, write lam^m: 4 x 8 B, plus the
//            per-cell inputs and the read-modify-write of per-cell gradients.
inline double alg_bytes_forward(int mode) {
  return 24.0 + (mode == kModeDField ? 4.0 : mode == kModeFields ? 24.0 : 0.0);
}
// Record which kernels ran the time loop of the latest propagation call
// (ernn_last_path).
void record_last_path(int32_t path);

inline double alg_bytes_adjoint(int mode) {
  return 32.0 + (mode == kModeDField ? 4.0 + 8.0 : mode == kModeFields ? 24.0 + 48.0 : 0.0);
}

}  // namespace ernn
