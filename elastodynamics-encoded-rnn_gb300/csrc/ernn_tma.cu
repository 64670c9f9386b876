// Per-step kernels for large grids (sm_103a), TMA-pipelined.
//
// One launch per time step, as the first per-step kernels, but each CTA is
// persistent over a list of 64 (y) x TR (x) tiles of the step (TR = 16 for
// the forward and the scalar adjoint, 32 for the D-field adjoint) and
// streams them through a two-stage shared-memory pipeline: while a tile is
// computed, the tensor-memory-accelerator loads of the next tile are in
// flight (cp.async.bulk.tensor, completion on an mbarrier per stage).
//
// The halo box of a tile is 72 x (TR + 2) cells: rows x0-1 .. x0+TR and
// columns y0-4 .. y0+67 (the innermost coordinate must be a multiple of four
// floats, so the box reaches four columns to the left where one is needed).
// Cells outside the grid are filled with zeros by the copy engine: that is
// the zero ghost ring of the scheme, with no predicated loads.  The two-step
// forward (recompute segments) takes a box two cells deep instead.
//
// Scalar constants (ERNN_MODE_SCALAR) and the degradation map (ERNN_MODE_DFIELD),
// ny % 4 == 0.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "ernn_launch.h"
#include "ernn_tma.h"

namespace ernn {

namespace {

constexpr int kTY = 64;                    // tile columns (y); rows per kernel layout
constexpr int kBW = kTY + 8;               // halo box width: tile + 4 columns each side
constexpr int kThreads = 256;              // 16 column quads x 16 rows

__device__ __forceinline__ uint32_t s32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Fetch a tensor map (a __grid_constant__ kernel parameter) into the
// descriptor cache ahead of its first copy.
__device__ __forceinline__ void prefetch_map(const CUtensorMap* m) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(s32(b)) : "memory");
}

__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s32(b)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(s32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait (about a second); on timeout records ERNN_ERR_TIMEOUT and
// returns so that the CTA's barriers stay matched.
__device__ __forceinline__ void bar_wait(uint64_t* b, uint32_t parity, int* err) {
  if (bar_try(b, parity)) return;
  if (*(volatile int*)err != 0) return;
  const long long t0 = clock64();
  for (;;) {
    for (int k = 0; k < 64; ++k)  // the clock is read once per 64 polls
      if (bar_try(b, parity)) return;
    if (clock64() - t0 > kWaitLimitCycles) {
      atomicExch(err, kDeviceTimeout);
      return;
    }
  }
}

// Error path of a tile pipeline.  A wait that gives up (its own time limit,
// or an error another CTA of the launch already recorded) marks the CTA
// failed: from then on no further tile loads are issued (the launch's
// outputs are invalid anyway), and before the CTA exits one thread waits,
// again with a time limit, for the loads it had already issued, so no copy
// is still writing into the shared memory of a CTA that has ended.
struct PipeGuard {
  int failed;  // a wait of this CTA gave up
  int issued;  // tiles 0 .. issued-1 of this CTA had their loads issued
};

__device__ __forceinline__ void pipe_init(PipeGuard* g) {
  g->failed = 0;
  g->issued = 0;
}
__device__ __forceinline__ bool pipe_failed(const PipeGuard* g) {
  return *reinterpret_cast<const volatile int*>(&g->failed) != 0;
}
__device__ __forceinline__ void pipe_issued(PipeGuard* g, int k) { atomicMax(&g->issued, k + 1); }

// bar_wait that reports whether the phase completed (false: timed out, or an
// error of the launch was already recorded); a false marks the CTA failed
__device__ __forceinline__ bool bar_wait_ok(uint64_t* b, uint32_t parity, int* err, PipeGuard* g) {
  if (bar_try(b, parity)) return true;
  if (*(volatile int*)err == 0) {
    const long long t0 = clock64();
    for (;;) {
      for (int k = 0; k < 64; ++k)
        if (bar_try(b, parity)) return true;
      if (clock64() - t0 > kWaitLimitCycles) {
        atomicExch(err, kDeviceTimeout);
        break;
      }
    }
  }
  *reinterpret_cast<volatile int*>(&g->failed) = 1;
  __threadfence_block();
  return false;
}

// After a failed CTA's tile loop (one thread): wait, each with a time limit,
// for the phases of the last `ns` issued tiles (tile k: stage k % ns, phase
// parity (k / ns) & 1).  A phase that already completed returns at once.
__device__ __forceinline__ void pipe_drain(uint64_t* bar, int ns, const PipeGuard* g) {
  const int issued = *reinterpret_cast<const volatile int*>(&g->issued);
  for (int k = issued - ns < 0 ? 0 : issued - ns; k < issued; ++k) {
    const long long t0 = clock64();
    while (!bar_try(&bar[k % ns], (uint32_t)(k / ns) & 1u))
      if (clock64() - t0 > kWaitLimitCycles) break;
  }
}

// 3D tile load (columns, rows, component planes) into shared memory.
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                          uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(s32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(s32(b))
      : "memory");
}

// End of a warp's reads of stage k & 1: the last of the CTA's warps to get
// there starts the loads of tile k + 2 into it, so no warp waits on the
// others between tiles.  The values read from the stage are all consumed
// (in registers) before a lane arrives.
template <typename F>
__device__ __forceinline__ void release_stage(int* done, int stage, F&& refill) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    const int old = atomicAdd(&done[stage], 1);
    if (old % (kThreads / 32) == kThreads / 32 - 1) refill();
  }
}
template <typename F>
__device__ __forceinline__ void release(int* done, int k, F&& refill) {
  release_stage(done, k & 1, refill);
}

// TMA destinations start on 128-byte boundaries: the dynamic shared block is
// allocated 128 bytes longer and its start rounded up.
// (pointer arithmetic on the __shared__ array, so the compiler keeps the
// shared state space and emits shared-memory loads)
__device__ __forceinline__ float* aligned128(float* p) {
  const uint32_t a = s32(p);
  return p + ((((a + 127u) & ~127u) - a) >> 2);
}

__device__ __forceinline__ void fence_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

struct Coefs {
  float k11, k22, kq12, k16, k26, k66, k16h, k26h;
};

__device__ __forceinline__ Coefs coefs(const Coef* c) {
  return Coefs{c->k11, c->k22, c->kq12, c->k16, c->k26, c->k66, c->k16h, c->k26h};
}

// window [j-1 .. j+4] of halo-box row r (box column of cell column j is j + 4)
__device__ __forceinline__ void win(const float* __restrict__ box, int r, int j, float w[6]) {
  const float* p = box + r * kBW + j + 4;
  const float4 m = *reinterpret_cast<const float4*>(p);
  w[0] = p[-1];
  w[1] = m.x;
  w[2] = m.y;
  w[3] = m.z;
  w[4] = m.w;
  w[5] = p[4];
}

// Packed FP32 (sm_100 family): one instruction applies the same operation to
// two cells of a quad, each lane rounded as the scalar operation would be,
// which halves the arithmetic instructions of a quad.  Sums whose operands
// are column neighbours (not register pairs of the window) are formed by
// scalar adds first, so every value keeps the association and rounding of
// the scalar formulas.
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 pair(const float v[4], int p) { return make_float2(v[2 * p], v[2 * p + 1]); }
__device__ __forceinline__ float2 pair4(const float4& v, int p) {
  return p == 0 ? make_float2(v.x, v.y) : make_float2(v.z, v.w);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void put(float v[4], int p, float2 a) {
  v[2 * p] = a.x;
  v[2 * p + 1] = a.y;
}

struct Sums4 {
  float cx[4], cy[4], xx_x[4], yy_x[4], xy_x[4], xx_y[4], yy_y[4], xy_y[4];
};

// Second differences of one component at the four cells of a window row
// (cell q at window column q + 1):
//   xx = (u[0][k] + u[2][k]) - 2 u[1][k],  yy = (u[1][k-1] + u[1][k+1]) - 2 u[1][k],
//   xy = (u[2][k+1] + u[0][k-1]) - (u[2][k-1] + u[0][k+1]).
__device__ __forceinline__ void comp_sums(const float u[3][6], float xx[4], float yy[4], float xy[4]) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int k = 2 * p + 1;
    const float2 m0 = make_float2(u[0][k], u[0][k + 1]);
    const float2 m1 = make_float2(u[1][k], u[1][k + 1]);
    const float2 m2 = make_float2(u[2][k], u[2][k + 1]);
    put(xx, p, fma2(dup2(-2.f), m1, __fadd2_rn(m0, m2)));
    put(yy, p, fma2(dup2(-2.f), m1, make_float2(u[1][k - 1] + u[1][k + 1], u[1][k] + u[1][k + 2])));
    const float2 a = make_float2(u[2][k + 1] + u[0][k - 1], u[2][k + 2] + u[0][k]);
    const float2 b = make_float2(u[2][k - 1] + u[0][k + 1], u[2][k] + u[0][k + 2]);
    put(xy, p, __fadd2_rn(a, neg2(b)));
  }
}

// The same sums one cell per instruction (identical values: every sum is
// the same rounded operation); for kernels at their register limit.
__device__ __forceinline__ void comp_sums_scalar(const float u[3][6], float xx[4], float yy[4], float xy[4]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q + 1;
    xx[q] = (u[0][k] + u[2][k]) - 2.f * u[1][k];
    yy[q] = (u[1][k - 1] + u[1][k + 1]) - 2.f * u[1][k];
    xy[q] = (u[2][k + 1] + u[0][k - 1]) - (u[2][k - 1] + u[0][k + 1]);
  }
}

template <bool PACKED = true>
__device__ __forceinline__ void sums4(const float ux[3][6], const float uy[3][6], Sums4& s) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    s.cx[q] = ux[1][q + 1];
    s.cy[q] = uy[1][q + 1];
  }
  if (PACKED) {
    comp_sums(ux, s.xx_x, s.yy_x, s.xy_x);
    comp_sums(uy, s.xx_y, s.yy_y, s.xy_y);
  } else {
    comp_sums_scalar(ux, s.xx_x, s.yy_x, s.xy_x);
    comp_sums_scalar(uy, s.xx_y, s.yy_y, s.xy_y);
  }
}

__device__ __forceinline__ void apply(const Coefs& k, const Sums4& s, int q, float& lx, float& ly) {
  lx = k.k11 * s.xx_x[q] + k.k66 * s.yy_x[q] + k.kq12 * s.xy_y[q] + k.k16h * s.xy_x[q] +
       k.k16 * s.xx_y[q] + k.k26 * s.yy_y[q];
  ly = k.k66 * s.xx_y[q] + k.k22 * s.yy_y[q] + k.kq12 * s.xy_x[q] + k.k16 * s.xx_x[q] +
       k.k26 * s.yy_x[q] + k.k26h * s.xy_y[q];
}

__device__ __forceinline__ void shift(float u[3][6]) {
#pragma unroll
  for (int k = 0; k < 6; ++k) { u[0][k] = u[1][k]; u[1][k] = u[2][k]; }
}

__device__ __forceinline__ float g4(const float4& v, int q) {
  return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w;
}

// (L u) of cells 2p and 2p+1: the terms of apply() in the same order.
__device__ __forceinline__ void apply2(const Coefs& k, const Sums4& s, int p, float2& lx, float2& ly) {
  lx = __fmul2_rn(dup2(k.k11), pair(s.xx_x, p));
  lx = fma2(dup2(k.k66), pair(s.yy_x, p), lx);
  lx = fma2(dup2(k.kq12), pair(s.xy_y, p), lx);
  lx = fma2(dup2(k.k16h), pair(s.xy_x, p), lx);
  lx = fma2(dup2(k.k16), pair(s.xx_y, p), lx);
  lx = fma2(dup2(k.k26), pair(s.yy_y, p), lx);
  ly = __fmul2_rn(dup2(k.k66), pair(s.xx_y, p));
  ly = fma2(dup2(k.k22), pair(s.yy_y, p), ly);
  ly = fma2(dup2(k.kq12), pair(s.xy_x, p), ly);
  ly = fma2(dup2(k.k16), pair(s.xx_x, p), ly);
  ly = fma2(dup2(k.k26), pair(s.yy_x, p), ly);
  ly = fma2(dup2(k.k26h), pair(s.xy_y, p), ly);
}

// The forward update in two parts, so that the load joins the operator sum
// before the update, as in the reference's (A u + f) / rho: oper4 writes the
// operator terms w (L u) of a quad (w = 1 unless WEIGHT) into vx, vy, the
// caller adds the load there, and update4 turns them into v = (2 c - p) +
// (w (L u) + f), one rounding of the increment into 2 c - p.  (Added after
// the update instead, the forward's rounding near the source projects onto
// the gradient: ten times the FP32 reference's gradient error close to
// convergence.)
template <bool WEIGHT>
__device__ __forceinline__ void oper4(const Coefs& k, const Sums4& s, const float4& w, float vx[4], float vy[4]) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float2 lx, ly;
    apply2(k, s, p, lx, ly);
    if (WEIGHT) {
      lx = __fmul2_rn(lx, pair4(w, p));
      ly = __fmul2_rn(ly, pair4(w, p));
    }
    vx[2 * p] = lx.x;
    vx[2 * p + 1] = lx.y;
    vy[2 * p] = ly.x;
    vy[2 * p + 1] = ly.y;
  }
}
__device__ __forceinline__ void update4(const float cx[4], const float cy[4], const float4& pvx, const float4& pvy,
                                        float vx[4], float vy[4]) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const float2 px = pair4(pvx, p), py = pair4(pvy, p);
    const float2 ax = __fadd2_rn(fma2(dup2(2.f), pair(cx, p), neg2(px)), make_float2(vx[2 * p], vx[2 * p + 1]));
    const float2 ay = __fadd2_rn(fma2(dup2(2.f), pair(cy, p), neg2(py)), make_float2(vy[2 * p], vy[2 * p + 1]));
    vx[2 * p] = ax.x;
    vx[2 * p + 1] = ax.y;
    vy[2 * p] = ay.x;
    vy[2 * p + 1] = ay.y;
  }
}

// Leapfrog update of a quad without a load: v = (2 c - p) + w (L u), w = 1
// unless WEIGHT (2 c is exact, so 2 c - p is one rounding either way).
template <bool WEIGHT>
__device__ __forceinline__ void leap4(const Coefs& k, const Sums4& s, const float cx[4], const float cy[4],
                                      const float4& pvx, const float4& pvy, const float4& w, float vx[4],
                                      float vy[4]) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float2 lx, ly;
    apply2(k, s, p, lx, ly);
    if (WEIGHT) {
      lx = __fmul2_rn(lx, pair4(w, p));
      ly = __fmul2_rn(ly, pair4(w, p));
    }
    const float2 px = pair4(pvx, p), py = pair4(pvy, p);
    const float2 ax = __fadd2_rn(fma2(dup2(2.f), pair(cx, p), neg2(px)), lx);
    const float2 ay = __fadd2_rn(fma2(dup2(2.f), pair(cy, p), neg2(py)), ly);
    vx[2 * p] = ax.x;
    vx[2 * p + 1] = ax.y;
    vy[2 * p] = ay.x;
    vy[2 * p + 1] = ay.y;
  }
}

// A tile: its state plane (shot), origin, and the instance it belongs to
// with that instance's region [xs, xe) x [ys, ye) (the shot and the whole
// grid unless the problem has instances on a canvas).
struct TileId {
  int shot, x0, y0;
  int inst, xs, ys, xe, ye;
};

// The grid's own tile as a TileId of its shot.
__device__ __forceinline__ TileId grid_tile(TileId id, int nx, int ny) {
  id.inst = id.shot;
  id.xs = 0;
  id.ys = 0;
  id.xe = nx;
  id.ye = ny;
  return id;
}

// An entry of an instance tile table (canvas plane 0): instance, then the
// tile's origin and its instance's region [xs, xe) x [ys, ye) as pairs of
// 16-bit canvas coordinates (row | column << 16; canvases are below 65536
// cells a side), so one 16-byte load gives the whole tile.
__device__ __forceinline__ TileId decode_tile(const int4 e) {
  TileId id;
  id.shot = 0;
  id.inst = e.x;
  id.x0 = (int)((unsigned)e.y & 0xffffu);
  id.y0 = (int)((unsigned)e.y >> 16);
  id.xs = (int)((unsigned)e.z & 0xffffu);
  id.ys = (int)((unsigned)e.z >> 16);
  id.xe = (int)((unsigned)e.w & 0xffffu);
  id.ye = (int)((unsigned)e.w >> 16);
  return id;
}
__device__ __forceinline__ TileId table_tile(const InstTiles& in, int t) { return decode_tile(__ldg(&in.tiles[t])); }

// The tiles t = first, first + stride, ... of a CTA, walked in (shot, row
// block, column block) coordinates: the stride is split once into the same
// mixed radix, so a step is an addition with two carries, not a division.
template <int TR>
struct TileWalk {
  int shot, xt, yt, ds, dx, dy, tiles_x, tiles_y;
  __device__ __forceinline__ void init(int first, int stride, int tx, int ty) {
    tiles_x = tx;
    tiles_y = ty;
    const int per = tx * ty;
    shot = first / per;
    int r = first - shot * per;
    xt = r / ty;
    yt = r - xt * ty;
    ds = stride / per;
    r = stride - ds * per;
    dx = r / ty;
    dy = r - dx * ty;
  }
  __device__ __forceinline__ TileId id() const { return TileId{shot, xt * TR, yt * kTY, shot, 0, 0, 0, 0}; }
  __device__ __forceinline__ void next() {
    yt += dy;
    if (yt >= tiles_y) { yt -= tiles_y; ++xt; }
    xt += dx;
    if (xt >= tiles_x) { xt -= tiles_x; ++shot; }
    shot += ds;
  }
};

template <int TR>  // tile rows
__device__ __forceinline__ TileId tile_of(int t, int tiles_x, int tiles_y) {
  const int per_shot = tiles_x * tiles_y;
  TileId id;
  id.shot = t / per_shot;
  const int r = t - id.shot * per_shot;
  id.x0 = (r / tiles_y) * TR;
  id.y0 = (r % tiles_y) * kTY;
  return id;
}

// Tile t of a step where a CTA issues its loads: an entry of the instance
// table (INST) or tile t of the shot-major grid of tiles.
template <bool INST, int TR>
__device__ __forceinline__ TileId step_tile(const InstTiles& in, int t, int tiles_x, int tiles_y) {
  if constexpr (INST) return table_tile(in, t);
  else return tile_of<TR>(t, tiles_x, tiles_y);
}

// Tile t of a CTA's compute loop, whose next tile is t + step (below end).
// The grid of tiles is walked in step with t (advanced here); table entries
// are loaded one tile ahead (`ahead` holds tile t's on entry, the next
// tile's on return), so a tile's entry is in registers when it starts.
template <bool INST, int TR>
__device__ __forceinline__ TileId walk_tile(const InstTiles& in, int t, int step, int end, int4& ahead,
                                            TileWalk<TR>& walk, int nx, int ny) {
  if constexpr (INST) {
    const TileId id = decode_tile(ahead);
    if (t + step < end) ahead = __ldg(&in.tiles[t + step]);
    return id;
  } else {
    const TileId id = grid_tile(walk.id(), nx, ny);
    walk.next();
    return id;
  }
}
// The first entry of a CTA's table walk (INST), else zeros.
template <bool INST>
__device__ __forceinline__ int4 first_entry(const InstTiles& in, int t, int end) {
  if constexpr (INST) return t < end ? __ldg(&in.tiles[t]) : make_int4(0, 0, 0, 0);
  else return make_int4(0, 0, 0, 0);
}

// 2D tile load (columns, rows) into shared memory: the degradation plane.
__device__ __forceinline__ void tma_load2(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(s32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(s32(b))
      : "memory");
}

__device__ __forceinline__ float4 one_minus(const float4 d) {
  return make_float4(1.f - d.x, 1.f - d.y, 1.f - d.z, 1.f - d.w);
}

// ----------------------------------------------------------------- forward
// Stage: halo box of u^i, own box of u^{i-1}.  DFIELD reads its 4 weights
// per row straight from global memory (one plane shared by every shot, L2
// resident).
// 64 x TR tiles, TR / 16 rows per thread: 16 rows by default (four CTAs per
// SM), 32 rows as a measured alternative (three CTAs per SM, a tenth fewer
// halo rows per cell).
template <int TR>
struct FwdLayoutT {
  static constexpr int kTR = TR;         // tile rows
  static constexpr int kRT = kTR / 16;   // rows per thread
  static constexpr int kBHa = kTR + 2;   // halo box rows
  static constexpr int kHalo = 2 * kBHa * kBW;
  static constexpr int kOwn = 2 * kTR * kTY;
  static constexpr int kStage = (kHalo + kOwn + 31) / 32 * 32;  // 128-byte multiple
  static constexpr int kCtasPerSm = TR == 16 ? 4 : 3;
};
using FwdLayout = FwdLayoutT<16>;

// INST: tiles from the instance table (one canvas plane, instance-bounded
// stores); otherwise the shot-major grid of tiles, with no table lookups.
template <int MODE, int TR, bool INST>
__global__ void __launch_bounds__(kThreads, FwdLayoutT<TR>::kCtasPerSm)
    tma_fwd_kernel(const FwdStep a, const __grid_constant__ CUtensorMap cur_map,
                   const __grid_constant__ CUtensorMap prev_map, int tiles_x, int tiles_y, int has_prev,
                   int* err) {
  extern __shared__ float sm_raw[];
  float* sm = aligned128(sm_raw);
  using F = FwdLayoutT<TR>;
  constexpr int kStage = F::kStage;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * kStage);
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny;
  const size_t N = (size_t)nx * ny;
  const int ntiles = INST ? a.inst.ntiles : a.S * tiles_x * tiles_y;
  const uint32_t bytes = (uint32_t)(F::kHalo + (has_prev ? F::kOwn : 0)) * 4u;
  grid_dep_trigger();
  __shared__ int done[2];
  __shared__ PipeGuard guard;
  if (tid == 0) {
    prefetch_map(&cur_map);
    prefetch_map(&prev_map);
    bar_init(&bar[0]);
    bar_init(&bar[1]);
    done[0] = done[1] = 0;
    pipe_init(&guard);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  grid_dep_wait();  // the state of the previous step is complete from here on

  // receiver gather of the input state u^i, spread over the grid
  if (a.gframe >= 0) {
    for (int e = blockIdx.x * kThreads + tid; e < a.S * a.nrec; e += gridDim.x * kThreads) {
      const int s = e / a.nrec, r = e - s * a.nrec;
      const int32_t idx = a.rec_idx[e];
      const size_t o = ((size_t)s * a.nt_out + a.gframe) * a.nrec + r;
      // instances: one canvas plane; an instance past its last step records zeros
      const size_t plane = INST ? 0 : (size_t)s * 2 * N;
      const bool ok = a.cur != nullptr && idx >= 0 && (size_t)idx < N && (!INST || a.i <= a.inst.box[2 * s + 1].z);
      a.tr_x[o] = ok ? a.cur[plane + idx] : 0.f;
      a.tr_y[o] = ok ? a.cur[plane + N + idx] : 0.f;
    }
  }
  __syncthreads();
  const bool has_src = a.bx > 0 && a.by > 0;
  auto issue = [&](int k) {  // loads of this CTA's k-th tile into stage k & 1
    const int t = blockIdx.x + k * gridDim.x;
    if (t >= ntiles || pipe_failed(&guard)) return;
    pipe_issued(&guard, k);
    const TileId id = step_tile<INST, F::kTR>(a.inst, t, tiles_x, tiles_y);
    float* st = sm + (k & 1) * kStage;
    fence_async();
    bar_expect(&bar[k & 1], bytes);
    tma_load3(st, &cur_map, id.y0 - 4, id.x0 - 1, 2 * id.shot, &bar[k & 1]);
    if (has_prev) tma_load3(st + F::kHalo, &prev_map, id.y0, id.x0, 2 * id.shot, &bar[k & 1]);
  };
  if (tid == 0) {
    issue(0);
    issue(1);
  }
  const int qc = tid & 15, rg = tid >> 4;
  const int j = 4 * qc;
  const Coefs ks0 = coefs(a.coef);  // every shot's, unless per-shot constants
  TileWalk<F::kTR> walk;
  walk.init(blockIdx.x, gridDim.x, tiles_x, tiles_y);
  int4 ahead = first_entry<INST>(a.inst, blockIdx.x, ntiles);
  for (int k = 0;; ++k) {
    const int t = blockIdx.x + k * gridDim.x;
    if (t >= ntiles) break;
    const TileId id = walk_tile<INST>(a.inst, t, (int)gridDim.x, ntiles, ahead, walk, nx, ny);
    // per-tile scalars, loaded before the wait (coefficients per shot with
    // per-shot constants)
    const Coef* K = a.coef + (size_t)id.inst * a.coef_stride;
    const Coefs ks = a.coef_stride != 0 ? coefs(K) : ks0;
    const float amp = a.src_signal[(size_t)id.inst * a.nt + a.i] * K->kappa;
    const int ox = has_src ? a.src_origin[2 * id.inst] : 0, oy = has_src ? a.src_origin[2 * id.inst + 1] : 0;
    const int gj = id.y0 + j;
    const int r0 = F::kRT * rg;  // tile row r0 + q2 -> box row r0 + q2 + 1
    float4 w4[F::kRT];
    if (MODE == kModeDField) {  // issued before the wait: overlaps the tile's loads
#pragma unroll
      for (int q2 = 0; q2 < F::kRT; ++q2) {
        const int gi = id.x0 + r0 + q2;
        w4[q2] = (gi < nx && gj < ny)
                     ? one_minus(__ldg(reinterpret_cast<const float4*>(a.field + (size_t)gi * ny + gj)))
                     : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    bar_wait_ok(&bar[k & 1], (uint32_t)(k >> 1) & 1u, err, &guard);
    const float* hb = sm + (k & 1) * kStage;
    const float* pb = hb + F::kHalo;
    float* out = a.out + (size_t)id.shot * 2 * N;
    float wx[3][6], wy[3][6];
    win(hb, r0, j, wx[0]);
    win(hb + F::kBHa * kBW, r0, j, wy[0]);
    win(hb, r0 + 1, j, wx[1]);
    win(hb + F::kBHa * kBW, r0 + 1, j, wy[1]);
#pragma unroll
    for (int q2 = 0; q2 < F::kRT; ++q2) {
      const int r = r0 + q2;
      win(hb, r + 2, j, wx[2]);
      win(hb + F::kBHa * kBW, r + 2, j, wy[2]);
      Sums4 st;
      sums4(wx, wy, st);
      const int gi = id.x0 + r;
      // computed for every cell of the tile (the boxes are zero outside the
      // grid); only the stores are guarded
      float4 pvx = make_float4(0.f, 0.f, 0.f, 0.f), pvy = pvx;
      if (has_prev) {
        pvx = *reinterpret_cast<const float4*>(pb + r * kTY + j);
        pvy = *reinterpret_cast<const float4*>(pb + F::kTR * kTY + r * kTY + j);
      }
      float vx[4], vy[4];
      // source box: rows and columns of this thread's 4 cells inside it
      const int sa = gi - ox;
      oper4<MODE == kModeDField>(ks, st, MODE == kModeDField ? w4[q2] : pvx, vx, vy);
      if (has_src && (unsigned)sa < (unsigned)a.bx && gj + 3 >= oy && gj < oy + a.by) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int sb = gj + q - oy;
          if ((unsigned)sb < (unsigned)a.by) {
            const float f = a.src_map[((size_t)id.inst * a.bx + sa) * a.by + sb];  // L + amp f, one rounding
            if (a.src_comp == 0) vx[q] = fmaf(amp, f, vx[q]); else vy[q] = fmaf(amp, f, vy[q]);
          }
        }
      }
      update4(st.cx, st.cy, pvx, pvy, vx, vy);
      if (gi < id.xe && gj < id.ye) {
        const float4 nvx = make_float4(vx[0], vx[1], vx[2], vx[3]);
        const float4 nvy = make_float4(vy[0], vy[1], vy[2], vy[3]);
        const size_t o = (size_t)gi * ny + gj;
        *reinterpret_cast<float4*>(out + o) = nvx;
        *reinterpret_cast<float4*>(out + N + o) = nvy;
        if (a.copy0) {
          *reinterpret_cast<float4*>(a.copy0 + (size_t)id.shot * 2 * N + o) = nvx;
          *reinterpret_cast<float4*>(a.copy0 + (size_t)id.shot * 2 * N + N + o) = nvy;
        }
        if (a.copy1) {
          *reinterpret_cast<float4*>(a.copy1 + (size_t)id.shot * 2 * N + o) = nvx;
          *reinterpret_cast<float4*>(a.copy1 + (size_t)id.shot * 2 * N + N + o) = nvy;
        }
        if (a.frame >= 0) {
          const size_t ho = ((size_t)id.shot * a.nt_out + a.frame) * N + o;
          *reinterpret_cast<float4*>(a.hist_x + ho) = nvx;
          *reinterpret_cast<float4*>(a.hist_y + ho) = nvy;
        }
      }
      shift(wx);
      shift(wy);
    }
    release(done, k, [&] { issue(k + 2); });
  }
  if (tid == 0 && pipe_failed(&guard)) pipe_drain(bar, 2, &guard);
}

// ------------------------------------------------------- two-step forward
// u^{i+1} and u^{i+2} of a tile in one pass (temporal blocking).  The box of
// u^i with a two-cell halo and the box of u^{i-1} with a one-cell halo give
// u^{i+1} on the tile and on a one-cell ring around it (cells outside the
// grid forced to zero: the scheme's ghost ring), kept in shared memory; from
// it and u^i's own cells, u^{i+2} on the tile.  HBM traffic per two steps:
// read u^i and u^{i-1}, write u^{i+1} and u^{i+2} (16 B per cell-step
// instead of 24).  Steps without history frames, checkpoint copies or
// receiver gathers only: the recompute segments of the adjoint.
struct Fwd2Layout {
  static constexpr int kTR = 16;                    // tile rows
  static constexpr int kBH2 = kTR + 4;              // u^i box rows: tile rows -2 .. kTR+1
  static constexpr int kBH1 = kTR + 2;              // u^{i-1} box and u^{i+1} rows: -1 .. kTR
  static constexpr int kCur = 2 * kBH2 * kBW;
  static constexpr int kPrev = 2 * kBH1 * kBW;
  static constexpr int kStage = (kCur + kPrev + 31) / 32 * 32;  // 128-byte multiple
  static constexpr int kMid = 2 * kBH1 * kBW;       // u^{i+1}; one buffer per tile parity
  static constexpr int kQuads = kBW / 4;            // quads per box row
  static constexpr int kItems1 = kBH1 * kQuads;     // first-step quads (18 x 18)
  static constexpr int kCtasPerSm = 3;
};

// Window [b-1 .. b+4] of box row r at box column b (b % 4 == 0), zero beyond
// the box's kBW columns (only the box's first and last columns of u^{i+1}
// depend on those, and the second step never reads them), for a warp whose
// lanes hold consecutive quads of a row:
// the edge cells come from the neighbouring lanes (left_ok / right_ok: the
// lane before / after holds the quad before / after in the same row), so a
// window costs one 16-byte load per lane and the edge loads run only in the
// lanes at the ends of a row or of the warp.  Every lane of the warp calls it.
__device__ __forceinline__ void win_lanes(const float* __restrict__ box, int r, int b, bool left_ok,
                                          bool right_ok, float w[6]) {
  const float* p = box + r * kBW + b;
  const float4 m = *reinterpret_cast<const float4*>(p);
  const float from_left = __shfl_up_sync(0xffffffffu, m.w, 1);
  const float from_right = __shfl_down_sync(0xffffffffu, m.x, 1);
  w[0] = left_ok ? from_left : (b > 0 ? p[-1] : 0.f);
  w[1] = m.x;
  w[2] = m.y;
  w[3] = m.z;
  w[4] = m.w;
  w[5] = right_ok ? from_right : (b + 4 < kBW ? p[4] : 0.f);
}

template <int MODE, bool INST>
__global__ void __launch_bounds__(kThreads, Fwd2Layout::kCtasPerSm)
    tma_fwd2_kernel(const FwdStep a, const __grid_constant__ CUtensorMap cur_map,
                    const __grid_constant__ CUtensorMap prev_map, int tiles_x, int tiles_y, int has_prev,
                    int* err) {
  extern __shared__ float sm_raw[];
  float* sm = aligned128(sm_raw);
  using F = Fwd2Layout;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * F::kStage + 2 * F::kMid);
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny;
  const size_t N = (size_t)nx * ny;
  const int ntiles = INST ? a.inst.ntiles : a.S * tiles_x * tiles_y;
  const uint32_t bytes = (uint32_t)(F::kCur + (has_prev ? F::kPrev : 0)) * 4u;
  grid_dep_trigger();
  __shared__ int done[2];
  __shared__ PipeGuard guard;
  if (tid == 0) {
    prefetch_map(&cur_map);
    prefetch_map(&prev_map);
    bar_init(&bar[0]);
    bar_init(&bar[1]);
    done[0] = done[1] = 0;
    pipe_init(&guard);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  grid_dep_wait();  // the state of the previous step is complete from here on
  const bool has_src = a.bx > 0 && a.by > 0;
  auto issue = [&](int k) {  // loads of this CTA's k-th tile into stage k & 1
    const int t = blockIdx.x + k * gridDim.x;
    if (t >= ntiles || pipe_failed(&guard)) return;
    pipe_issued(&guard, k);
    const TileId id = step_tile<INST, F::kTR>(a.inst, t, tiles_x, tiles_y);
    float* st = sm + (k & 1) * F::kStage;
    fence_async();
    bar_expect(&bar[k & 1], bytes);
    tma_load3(st, &cur_map, id.y0 - 4, id.x0 - 2, 2 * id.shot, &bar[k & 1]);
    if (has_prev) tma_load3(st + F::kCur, &prev_map, id.y0 - 4, id.x0 - 1, 2 * id.shot, &bar[k & 1]);
  };
  if (tid == 0) {
    issue(0);
    issue(1);
  }
  const int qc = tid & 15, rg = tid >> 4;
  const int j = 4 * qc;
  const Coefs ks0 = coefs(a.coef);  // every shot's, unless per-shot constants
  TileWalk<F::kTR> walk;
  walk.init(blockIdx.x, gridDim.x, tiles_x, tiles_y);
  int4 ahead = first_entry<INST>(a.inst, blockIdx.x, ntiles);
  for (int k = 0;; ++k) {
    const int t = blockIdx.x + k * gridDim.x;
    if (t >= ntiles) break;
    const TileId id = walk_tile<INST>(a.inst, t, (int)gridDim.x, ntiles, ahead, walk, nx, ny);
    const Coef* K = a.coef + (size_t)id.inst * a.coef_stride;
    const Coefs ks = a.coef_stride != 0 ? coefs(K) : ks0;
    const float* sig = a.src_signal + (size_t)id.inst * a.nt;
    const float amp1 = sig[a.i] * K->kappa, amp2 = sig[a.i + 1] * K->kappa;
    const int ox = has_src ? a.src_origin[2 * id.inst] : 0, oy = has_src ? a.src_origin[2 * id.inst + 1] : 0;
    const float* smap = has_src ? a.src_map + (size_t)id.inst * a.bx * a.by : nullptr;
    bar_wait_ok(&bar[k & 1], (uint32_t)(k >> 1) & 1u, err, &guard);
    const float* cb = sm + (k & 1) * F::kStage;           // u^i: rows -2 .. kTR+1
    const float* pb = cb + F::kCur;                        // u^{i-1}: rows -1 .. kTR
    float* mid = sm + 2 * F::kStage + (k & 1) * F::kMid;  // u^{i+1}: rows -1 .. kTR
    float* out1 = a.out + (size_t)id.shot * 2 * N;
    float* out2 = a.out2 + (size_t)id.shot * 2 * N;

    // step i: u^{i+1} on rows -1 .. kTR of every box column (box column b is
    // grid column y0 - 4 + b).  Items run warp by warp (every lane takes part
    // in the window shuffles); lanes past the last item compute a copy of it
    // and store nothing.
    const int lane = tid & 31;
    for (int base = tid - lane; base < F::kItems1; base += kThreads) {
      const int it = base + lane;
      const bool valid = it < F::kItems1;
      const int itc = valid ? it : F::kItems1 - 1;
      const int m = itc / F::kQuads, qb = itc - m * F::kQuads, b = 4 * qb;
      const bool left_ok = lane > 0 && qb > 0, right_ok = lane < 31 && qb < F::kQuads - 1 && valid;
      float wx[3][6], wy[3][6];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        win_lanes(cb, m + d, b, left_ok, right_ok, wx[d]);
        win_lanes(cb + F::kBH2 * kBW, m + d, b, left_ok, right_ok, wy[d]);
      }
      Sums4 st;
      sums4<false>(wx, wy, st);
      float4 pvx = make_float4(0.f, 0.f, 0.f, 0.f), pvy = pvx;
      if (has_prev) {
        pvx = *reinterpret_cast<const float4*>(pb + m * kBW + b);
        pvy = *reinterpret_cast<const float4*>(pb + F::kBH1 * kBW + m * kBW + b);
      }
      const int gi = id.x0 + m - 1, gj = id.y0 - 4 + b;  // ny % 4 == 0: a quad is in or out
      const bool inside = gi >= id.xs && gi < id.xe && gj >= id.ys && gj < id.ye;
      float vx[4], vy[4];
      const int sa = gi - ox;
      oper4<false>(ks, st, pvx, vx, vy);
      if (inside && has_src && (unsigned)sa < (unsigned)a.bx && gj + 3 >= oy && gj < oy + a.by) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int sb = gj + q - oy;
          if ((unsigned)sb < (unsigned)a.by) {
            const float f = smap[(size_t)sa * a.by + sb];  // L + amp f, one rounding
            if (a.src_comp == 0) vx[q] = fmaf(amp1, f, vx[q]); else vy[q] = fmaf(amp1, f, vy[q]);
          }
        }
      }
      update4(st.cx, st.cy, pvx, pvy, vx, vy);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        vx[q] = inside ? vx[q] : 0.f;
        vy[q] = inside ? vy[q] : 0.f;
      }
      const float4 nvx = make_float4(vx[0], vx[1], vx[2], vx[3]);
      const float4 nvy = make_float4(vy[0], vy[1], vy[2], vy[3]);
      if (!valid) continue;
      *reinterpret_cast<float4*>(mid + m * kBW + b) = nvx;
      *reinterpret_cast<float4*>(mid + F::kBH1 * kBW + m * kBW + b) = nvy;
      if (inside && m >= 1 && m <= F::kTR && b >= 4 && b < 4 + kTY) {
        const size_t o = (size_t)gi * ny + gj;
        *reinterpret_cast<float4*>(out1 + o) = nvx;
        *reinterpret_cast<float4*>(out1 + N + o) = nvy;
      }
    }
    __syncthreads();  // u^{i+1} complete (and the other buffer's readers are done)

    // step i + 1: u^{i+2} on the tile from u^{i+1} and u^i's own cells
    // (lanes 0-15 and 16-31 of a warp hold the 16 quads of two rows)
    {
      float wx[3][6], wy[3][6];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        win_lanes(mid, rg + d, j + 4, qc > 0, qc < 15, wx[d]);
        win_lanes(mid + F::kBH1 * kBW, rg + d, j + 4, qc > 0, qc < 15, wy[d]);
      }
      Sums4 st;
      sums4(wx, wy, st);
      const float4 pvx = *reinterpret_cast<const float4*>(cb + (rg + 2) * kBW + j + 4);
      const float4 pvy = *reinterpret_cast<const float4*>(cb + F::kBH2 * kBW + (rg + 2) * kBW + j + 4);
      const int gi = id.x0 + rg, gj = id.y0 + j;
      float vx[4], vy[4];
      const int sa = gi - ox;
      oper4<false>(ks, st, pvx, vx, vy);
      if (has_src && (unsigned)sa < (unsigned)a.bx && gj + 3 >= oy && gj < oy + a.by) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int sb = gj + q - oy;
          if ((unsigned)sb < (unsigned)a.by) {
            const float f = smap[(size_t)sa * a.by + sb];  // L + amp f, one rounding
            if (a.src_comp == 0) vx[q] = fmaf(amp2, f, vx[q]); else vy[q] = fmaf(amp2, f, vy[q]);
          }
        }
      }
      update4(st.cx, st.cy, pvx, pvy, vx, vy);
      if (gi < id.xe && gj < id.ye) {
        const size_t o = (size_t)gi * ny + gj;
        *reinterpret_cast<float4*>(out2 + o) = make_float4(vx[0], vx[1], vx[2], vx[3]);
        *reinterpret_cast<float4*>(out2 + N + o) = make_float4(vy[0], vy[1], vy[2], vy[3]);
      }
    }
    release(done, k, [&] { issue(k + 2); });
  }
  if (tid == 0 && pipe_failed(&guard)) pipe_drain(bar, 2, &guard);
}

// ----------------------------------------------------------------- adjoint
// Stage (SCALAR): halo box of lam^{m+1}, own boxes of lam^{m+2} and u^m
// (u^m enters only through its own cells).  The six
// imaging sums sum_cells lam . (dA/dC_k u) are evaluated in the transposed
// form sum_cells u . (dA/dC_k lam): the second differences with zero ghosts
// are symmetric operators, so both forms are the same sum over the grid, and
// the stencils of lam^{m+1} are the ones the update already computed.
// Stage (DFIELD): halo boxes of lam^{m+1}, u^m and D (its imaging is per
// cell, so u's stencils are needed); lam^{m+2} is read into registers
// before the wait (keeps two CTAs per SM within shared memory).
template <int MODE, int TR = (MODE == kModeScalar ? 16 : 32)>
struct AdjLayout {
  // SCALAR: 64 x 16 tiles, one row per thread (80 registers: three CTAs
  // per SM), or 64 x 32 tiles (two rows per thread, two CTAs per SM) as a
  // measured alternative.  DFIELD keeps 64 x 32 tiles and two rows per
  // thread: with one row its three halo windows per output row (lam, u, D)
  // cost more than the third CTA gains (24.4 vs 21.5 us per damage512 step)
  static constexpr int kTR = TR;                               // tile rows
  static constexpr int kRT = kTR / 16;                         // rows per thread
  static constexpr int kBHa = kTR + 2;                         // halo box rows
  static constexpr int kHalo = 2 * kBHa * kBW;
  static constexpr int kOwn = 2 * kTR * kTY;
  static constexpr int kLam = 0;
  static constexpr int kPrev = kHalo;  // SCALAR only
  // u^m: own box after lam^{m+2} (SCALAR), halo box (DFIELD)
  static constexpr int kU = (MODE == kModeScalar) ? kPrev + kOwn : kHalo;
  static constexpr int kD = kU + kHalo;  // DFIELD only
  static constexpr int kEnd = (MODE == kModeScalar) ? kU + kOwn : kD + kBHa * kBW;
  static constexpr int kStage = (kEnd + 31) / 32 * 32;  // 128-byte multiple
  // two stages (one tile in flight while one is computed); three stages at
  // two CTAs per SM measured slower for SCALAR (150 vs 114 us per shots1024
  // step): the kernel needs the third CTA's warps more than a deeper pipeline
  static constexpr int kStages = 2;
  static constexpr int kCtasPerSm = (MODE == kModeScalar && TR == 16) ? 3 : 2;
};

template <int MODE, int TR, bool INST>
__global__ void __launch_bounds__(kThreads, AdjLayout<MODE, TR>::kCtasPerSm)
    tma_adj_kernel(const AdjStep a, const __grid_constant__ CUtensorMap cur_map,
                   const __grid_constant__ CUtensorMap prev_map, const __grid_constant__ CUtensorMap u_map,
                   const __grid_constant__ CUtensorMap d_map, int tiles_x, int tiles_y, int has_u, int* err) {
  using L = AdjLayout<MODE, TR>;
  extern __shared__ float sm_raw[];
  float* sm = aligned128(sm_raw);
  constexpr int NS = L::kStages;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + NS * L::kStage);
  __shared__ double red[kThreads / 32][6];
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny;
  const size_t N = (size_t)nx * ny;
  const int ntiles = INST ? a.inst.ntiles : a.S * tiles_x * tiles_y;
  const uint32_t bytes = (uint32_t)(MODE == kModeScalar
                                        ? L::kHalo + L::kOwn + (has_u ? L::kOwn : 0)
                                        : L::kHalo + L::kBHa * kBW + (has_u ? L::kHalo : 0)) * 4u;
  grid_dep_trigger();
  __shared__ int done[NS];
  __shared__ PipeGuard guard;
  if (tid == 0) {
    prefetch_map(&cur_map);
    prefetch_map(MODE == kModeScalar ? &prev_map : &d_map);
    if (has_u) prefetch_map(&u_map);
    for (int q = 0; q < NS; ++q) {
      bar_init(&bar[q]);
      done[q] = 0;
    }
    pipe_init(&guard);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  grid_dep_wait();  // the state of the previous step is complete from here on
  const float gs = a.coef->gscale;  // one scale for every shot
  // This CTA's tiles: t_first + k t_step below t_end.  Strided over the grid
  // (CTAs working at the same time touch neighbouring tiles, which share
  // halo rows in L2), or, with per-shot constants and imaging, a contiguous
  // chunk: the sums are flushed whenever the list enters another shot, and a
  // strided list would do that at almost every tile.
  const bool per_shot = a.coef_stride != 0;
  const bool chunked = MODE == kModeScalar && per_shot && has_u;
  const int t_first = chunked ? (int)((long long)blockIdx.x * ntiles / gridDim.x) : (int)blockIdx.x;
  const int t_end = chunked ? (int)((long long)(blockIdx.x + 1) * ntiles / gridDim.x) : ntiles;
  const int t_step = chunked ? 1 : (int)gridDim.x;
  auto issue = [&](int k) {
    const int t = t_first + k * t_step;
    if (t >= t_end || pipe_failed(&guard)) return;
    pipe_issued(&guard, k);
    const TileId id = step_tile<INST, L::kTR>(a.inst, t, tiles_x, tiles_y);
    const int sg = k % NS;
    float* st = sm + sg * L::kStage;
    fence_async();
    bar_expect(&bar[sg], bytes);
    tma_load3(st + L::kLam, &cur_map, id.y0 - 4, id.x0 - 1, 2 * id.shot, &bar[sg]);
    if (MODE == kModeScalar)
      tma_load3(st + L::kPrev, &prev_map, id.y0, id.x0, 2 * id.shot, &bar[sg]);
    else
      tma_load2(st + L::kD, &d_map, id.y0 - 4, id.x0 - 1, &bar[sg]);
    if (has_u) {
      if (MODE == kModeScalar) tma_load3(st + L::kU, &u_map, id.y0, id.x0, 2 * id.shot, &bar[sg]);
      else tma_load3(st + L::kU, &u_map, id.y0 - 4, id.x0 - 1, 2 * id.shot, &bar[sg]);
    }
  };
  if (tid == 0)
    for (int q = 0; q < NS; ++q) issue(q);
  const int qc = tid & 15, rg = tid >> 4;
  const int j = 4 * qc;
  const bool inject = a.frame >= 0 && a.record == kRecordReceivers;
  // imaging sums (SCALAR): FP32 over a thread's 8 cells of a tile,
  // accumulated over tiles as FP32 pairs (TwoSum), FP64 across threads and
  // launches.  Partial row: blockIdx.x; with per-shot constants
  // shot * kTiledRowsPerShot + blockIdx.x, flushed when the CTA's
  // tile list moves on to the next shot (shots never recur: t increases).
  // (the FP32 sums of a thread's cells, two lanes of packed sums, are folded
  // into the pair every four tiles and before a flush)
  float hi[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, lo[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float2 acc[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) acc[q] = dup2(0.f);
  auto fold = [&] {
#pragma unroll
    for (int q = 0; q < 6; ++q) {  // TwoSum(hi, acc)
      const float a = acc[q].x + acc[q].y;
      const float s = hi[q] + a;
      const float bp = s - hi[q];
      lo[q] += (hi[q] - (s - bp)) + (a - bp);
      hi[q] = s;
      acc[q] = dup2(0.f);
    }
  };
  int acc_shot = -1;
  auto flush = [&](int shot) {  // CTA-uniform: every warp calls it at the same point
    fold();
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      double v = (double)hi[q] + (double)lo[q];
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (lane == 0) red[warp][q] = v;
      hi[q] = 0.f;
      lo[q] = 0.f;
    }
    __syncthreads();
    if (tid < 6) {
      double v = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) v += red[w][tid];
      const size_t row = per_shot ? (size_t)shot * kTiledRowsPerShot + blockIdx.x : blockIdx.x;
      a.partials[row * 8 + tid] += v;
    }
    __syncthreads();  // red is free again
  };
  const Coefs ks0 = coefs(a.coef);  // every shot's, unless per-shot constants
  TileWalk<L::kTR> walk;
  walk.init(t_first, t_step, tiles_x, tiles_y);
  // (table entries loaded when a tile starts: one ahead measured the same
  // here and needs registers this kernel does not have)
  for (int k = 0;; ++k) {
    const int t = t_first + k * t_step;
    if (t >= t_end) break;
    TileId id;
    if constexpr (INST) {
      id = table_tile(a.inst, t);
    } else {
      id = grid_tile(walk.id(), nx, ny);
      walk.next();
    }
    if (MODE == kModeScalar && per_shot && has_u && id.inst != acc_shot) {
      if (acc_shot >= 0) flush(acc_shot);
      acc_shot = id.inst;
    }
    const Coefs ks = per_shot ? coefs(a.coef + (size_t)id.inst * a.coef_stride) : ks0;
    const int gj = id.y0 + j;
    const int r0 = L::kRT * rg;
    // receivers in this tile (uniform over the CTA): the injection and its
    // barriers only run where the per-call table says there are some
    const bool tile_inject = inject && (a.tile_flags == nullptr || a.tile_flags[t] != 0);
    float4 pv[L::kRT][2];  // DFIELD: lam^{m+2} of the thread's rows (x, y)
    if (MODE == kModeDField) {
#pragma unroll
      for (int q2 = 0; q2 < L::kRT; ++q2) {
        const int gi = id.x0 + r0 + q2;
        const size_t o = (size_t)id.shot * 2 * N + (size_t)gi * ny + gj;
        const bool in = gi < nx && gj < ny;
        pv[q2][0] = in ? *reinterpret_cast<const float4*>(a.prev + o) : make_float4(0.f, 0.f, 0.f, 0.f);
        pv[q2][1] = in ? *reinterpret_cast<const float4*>(a.prev + N + o) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    const int stage = k % NS;
    bar_wait_ok(&bar[stage], (uint32_t)(k / NS) & 1u, err, &guard);
    float* hb = sm + stage * L::kStage;
    float* pb = hb + L::kPrev;
    const float* ub = hb + L::kU;
    const float* db = hb + L::kD;
    // adjoint source at receiver cells (SCALAR): subtract it from this
    // tile's copy of lam^{m+2} (lam^m = ... - lam^{m+2} + ... + g)
    if (MODE == kModeScalar && tile_inject) {
      for (int rr = tid; rr < a.nrec; rr += kThreads) {
        const int32_t idx = a.rec_idx[(size_t)id.inst * a.nrec + rr];
        if (idx < 0 || (size_t)idx >= N) continue;
        const int gi = idx / ny, gjj = idx - gi * ny;
        if (gi >= id.x0 && gi < id.x0 + L::kTR && gjj >= id.y0 && gjj < id.y0 + kTY) {
          const size_t go = ((size_t)id.inst * a.nt_out + a.frame) * a.nrec + rr;
          atomicAdd(&pb[(gi - id.x0) * kTY + (gjj - id.y0)], -gs * a.g_x[go]);
          atomicAdd(&pb[L::kTR * kTY + (gi - id.x0) * kTY + (gjj - id.y0)], -gs * a.g_y[go]);
        }
      }
      __syncthreads();
    }
    float* out = a.out + (size_t)id.shot * 2 * N;
    // lam windows for the stencils: weighted by 1 - D in DFIELD (A^T lam =
    // A0((1 - D) lam)); the centre value itself stays unweighted
    auto lam_win = [&](int r, float wx_[6], float wy_[6]) {
      win(hb, r, j, wx_);
      win(hb + L::kBHa * kBW, r, j, wy_);
      if (MODE == kModeDField) {
        float dw[6];
        win(db, r, j, dw);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const float w = 1.f - dw[c];
          wx_[c] = w * wx_[c];
          wy_[c] = w * wy_[c];
        }
      }
    };
    float wx[3][6], wy[3][6], vx_[3][6], vy_[3][6];
    lam_win(r0, wx[0], wy[0]);
    lam_win(r0 + 1, wx[1], wy[1]);
    if (MODE == kModeDField && has_u) {
      win(ub, r0, j, vx_[0]);
      win(ub + L::kBHa * kBW, r0, j, vy_[0]);
      win(ub, r0 + 1, j, vx_[1]);
      win(ub + L::kBHa * kBW, r0 + 1, j, vy_[1]);
    }
#pragma unroll
    for (int q2 = 0; q2 < L::kRT; ++q2) {
      const int r = r0 + q2;
      lam_win(r + 2, wx[2], wy[2]);
      Sums4 st;
      sums4(wx, wy, st);
      const int gi = id.x0 + r;
      // the cells of the tile inside its instance's region (the whole grid
      // without instances; ny % 4 == 0: a quad is in or out)
      const bool in = gi < id.xe && gj < id.ye;
      // unweighted lam^{m+1} at the 4 cells (zero outside the grid, so the
      // imaging products of those cells vanish without a guard)
      float c1x[4], c1y[4];
      if (MODE == kModeScalar) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          c1x[q] = st.cx[q];
          c1y[q] = st.cy[q];
        }
      } else {
        const float4 cx4 = *reinterpret_cast<const float4*>(hb + (r + 1) * kBW + j + 4);
        const float4 cy4 = *reinterpret_cast<const float4*>(hb + L::kBHa * kBW + (r + 1) * kBW + j + 4);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          c1x[q] = g4(cx4, q);
          c1y[q] = g4(cy4, q);
        }
      }
      const size_t o = (size_t)gi * ny + gj;
      float4 pvx, pvy;
      if (MODE == kModeScalar) {
        pvx = *reinterpret_cast<const float4*>(pb + r * kTY + j);
        pvy = *reinterpret_cast<const float4*>(pb + L::kTR * kTY + r * kTY + j);
      } else {
        pvx = pv[q2][0];
        pvy = pv[q2][1];
      }
      float vx[4], vy[4];
      leap4<false>(ks, st, c1x, c1y, pvx, pvy, pvx, vx, vy);
      if (in) {
        if (a.frame >= 0 && a.record == kRecordFields) {
          const size_t go = ((size_t)id.shot * a.nt_out + a.frame) * N + o;
          const float4 gx = *reinterpret_cast<const float4*>(a.g_x + go);
          const float4 gy = *reinterpret_cast<const float4*>(a.g_y + go);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            vx[q] += gs * g4(gx, q);
            vy[q] += gs * g4(gy, q);
          }
        }
        *reinterpret_cast<float4*>(out + o) = make_float4(vx[0], vx[1], vx[2], vx[3]);
        *reinterpret_cast<float4*>(out + N + o) = make_float4(vy[0], vy[1], vy[2], vy[3]);
      }
      if (MODE == kModeScalar && has_u) {
        // transposed imaging: u^m at the cell times the stencils of lam^{m+1}
        // (cells of a tile beyond its instance's region take no part: on a
        // canvas they may hold another instance's state)
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 u4x = in ? *reinterpret_cast<const float4*>(ub + r * kTY + j) : zero4;
        const float4 u4y = in ? *reinterpret_cast<const float4*>(ub + L::kTR * kTY + r * kTY + j) : zero4;
#pragma unroll
        for (int p = 0; p < 2; ++p) {  // each sum as a chain of fused multiply-adds, two cells per op
          const float2 ux = pair4(u4x, p), uy = pair4(u4y, p);
          const float2 xx_x = pair(st.xx_x, p), yy_x = pair(st.yy_x, p), xy_x = pair(st.xy_x, p);
          const float2 xx_y = pair(st.xx_y, p), yy_y = pair(st.yy_y, p), xy_y = pair(st.xy_y, p);
          acc[0] = fma2(ux, xx_x, acc[0]);
          acc[1] = fma2(uy, yy_y, acc[1]);
          acc[2] = fma2(ux, xy_y, fma2(uy, xy_x, acc[2]));
          acc[3] = fma2(uy, xx_x, fma2(ux, fma2(dup2(0.5f), xy_x, xx_y), acc[3]));
          acc[4] = fma2(ux, yy_y, fma2(uy, fma2(dup2(0.5f), xy_y, yy_x), acc[4]));
          acc[5] = fma2(uy, xx_y, fma2(ux, yy_x, acc[5]));
        }
      }
      if (MODE == kModeDField && has_u) {
        win(ub, r + 2, j, vx_[2]);
        win(ub + L::kBHa * kBW, r + 2, j, vy_[2]);
        Sums4 su;
        sums4(vx_, vy_, su);
        if (in) {
          float* ga = a.gacc + (size_t)id.shot * N + o;
          float4 g = *reinterpret_cast<const float4*>(ga);
          float gv[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            float Lx, Ly;
            apply(ks, su, q, Lx, Ly);
            gv[q] += c1x[q] * Lx + c1y[q] * Ly;
          }
          *reinterpret_cast<float4*>(ga) = make_float4(gv[0], gv[1], gv[2], gv[3]);
        }
        shift(vx_);
        shift(vy_);
      }
      shift(wx);
      shift(wy);
    }
    if (MODE == kModeScalar && (k & 3) == 3) fold();
    if (MODE == kModeDField && tile_inject) {
      // adjoint source at receiver cells, added to the stored lam^m (several
      // receivers may share a cell); the block's own stores are visible
      // after the barrier
      __syncthreads();
      for (int rr = tid; rr < a.nrec; rr += kThreads) {
        const int32_t idx = a.rec_idx[(size_t)id.shot * a.nrec + rr];
        if (idx < 0 || (size_t)idx >= N) continue;
        const int gi = idx / ny, gjj = idx - gi * ny;
        if (gi >= id.x0 && gi < id.x0 + L::kTR && gjj >= id.y0 && gjj < id.y0 + kTY) {
          const size_t go = ((size_t)id.shot * a.nt_out + a.frame) * a.nrec + rr;
          atomicAdd(out + idx, gs * a.g_x[go]);
          atomicAdd(out + N + idx, gs * a.g_y[go]);
        }
      }
    }
    release_stage(done, stage, [&] { issue(k + NS); });
  }
  if (tid == 0 && pipe_failed(&guard)) pipe_drain(bar, NS, &guard);
  if (MODE != kModeScalar || !has_u) return;
  flush(per_shot ? acc_shot : 0);
}

// ------------------------------------------------------ wait self-test
// One thread waits on an mbarrier that nothing arrives at (no copy is in
// flight towards this CTA), through the same bounded wait as the tile loop.
__global__ void wait_selftest_kernel(int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    bar_init(&bar);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    bar_wait(&bar, 0u, status);
  }
}

__device__ int g_selftest_status;

// Receiver table of the tiled adjoint: flags[(shot, tile)] = 1 where the
// shot has a receiver in the tile.
__global__ void tile_flags_kernel(const int32_t* __restrict__ rec_idx, int S, int nrec, int nx, int ny,
                                  int tile_rows, int tiles_x, int tiles_y, uint8_t* __restrict__ flags) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= S * nrec) return;
  const int s = e / nrec;
  const int32_t idx = rec_idx[e];
  if (idx < 0 || (int64_t)idx >= (int64_t)nx * ny) return;  // ignored, as in the kernels
  const int gi = idx / ny, gj = idx - gi * ny;
  flags[(size_t)s * tiles_x * tiles_y + (size_t)(gi / tile_rows) * tiles_y + gj / kTY] = 1;
}

// ----------------------------------------------------------------- host
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::mutex mu;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (fn == nullptr) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Tensor map over S shots of [comp][nx][ny] floats: dims (ny, nx, 2 S).
bool make_map(CUtensorMap* m, const float* base, int nx, int ny, int S, int bw, int bh) {
  auto fn = encode_fn();
  if (fn == nullptr || base == nullptr) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)ny, (cuuint64_t)nx, (cuuint64_t)2 * S};
  const cuuint64_t strides[2] = {(cuuint64_t)ny * 4, (cuuint64_t)nx * ny * 4};
  const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 2};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
  }
  return n;
}

// Tensor map over the degradation plane [nx][ny]: dims (ny, nx).
bool make_map2(CUtensorMap* m, const float* base, int nx, int ny, int bw, int bh) {
  auto fn = encode_fn();
  if (fn == nullptr || base == nullptr) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)ny, (cuuint64_t)nx};
  const cuuint64_t strides[1] = {(cuuint64_t)ny * 4};
  const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int TR>
constexpr size_t fwd_smem() {
  return 2 * (size_t)FwdLayoutT<TR>::kStage * 4 + 16 + 128;
}
constexpr size_t kFwd2Smem = (2 * (size_t)Fwd2Layout::kStage + 2 * (size_t)Fwd2Layout::kMid) * 4 + 16 + 128;
template <int MODE, int TR = (MODE == kModeScalar ? 16 : 32)>
constexpr size_t adj_smem() {
  using L = AdjLayout<MODE, TR>;
  return (size_t)L::kStages * L::kStage * 4 + 8 * L::kStages + 128;
}

cudaError_t set_smem() {
  static std::once_flag once;
  static cudaError_t result = cudaSuccess;
  std::call_once(once, [] {
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e[11] = {
        cudaFuncSetAttribute(tma_fwd_kernel<kModeScalar, 16, false>, at, (int)fwd_smem<16>()),
        cudaFuncSetAttribute(tma_fwd_kernel<kModeDField, 16, false>, at, (int)fwd_smem<16>()),
        cudaFuncSetAttribute(tma_fwd_kernel<kModeScalar, 32, false>, at, (int)fwd_smem<32>()),
        cudaFuncSetAttribute(tma_fwd_kernel<kModeDField, 32, false>, at, (int)fwd_smem<32>()),
        cudaFuncSetAttribute(tma_fwd_kernel<kModeScalar, 16, true>, at, (int)fwd_smem<16>()),
        cudaFuncSetAttribute(tma_fwd2_kernel<kModeScalar, false>, at, (int)kFwd2Smem),
        cudaFuncSetAttribute(tma_fwd2_kernel<kModeScalar, true>, at, (int)kFwd2Smem),
        cudaFuncSetAttribute(tma_adj_kernel<kModeScalar, 16, false>, at, (int)adj_smem<kModeScalar, 16>()),
        cudaFuncSetAttribute(tma_adj_kernel<kModeScalar, 32, false>, at, (int)adj_smem<kModeScalar, 32>()),
        cudaFuncSetAttribute(tma_adj_kernel<kModeDField, 32, false>, at, (int)adj_smem<kModeDField, 32>()),
        cudaFuncSetAttribute(tma_adj_kernel<kModeScalar, 16, true>, at, (int)adj_smem<kModeScalar, 16>())};
    for (cudaError_t x : e)
      if (x != cudaSuccess) result = x;
  });
  return result;
}

}  // namespace

cudaError_t wait_selftest(int* status_host, cudaStream_t st) {
  const int zero = 0;
  cudaError_t e = cudaMemcpyToSymbolAsync(g_selftest_status, &zero, sizeof(int), 0,
                                          cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  int* dev_status = nullptr;
  if ((e = cudaGetSymbolAddress(reinterpret_cast<void**>(&dev_status), g_selftest_status)) != cudaSuccess)
    return e;
  if ((e = tracked_launch(kProfOther, st, [&] { wait_selftest_kernel<<<1, 32, 0, st>>>(dev_status); })) !=
      cudaSuccess)
    return e;
  if ((e = cudaMemcpyFromSymbolAsync(status_host, g_selftest_status, sizeof(int), 0,
                                     cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  return cudaStreamSynchronize(st);
}

cudaError_t launch_tile_flags(int mode, const int32_t* rec_idx, int S, int nrec, int nx, int ny,
                              uint8_t* flags, cudaStream_t st, int tile_rows) {
  const int tr = tma_adj_tile_rows(mode, tile_rows);
  const int tiles_x = (nx + tr - 1) / tr, tiles_y = (ny + kTY - 1) / kTY;
  cudaError_t e = cudaMemsetAsync(flags, 0, tma_tiles(nx, ny, S, tr), st);
  if (e != cudaSuccess) return e;
  const int n = S * nrec;
  return tracked_launch(kProfOther, st, [&] {
    tile_flags_kernel<<<(n + 255) / 256, 256, 0, st>>>(rec_idx, S, nrec, nx, ny, tr, tiles_x, tiles_y,
                                                         flags);
  });
}

namespace {
// Block b writes the tiles of instance d.id[b] (entry base[b] + xt * tiles_y
// + yt for the tile at rows x0 + 16 xt, columns y0 + 64 yt) and its box.
__global__ void inst_table_kernel(const InstDesc d, int4* __restrict__ tiles, int4* __restrict__ box) {
  const int b = blockIdx.x;
  const int k = d.id[b];
  const int tiles_y = (d.ny[b] + 63) / 64;
  const int n = inst_tiles(d.nx[b], d.ny[b]);
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int xt = t / tiles_y, yt = t - xt * tiles_y;
    // the entry: instance, tile origin, instance region (16-bit pairs)
    const unsigned rx = (unsigned)(d.x0[b] + kInstTileRows * xt), ry = (unsigned)(d.y0[b] + 64 * yt);
    const unsigned xs = (unsigned)d.x0[b], ys = (unsigned)d.y0[b];
    const unsigned xe = xs + (unsigned)d.nx[b], ye = ys + (unsigned)d.ny[b];
    tiles[d.base[b] + t] = make_int4(k, (int)(rx | (ry << 16)), (int)(xs | (ys << 16)), (int)(xe | (ye << 16)));
  }
  if (threadIdx.x == 0) {
    box[2 * k] = make_int4(d.x0[b], d.y0[b], d.x0[b] + d.nx[b], d.y0[b] + d.ny[b]);
    box[2 * k + 1] = make_int4(d.base[b], tiles_y, d.nt[b], 0);
  }
}

__global__ void inst_tile_flags_kernel(const int32_t* __restrict__ rec_idx, int S, int nrec, int ny,
                                       const int4* __restrict__ box, uint8_t* __restrict__ flags) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= S * nrec) return;
  const int s = e / nrec;
  const int32_t idx = rec_idx[e];
  if (idx < 0) return;
  const int gi = idx / ny, gj = idx - gi * ny;
  const int4 r = box[2 * s], m = box[2 * s + 1];
  if (gi < r.x || gi >= r.z || gj < r.y || gj >= r.w) return;
  flags[m.x + ((gi - r.x) / kInstTileRows) * m.y + (gj - r.y) / 64] = 1;
}
}  // namespace

namespace {
// Block (k, s0) zeroes instance k's ghost ring in states s0, s0 + gridDim.y,
// ...: the rows above and below the region (corners included) and the
// columns left and right of it, clipped to the canvas.
__global__ void inst_ring_zero_kernel(float* __restrict__ base, size_t slot_floats, int nslots, int nx, int ny,
                                      const int4* __restrict__ box) {
  const int4 r = box[2 * blockIdx.x];  // region [r.x, r.z) x [r.y, r.w)
  const int W = r.w - r.y + 2, H = r.z - r.x;
  const size_t N = (size_t)nx * ny;
  const int n = 2 * W + 2 * H;
  for (int s = blockIdx.y; s < nslots; s += gridDim.y) {
    float* p = base + (size_t)s * slot_floats;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      int gi, gj;
      if (e < 2 * W) {
        gi = e < W ? r.x - 1 : r.z;
        gj = r.y - 1 + (e < W ? e : e - W);
      } else {
        const int f = e - 2 * W;
        gi = r.x + (f < H ? f : f - H);
        gj = f < H ? r.y - 1 : r.w;
      }
      if (gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
      const size_t o = (size_t)gi * ny + gj;
      p[o] = 0.f;
      p[N + o] = 0.f;
    }
  }
}
}  // namespace

cudaError_t launch_inst_ring_zero(float* base, size_t slot_floats, int nslots, int nx, int ny, const int4* box,
                                  int count, cudaStream_t st) {
  if (count < 1 || nslots < 1) return cudaSuccess;
  const dim3 grid((unsigned)count, (unsigned)(nslots < 1024 ? nslots : 1024));
  return tracked_launch(kProfOther, st, [&] {
    inst_ring_zero_kernel<<<grid, 256, 0, st>>>(base, slot_floats, nslots, nx, ny, box);
  });
}

cudaError_t launch_inst_table(const InstDesc& d, int4* tiles, int4* box, cudaStream_t st) {
  if (d.count < 1) return cudaSuccess;
  return tracked_launch(kProfOther, st, [&] { inst_table_kernel<<<d.count, 256, 0, st>>>(d, tiles, box); });
}

cudaError_t launch_inst_tile_flags(const int32_t* rec_idx, int S, int nrec, int ny, const int4* box,
                                   uint8_t* flags, int ntiles, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(flags, 0, (size_t)ntiles, st);
  if (e != cudaSuccess) return e;
  const int n = S * nrec;
  return tracked_launch(kProfOther, st, [&] {
    inst_tile_flags_kernel<<<(n + 255) / 256, 256, 0, st>>>(rec_idx, S, nrec, ny, box, flags);
  });
}

bool tma_eligible(int mode, int nx, int ny, int S) {
  (void)nx;
  (void)S;
  return (mode == kModeScalar || mode == kModeDField) && ny % 4 == 0 && encode_fn() != nullptr;
}

size_t tma_tiles(int nx, int ny, int S, int tile_rows) {
  return (size_t)S * ((nx + tile_rows - 1) / tile_rows) * ((ny + kTY - 1) / kTY);
}

int tma_adj_tile_rows(int mode, int tile_rows) {
  return mode == kModeScalar ? (tile_rows == 32 ? 32 : 16) : AdjLayout<kModeDField>::kTR;
}

namespace {
inline bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// CTAs of a persistent launch over `ntiles` tiles with room for `slots`
// resident CTAs: every slot.  (Spreading the tiles evenly over the fewest
// CTAs of the same number of waves measured slower, damage512 81.7 -> 88.8
// ms and multi64 734 -> 737 ms: the memory-bound kernels lose more to the
// fewer CTAs in flight than the last partial wave costs.)
inline int persistent_grid(int ntiles, int slots) { return ntiles < slots ? ntiles : slots; }
}  // namespace

// Steps the tiled kernels cannot take (u^i == 0 at the first step, buffers
// not on 16-byte boundaries) run on the first per-step kernels instead.
// Launch overlap of the tiled kernels.  Their grids fill every SM (one
// CTA per resident slot), so a dependent grid cannot start early on an SM
// that is still busy; measured on a GB300 in graph replay, chaining the
// scalar-constant kernels gains 1 % (1024^2 x 16 shots: 935 -> 926 ms per
// iteration) and chaining the D-field kernels loses 7 % (512^2 x 8 shots:
// 82.0 -> 88.6 ms, all of it in the adjoint).  Only the former are chained.
static bool chain_tiled(int mode) { return mode == kModeScalar; }

bool tma_fwd2_would_run(int mode, const FwdStep& a) {
  return mode == kModeScalar && a.cur != nullptr && a.out2 != nullptr && a.ny % 4 == 0 &&
         a.frame < 0 && a.gframe < 0 && a.copy0 == nullptr && a.copy1 == nullptr && al16(a.cur) &&
         al16(a.prev) && al16(a.out) && al16(a.out2) && encode_fn() != nullptr;
}

cudaError_t launch_tma_fwd2(int mode, const FwdStep& a, int* err, cudaStream_t st) {
  using F = Fwd2Layout;
  CUtensorMap cur_map, prev_map;
  const int planes = a.inst.tiles ? 1 : a.S;  // instances share one canvas plane
  if (!tma_fwd2_would_run(mode, a) || !make_map(&cur_map, a.cur, a.nx, a.ny, planes, kBW, F::kBH2) ||
      !make_map(&prev_map, a.prev ? a.prev : a.cur, a.nx, a.ny, planes, kBW, F::kBH1))
    return cudaErrorNotSupported;
  cudaError_t e = set_smem();
  if (e != cudaSuccess) return e;
  const int tiles_x = (a.nx + F::kTR - 1) / F::kTR, tiles_y = (a.ny + kTY - 1) / kTY;
  const int ntiles = a.inst.tiles ? a.inst.ntiles : a.S * tiles_x * tiles_y;
  const int grid = persistent_grid(ntiles, num_sms() * F::kCtasPerSm);
  const int hp = a.prev ? 1 : 0;
  const bool chained = a.chained != 0 && chain_tiled(mode);
  return tracked_launch(kProfForward, st, [&] {
    if (a.inst.tiles)
      launch_step_kernel(tma_fwd2_kernel<kModeScalar, true>, dim3(grid), dim3(kThreads), kFwd2Smem, st, chained,
                         a, cur_map, prev_map, tiles_x, tiles_y, hp, err);
    else
      launch_step_kernel(tma_fwd2_kernel<kModeScalar, false>, dim3(grid), dim3(kThreads), kFwd2Smem, st, chained,
                         a, cur_map, prev_map, tiles_x, tiles_y, hp, err);
  }, 2.0 * (a.inst.tiles ? (double)a.inst.ntiles * F::kTR * kTY : (double)a.S * a.nx * a.ny) * 16.0);
}

namespace {
template <int TR, bool INST>
cudaError_t launch_tma_fwd_t(int mode, const FwdStep& a, int* err, cudaStream_t st) {
  using F = FwdLayoutT<TR>;
  if (INST && mode != kModeScalar) return cudaErrorNotSupported;
  const bool ok = (mode == kModeScalar || (mode == kModeDField && al16(a.field))) && a.cur != nullptr &&
                  a.ny % 4 == 0 && al16(a.cur) && al16(a.prev) && al16(a.out) && al16(a.copy0) &&
                  al16(a.copy1) && (a.frame < 0 || (al16(a.hist_x) && al16(a.hist_y)));
  CUtensorMap cur_map, prev_map;
  const int planes = INST ? 1 : a.S;  // instances share one canvas plane
  if (!ok || !make_map(&cur_map, a.cur, a.nx, a.ny, planes, kBW, F::kBHa) ||
      !make_map(&prev_map, a.prev ? a.prev : a.cur, a.nx, a.ny, planes, kTY, F::kTR))
    return INST ? cudaErrorNotSupported : launch_fwd_step(mode, a, st);
  cudaError_t e = set_smem();
  if (e != cudaSuccess) return e;
  const int tiles_x = (a.nx + F::kTR - 1) / F::kTR, tiles_y = (a.ny + kTY - 1) / kTY;
  const int ntiles = INST ? a.inst.ntiles : a.S * tiles_x * tiles_y;
  const int grid = persistent_grid(ntiles, num_sms() * F::kCtasPerSm);
  const double cells = INST ? (double)a.inst.ntiles * F::kTR * kTY : (double)a.S * a.nx * a.ny;
  const int hp = a.prev ? 1 : 0;
  const bool chained = a.chained != 0 && chain_tiled(mode);
  return tracked_launch(kProfForward, st, [&] {
    if constexpr (INST)  // scalar constants only (checked above)
      launch_step_kernel(tma_fwd_kernel<kModeScalar, TR, true>, grid, dim3(kThreads), fwd_smem<TR>(), st,
                         chained, a, cur_map, prev_map, tiles_x, tiles_y, hp, err);
    else if (mode == kModeScalar)
      launch_step_kernel(tma_fwd_kernel<kModeScalar, TR, false>, grid, dim3(kThreads), fwd_smem<TR>(), st,
                         chained, a, cur_map, prev_map, tiles_x, tiles_y, hp, err);
    else
      launch_step_kernel(tma_fwd_kernel<kModeDField, TR, false>, grid, dim3(kThreads), fwd_smem<TR>(), st,
                         chained, a, cur_map, prev_map, tiles_x, tiles_y, hp, err);
  }, cells * alg_bytes_forward(mode));
}
}  // namespace

cudaError_t launch_tma_fwd(int mode, const FwdStep& a, int* err, cudaStream_t st) {
  // the instance tile table holds 16-row tiles
  if (a.inst.tiles != nullptr) return launch_tma_fwd_t<16, true>(mode, a, err, st);
  if (a.tile_rows == 32) return launch_tma_fwd_t<32, false>(mode, a, err, st);
  return launch_tma_fwd_t<16, false>(mode, a, err, st);
}

namespace {
bool adj_maps(int mode, const AdjStep& a, CUtensorMap* cur_map, CUtensorMap* prev_map, CUtensorMap* u_map,
              CUtensorMap* d_map) {
  const bool dfield = mode == kModeDField;
  const bool ok = (mode == kModeScalar || (dfield && al16(a.field) && al16(a.gacc))) && a.ny % 4 == 0 &&
                  a.cur != nullptr && a.prev != nullptr && al16(a.cur) && al16(a.prev) && al16(a.out) &&
                  al16(a.u) && (a.record != kRecordFields || (al16(a.g_x) && al16(a.g_y)));
  const int tr = tma_adj_tile_rows(mode, a.inst.tiles ? 16 : a.tile_rows), bh = tr + 2;
  const int planes = a.inst.tiles ? 1 : a.S;  // instances share one canvas plane
  return ok && make_map(cur_map, a.cur, a.nx, a.ny, planes, kBW, bh) &&
         make_map(prev_map, a.prev, a.nx, a.ny, planes, kTY, tr) &&
         make_map(u_map, a.u ? a.u : a.cur, a.nx, a.ny, planes, dfield ? kBW : kTY, dfield ? bh : tr) &&
         make_map2(d_map, dfield ? a.field : a.cur, a.nx, a.ny, kBW, bh);
}
}  // namespace

bool tma_adj_would_run(int mode, const AdjStep& a) {
  CUtensorMap m[4];
  return adj_maps(mode, a, &m[0], &m[1], &m[2], &m[3]);
}

cudaError_t launch_tma_adj(int mode, const AdjStep& a, int* err, cudaStream_t st) {
  const bool dfield = mode == kModeDField;
  if (a.inst.tiles && dfield) return cudaErrorNotSupported;
  CUtensorMap cur_map, prev_map, u_map, d_map;
  if (!adj_maps(mode, a, &cur_map, &prev_map, &u_map, &d_map))
    return a.inst.tiles ? cudaErrorNotSupported : launch_adj_step(mode, a, st);
  cudaError_t e = set_smem();
  if (e != cudaSuccess) return e;
  const int tr = tma_adj_tile_rows(mode, a.inst.tiles ? 16 : a.tile_rows);
  const int tiles_x = (a.nx + tr - 1) / tr, tiles_y = (a.ny + kTY - 1) / kTY;
  const int ntiles = a.inst.tiles ? a.inst.ntiles : a.S * tiles_x * tiles_y;
  int slots = num_sms() * (dfield ? AdjLayout<kModeDField>::kCtasPerSm
                                  : (tr == 32 ? AdjLayout<kModeScalar, 32>::kCtasPerSm
                                              : AdjLayout<kModeScalar, 16>::kCtasPerSm));
  if (slots > kTiledRowsPerShot) slots = kTiledRowsPerShot;  // one partial row per CTA
  const int grid = persistent_grid(ntiles, slots);
  const double cells = a.inst.tiles ? (double)a.inst.ntiles * tr * kTY : (double)a.S * a.nx * a.ny;
  const int hu = a.u ? 1 : 0;
  const bool chained = a.chained != 0 && chain_tiled(mode);
  return tracked_launch(kProfAdjoint, st, [&] {
    if (a.inst.tiles)  // scalar constants, 16-row tiles (checked by the planner)
      launch_step_kernel(tma_adj_kernel<kModeScalar, 16, true>, grid, dim3(kThreads),
                         adj_smem<kModeScalar, 16>(), st, chained, a, cur_map, prev_map, u_map, d_map, tiles_x,
                         tiles_y, hu, err);
    else if (dfield)
      launch_step_kernel(tma_adj_kernel<kModeDField, 32, false>, grid, dim3(kThreads),
                         adj_smem<kModeDField, 32>(), st, chained, a, cur_map, prev_map, u_map, d_map, tiles_x,
                         tiles_y, hu, err);
    else if (tr == 32)
      launch_step_kernel(tma_adj_kernel<kModeScalar, 32, false>, grid, dim3(kThreads),
                         adj_smem<kModeScalar, 32>(), st, chained, a, cur_map, prev_map, u_map, d_map, tiles_x,
                         tiles_y, hu, err);
    else
      launch_step_kernel(tma_adj_kernel<kModeScalar, 16, false>, grid, dim3(kThreads),
                         adj_smem<kModeScalar, 16>(), st, chained, a, cur_map, prev_map, u_map, d_map, tiles_x,
                         tiles_y, hu, err);
  }, cells * alg_bytes_adjoint(mode));
}

}  // namespace ernn
