// Cluster-resident time loop (sm_103a): one thread-block cluster of CL CTAs
// per shot keeps the shot's whole wavefield in distributed shared memory for
// every step of a launch.
//
// Partition: CTA c of the cluster owns grid rows [c R, c R + R) (x), all ny
// columns.  Its shared memory holds a ring of three levels of the field with
// one halo row above and below, L[level][comp][R + 2][ny], and the CTA's
// force map.  Step t reads level t % 3 and writes level (t + 1) % 3 over the
// level before it (each thread reads its own cells of that level first).
// One step: a thread computes (column quad, row chunk) units; the interior
// rows first (they read only this CTA's rows), then a bounded wait on the
// level's mbarrier for the neighbours' boundary rows, then the first and
// last row, which go into the neighbours' halo rows of the next level as
// st.async stores completing transaction bytes on the neighbour's mbarrier
// of that level.  No cluster barrier per step: waiting for the neighbours'
// rows of level t means they have finished step t - 2, the last reader of
// the level this CTA's pushes overwrite.  States that must reach global
// memory leave through TMA bulk copies.
//
// A launch runs up to three roles, selected by blockIdx.z:
//   FWD  steps i0..i1-1 of the forward recursion (the forward pass, or the
//        recomputation of a checkpoint segment into a segment buffer);
//   LAM  steps m_hi..m_lo+1 of the adjoint recursion, which needs no forward
//        state, storing every lam it produces into a lam buffer;
//   IMG  the imaging condition of the previous segment: products of
//        lam^{n+1} with the stencils of u^n, independent across n and cells,
//        spread over all remaining SMs.
// Within a launch the roles share no data, so no cluster waits on another.
//
// Scalar constants only (the per-cell modes use the per-step kernels).
#include <cooperative_groups.h>

#include <mutex>
#include <utility>
#include <vector>

#include "ernn_launch.h"
#include "ernn_resident.h"

namespace cg = cooperative_groups;

namespace ernn {

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the halo rows the neighbours store into this CTA: gives
// up after ~2^31 cycles (about a second), records ERNN_ERR_TIMEOUT in *err,
// and from then on every later wait of the launch returns at once, so the
// kernel still ends (with the error recorded) instead of spinning.
__device__ __forceinline__ void halo_wait(uint64_t* bar, uint32_t parity, int* err) {
  if (mbar_try_wait_cluster(bar, parity)) return;
  if (*(volatile int*)err != 0) return;
  const long long t0 = clock64();
  while (!mbar_try_wait_cluster(bar, parity)) {
    if (clock64() - t0 > kWaitLimitCycles) {
      atomicExch(err, kDeviceTimeout);
      return;
    }
  }
}

// shared::cluster address of the same shared-memory offset in CTA `rank`
__device__ __forceinline__ uint32_t map_rank(uint32_t local, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}

// 16-byte store into another CTA's shared memory, completing 16 bytes of
// transaction count on that CTA's mbarrier
__device__ __forceinline__ void st_async16(uint32_t addr, const float4& v, uint32_t bar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
          addr),
      "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(bar)
      : "memory");
}

// 1D bulk copy shared (this CTA) -> global in the current bulk group.
__device__ __forceinline__ void bulk_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(smem_u32(ssrc)), "r"(bytes)
               : "memory");
}
// 1D bulk copy global -> shared (this CTA), completing on mbarrier `bar`.
__device__ __forceinline__ void bulk_g2s(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(sdst)),
               "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// wait until the committed bulk stores have finished reading shared memory
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// wait until the committed bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---------------------------------------------------------------- layout
struct Tile {
  int R, ny, rows;      // rows: valid rows of this CTA (<= R)
  int plane;            // floats per component plane: (R + 2) * ny
  __device__ __forceinline__ float* comp(float* level, int c) const { return level + (size_t)c * plane; }
  // halo-coordinate row s (0 .. R+1), column j
  __device__ __forceinline__ int at(int s, int j) const { return s * ny + j; }
};

// Row window [j-1 .. j+4] of one component (zero outside 0..ny-1); j % 4 == 0.
__device__ __forceinline__ void load_row6(const float* __restrict__ p, int j, int ny, float w[6]) {
  const float4 m = *reinterpret_cast<const float4*>(p + j);
  w[0] = (j >= 1) ? p[j - 1] : 0.f;
  w[1] = m.x;
  w[2] = m.y;
  w[3] = m.z;
  w[4] = m.w;
  w[5] = (j + 4 < ny) ? p[j + 4] : 0.f;
}

// Stencil sums of the four cells (j .. j+3) of a row from its three row
// windows (rows above, at, below).
struct Quad {
  float cx[4], cy[4];
  float xx_x[4], yy_x[4], xy_x[4], xx_y[4], yy_y[4], xy_y[4];
};

// Packed FP32 (sm_100 family): one instruction for two cells of a quad, each
// lane rounded as the scalar operation; it shortens every row of the step
// loop, whose per-step chain sets the time.  Sums whose operands are column
// neighbours (not register pairs of the window) are formed by scalar adds
// first, so every value keeps the association and rounding of the scalar
// formulas.
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 pair(const float v[4], int p) { return make_float2(v[2 * p], v[2 * p + 1]); }
__device__ __forceinline__ float2 pair4(const float4& v, int p) {
  return p == 0 ? make_float2(v.x, v.y) : make_float2(v.z, v.w);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void put(float v[4], int p, float2 a) {
  v[2 * p] = a.x;
  v[2 * p + 1] = a.y;
}

// One component (cell q at window column k = q + 1):
//   xx = (u[0][k] + u[2][k]) - 2 u[1][k],  yy = (u[1][k-1] + u[1][k+1]) - 2 u[1][k],
//   xy = (u[2][k+1] + u[0][k-1]) - (u[2][k-1] + u[0][k+1]).
__device__ __forceinline__ void comp_stencils(const float u[3][6], float xx[4], float yy[4], float xy[4]) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int k = 2 * p + 1;
    const float2 m0 = make_float2(u[0][k], u[0][k + 1]);
    const float2 m1 = make_float2(u[1][k], u[1][k + 1]);
    const float2 m2 = make_float2(u[2][k], u[2][k + 1]);
    put(xx, p, __ffma2_rn(dup2(-2.f), m1, __fadd2_rn(m0, m2)));
    put(yy, p, __ffma2_rn(dup2(-2.f), m1, make_float2(u[1][k - 1] + u[1][k + 1], u[1][k] + u[1][k + 2])));
    const float2 a = make_float2(u[2][k + 1] + u[0][k - 1], u[2][k + 2] + u[0][k]);
    const float2 b = make_float2(u[2][k - 1] + u[0][k + 1], u[2][k] + u[0][k + 2]);
    put(xy, p, __fadd2_rn(a, neg2(b)));
  }
}

__device__ __forceinline__ void quad_stencils(const float ux[3][6], const float uy[3][6], Quad& s) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    s.cx[q] = ux[1][q + 1];
    s.cy[q] = uy[1][q + 1];
  }
  comp_stencils(ux, s.xx_x, s.yy_x, s.xy_x);
  comp_stencils(uy, s.xx_y, s.yy_y, s.xy_y);
}

struct KSr {
  float k11, k22, kq12, k16, k26, k66, k16h, k26h;
};

__device__ __forceinline__ void lq(const KSr& k, const Quad& s, int q, float& lx, float& ly) {
  lx = k.k11 * s.xx_x[q] + k.k66 * s.yy_x[q] + k.kq12 * s.xy_y[q] + k.k16h * s.xy_x[q] +
       k.k16 * s.xx_y[q] + k.k26 * s.yy_y[q];
  ly = k.k66 * s.xx_y[q] + k.k22 * s.yy_y[q] + k.kq12 * s.xy_x[q] + k.k16 * s.xx_x[q] +
       k.k26 * s.yy_x[q] + k.k26h * s.xy_y[q];
}

// (L u) of cells 2p and 2p+1: the terms of lq() in the same order.
__device__ __forceinline__ void lq2(const KSr& k, const Quad& s, int p, float2& lx, float2& ly) {
  lx = __fmul2_rn(dup2(k.k11), pair(s.xx_x, p));
  lx = __ffma2_rn(dup2(k.k66), pair(s.yy_x, p), lx);
  lx = __ffma2_rn(dup2(k.kq12), pair(s.xy_y, p), lx);
  lx = __ffma2_rn(dup2(k.k16h), pair(s.xy_x, p), lx);
  lx = __ffma2_rn(dup2(k.k16), pair(s.xx_y, p), lx);
  lx = __ffma2_rn(dup2(k.k26), pair(s.yy_y, p), lx);
  ly = __fmul2_rn(dup2(k.k66), pair(s.xx_y, p));
  ly = __ffma2_rn(dup2(k.k22), pair(s.yy_y, p), ly);
  ly = __ffma2_rn(dup2(k.kq12), pair(s.xy_x, p), ly);
  ly = __ffma2_rn(dup2(k.k16), pair(s.xx_x, p), ly);
  ly = __ffma2_rn(dup2(k.k26), pair(s.yy_x, p), ly);
  ly = __ffma2_rn(dup2(k.k26h), pair(s.xy_y, p), ly);
}

__device__ __forceinline__ void shift6(float u[3][6]) {
#pragma unroll
  for (int k = 0; k < 6; ++k) { u[0][k] = u[1][k]; u[1][k] = u[2][k]; }
}

__device__ __forceinline__ float4 f4(const float v[4]) { return make_float4(v[0], v[1], v[2], v[3]); }
__device__ __forceinline__ float at4(const float4& v, int q) {
  return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w;
}

// Per-step context of one CTA.  Levels form a ring of three: cur (read with
// its halo), prev (the level before, own rows), nxt (written).
struct StepCtx {
  const float* cur;
  const float* prev;
  float* nxt;
  uint32_t nxt_off_b;   // byte offset of nxt from the shared-memory base
  uint32_t up_base;     // shared::cluster address of the base in CTA rank-1 (0: none)
  uint32_t dn_base;     // ... in CTA rank+1 (0: none)
  uint32_t up_bar;      // shared::cluster address of the nxt-level mbarrier in rank-1
  uint32_t dn_bar;
  int rows, R, ny;
};

// Inputs of the right-hand side: FWD adds amp * F (one component), LAM adds
// gs * g at recording steps of the dense history.
struct Rhs {
  const float* F;
  float amp;
  int src_comp;
  const float* gx;
  const float* gy;
  float gs;
};

// One row lr (local) of one column quad j: windows w[0..1] hold halo rows
// lr, lr+1 on entry; loads halo row lr+2, computes, stores, pushes boundary
// rows to the neighbours, shifts the windows.  EDGE = false: lr is neither
// the CTA's first nor its last row (interior rows carry no push tests:
// measured 2.5 % faster on rot256).
template <bool LAM, bool DENSE, bool EDGE = true>
__device__ __forceinline__ void row_step(const Tile& T, const KSr& ks, const StepCtx& x,
                                         const Rhs& rhs, int lr, int j, float wx[3][6],
                                         float wy[3][6]) {
  const int ny = x.ny;
  const int s = lr + 1;
  float* cur = const_cast<float*>(x.cur);
  float4 fl = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!LAM) fl = *reinterpret_cast<const float4*>(rhs.F + lr * ny + j);  // first: it feeds the operator sum
  load_row6(T.comp(cur, 0) + T.at(s + 1, 0), j, ny, wx[2]);
  load_row6(T.comp(cur, 1) + T.at(s + 1, 0), j, ny, wy[2]);
  Quad st;
  quad_stencils(wx, wy, st);
  const float4 pvx = *reinterpret_cast<const float4*>(T.comp(const_cast<float*>(x.prev), 0) + T.at(s, j));
  const float4 pvy = *reinterpret_cast<const float4*>(T.comp(const_cast<float*>(x.prev), 1) + T.at(s, j));
  // v = (2 c - p) + (L u + f) (2 c is exact: one rounding either way); two
  // cells per instruction.  The load joins the operator sum before the
  // update, as in the reference's (A u + f) / rho: one rounding of the
  // increment into 2 c - p.  (Added after the update instead, the forward's
  // rounding near the source projects onto the gradient: ten times the FP32
  // reference's gradient error close to convergence.)
  float2 v2x[2], v2y[2];
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float2 lx, ly;
    lq2(ks, st, p, lx, ly);
    if (!LAM) {  // L + amp F, one rounding
      if (rhs.src_comp == 0) lx = __ffma2_rn(dup2(rhs.amp), pair4(fl, p), lx);
      else ly = __ffma2_rn(dup2(rhs.amp), pair4(fl, p), ly);
    }
    const float2 px = pair4(pvx, p), py = pair4(pvy, p);
    v2x[p] = __fadd2_rn(__ffma2_rn(dup2(2.f), pair(st.cx, p), neg2(px)), lx);
    v2y[p] = __fadd2_rn(__ffma2_rn(dup2(2.f), pair(st.cy, p), neg2(py)), ly);
  }
  if (LAM && DENSE && rhs.gx != nullptr) {
    const float4 a4 = *reinterpret_cast<const float4*>(rhs.gx + (size_t)lr * ny + j);
    const float4 b4 = *reinterpret_cast<const float4*>(rhs.gy + (size_t)lr * ny + j);
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      v2x[p] = __ffma2_rn(dup2(rhs.gs), pair4(a4, p), v2x[p]);
      v2y[p] = __ffma2_rn(dup2(rhs.gs), pair4(b4, p), v2y[p]);
    }
  }
  const float4 nvx = make_float4(v2x[0].x, v2x[0].y, v2x[1].x, v2x[1].y);
  const float4 nvy = make_float4(v2y[0].x, v2y[0].y, v2y[1].x, v2y[1].y);
  *reinterpret_cast<float4*>(T.comp(x.nxt, 0) + T.at(s, j)) = nvx;
  *reinterpret_cast<float4*>(T.comp(x.nxt, 1) + T.at(s, j)) = nvy;
  if (EDGE && lr == 0 && x.up_base) {  // into rank-1's bottom halo row
    const uint32_t o = x.nxt_off_b + 4u * (uint32_t)T.at(x.R + 1, j);
    st_async16(x.up_base + o, nvx, x.up_bar);
    st_async16(x.up_base + o + 4u * (uint32_t)T.plane, nvy, x.up_bar);
  }
  if (EDGE && lr == x.rows - 1 && x.dn_base) {  // into rank+1's top halo row
    const uint32_t o = x.nxt_off_b + 4u * (uint32_t)T.at(0, j);
    st_async16(x.dn_base + o, nvx, x.dn_bar);
    st_async16(x.dn_base + o + 4u * (uint32_t)T.plane, nvy, x.dn_bar);
  }
  shift6(wx);
  shift6(wy);
}

// Load the windows of halo rows s, s+1 (local rows s-1, s) of column quad j.
__device__ __forceinline__ void load_windows(const Tile& T, const StepCtx& x, int s, int j,
                                             float wx[3][6], float wy[3][6]) {
  float* cur = const_cast<float*>(x.cur);
  load_row6(T.comp(cur, 0) + T.at(s, 0), j, x.ny, wx[0]);
  load_row6(T.comp(cur, 1) + T.at(s, 0), j, x.ny, wy[0]);
  load_row6(T.comp(cur, 0) + T.at(s + 1, 0), j, x.ny, wx[1]);
  load_row6(T.comp(cur, 1) + T.at(s + 1, 0), j, x.ny, wy[1]);
}

// Rows a .. a+n-1 with windows already holding local rows a-1, a; on return
// they hold rows a+n-1, a+n.  Counts up to 4 are unrolled (window shifts
// become register renames).
template <bool LAM, bool DENSE, bool EDGE = true>
__device__ __forceinline__ void rows_from(const Tile& T, const KSr& ks, const StepCtx& x,
                                          const Rhs& rhs, int a, int n, int j, float wx[3][6],
                                          float wy[3][6]) {
  switch (n) {
    case 0: return;
    case 1:
      row_step<LAM, DENSE, EDGE>(T, ks, x, rhs, a, j, wx, wy);
      return;
    case 2:
#pragma unroll
      for (int q = 0; q < 2; ++q) row_step<LAM, DENSE, EDGE>(T, ks, x, rhs, a + q, j, wx, wy);
      return;
    case 3:
#pragma unroll
      for (int q = 0; q < 3; ++q) row_step<LAM, DENSE, EDGE>(T, ks, x, rhs, a + q, j, wx, wy);
      return;
    case 4:
#pragma unroll
      for (int q = 0; q < 4; ++q) row_step<LAM, DENSE, EDGE>(T, ks, x, rhs, a + q, j, wx, wy);
      return;
    default:
      for (int q = 0; q < n; ++q) row_step<LAM, DENSE, EDGE>(T, ks, x, rhs, a + q, j, wx, wy);
  }
}

// Work unit of a thread in a ring step: (column quad, chunk of consecutive
// rows).  The split depends only on the CTA's rows and the grid width, so it
// is computed once per launch (integer divisions out of the step loop).
struct Unit {
  int items;        // units of a step; > kResThreads: several per thread
  int rc;           // rows per chunk
  bool active;      // single-unit case: this thread has a unit
  int qc, ra, rb;   // its column quad and rows [ra, rb)
};

__device__ __forceinline__ Unit unit_of(int rows, int ny) {
  Unit u;
  const int ncq = ny / 4;
  const int nchunk = max(1, kResThreads / ncq);
  u.rc = (rows + nchunk - 1) / nchunk;
  u.items = ncq * nchunk;
  const int it = threadIdx.x;
  u.active = it < u.items;
  u.qc = u.active ? it % ncq : 0;
  const int ch = u.active ? it / ncq : 0;
  u.ra = ch * u.rc;
  u.rb = min(u.ra + u.rc, rows);
  return u;
}

// One step of the ring: interior rows first (they only read own rows of
// cur), then wait for the neighbours' boundary rows of cur, then the two
// boundary rows (pushed to the neighbours).  Work unit: (column quad, chunk
// of consecutive rows); the chunk holding the last row keeps its windows
// across the wait.
template <bool LAM, bool DENSE>
__device__ __forceinline__ void ring_step(const Tile& T, const KSr& ks, const StepCtx& x,
                                          const Rhs& rhs, uint64_t* cur_bar, uint32_t parity,
                                          bool wait, int* err, const Unit& U) {
  const int ncq = x.ny / 4;
  const int rc = U.rc;
  const int items = U.items;
  const int last = x.rows - 1;
  if (items <= kResThreads) {
    // one unit per thread: carry the windows over the wait
    const bool active = U.active;
    const int qc = U.qc;
    const int ra = U.ra, rb = U.rb;
    const int ia = max(ra, 1), ib = min(rb, last);
    float wx[3][6], wy[3][6];
    if (active && ia < ib) {
      load_windows(T, x, ia, 4 * qc, wx, wy);
      rows_from<LAM, DENSE, false>(T, ks, x, rhs, ia, ib - ia, 4 * qc, wx, wy);  // no boundary row
    }
    if (wait) halo_wait(cur_bar, parity, err);
    if (active && ra < rb) {
      if (rb == x.rows && last > 0) {
        if (!(ia < ib)) load_windows(T, x, last, 4 * qc, wx, wy);  // local rows last-1, last
        rows_from<LAM, DENSE>(T, ks, x, rhs, last, 1, 4 * qc, wx, wy);
      }
      if (ra == 0) {
        load_windows(T, x, 0, 4 * qc, wx, wy);  // halo row 0, local row 0
        rows_from<LAM, DENSE>(T, ks, x, rhs, 0, 1, 4 * qc, wx, wy);
      }
    }
    return;
  }
  for (int it = threadIdx.x; it < items; it += kResThreads) {
    const int qc = it % ncq, ch = it / ncq;
    const int ra = ch * rc, rb = min(ra + rc, x.rows);
    const int ia = max(ra, 1), ib = min(rb, last);
    if (ia < ib) {
      float wx[3][6], wy[3][6];
      load_windows(T, x, ia, 4 * qc, wx, wy);
      rows_from<LAM, DENSE, false>(T, ks, x, rhs, ia, ib - ia, 4 * qc, wx, wy);  // no boundary row
    }
  }
  if (wait) halo_wait(cur_bar, parity, err);
  for (int it = threadIdx.x; it < items; it += kResThreads) {
    const int qc = it % ncq, ch = it / ncq;
    const int ra = ch * rc, rb = min(ra + rc, x.rows);
    if (ra >= rb) continue;
    float wx[3][6], wy[3][6];
    if (ra == 0) {
      load_windows(T, x, 0, 4 * qc, wx, wy);
      rows_from<LAM, DENSE>(T, ks, x, rhs, 0, 1, 4 * qc, wx, wy);
    }
    if (rb == x.rows && last > 0) {
      load_windows(T, x, last, 4 * qc, wx, wy);
      rows_from<LAM, DENSE>(T, ks, x, rhs, last, 1, 4 * qc, wx, wy);
    }
  }
}

// ------------------------------------------------- register-resident step
// The step roles' fast form, for grids whose CTAs split into full chunks of
// RC rows (every thread one unit of exactly RC rows).  A thread's unit
// (column quad, RC consecutive rows) is fixed for the launch, so the thread
// keeps its own cells of the current and the previous level in registers
// from one step to the next: per step it reads from shared memory only the
// left and right neighbours of its rows and the rows just above and below
// its chunk, and writes its new cells (for the neighbours' windows of the
// next step and the state copies); the previous level never comes back from
// shared memory.  The three-level ring in shared memory stays complete
// (every cell is stored every step), so halo pushes, bulk state copies,
// trace recording and the final lam pair read it as before.  Receiver
// residuals (adjoint role) are added by the threads owning the receiver
// cells, in registers.
struct RegUnit {
  bool active;       // the thread has a unit (a chunk inside the CTA's rows)
  int j;             // first column of the quad
  int ra;            // rows ra .. ra+RC-1 (local)
  bool top_ext;      // row ra is the CTA's first row (its upper row is a halo row)
  bool bot_ext;      // row ra+RC-1 is the CTA's last row
  uint32_t src_rows; // bit k: row ra+k meets the source box (forward role)
  uint32_t rmask;    // bit 4k+q: cell (ra+k, j+q) holds a receiver (adjoint role)
};

// The thread's own cells of a level: rows ra .. ra+RC-1 of the quad at j.
template <int RC>
__device__ __forceinline__ void own_load(const Tile& T, const float* level, const RegUnit& U,
                                         float (&vx)[RC][4], float (&vy)[RC][4]) {
#pragma unroll
  for (int k = 0; k < RC; ++k) {
    const float4 a = *reinterpret_cast<const float4*>(T.comp(const_cast<float*>(level), 0) + T.at(U.ra + k + 1, U.j));
    const float4 b = *reinterpret_cast<const float4*>(T.comp(const_cast<float*>(level), 1) + T.at(U.ra + k + 1, U.j));
    vx[k][0] = a.x; vx[k][1] = a.y; vx[k][2] = a.z; vx[k][3] = a.w;
    vy[k][0] = b.x; vy[k][1] = b.y; vy[k][2] = b.z; vy[k][3] = b.w;
  }
}

// A row window as register references: left neighbour, the four cells, right
// neighbour (columns j-1 .. j+4).
struct RowRef {
  const float& l;
  const float (&c)[4];
  const float& r;
};

// One component's stencil sums of the four cells from the rows above (u0),
// at (u1) and below (u2): the terms of comp_stencils in the same order and
// rounding.
__device__ __forceinline__ void ref_stencils(const RowRef& u0, const RowRef& u1, const RowRef& u2,
                                             float xx[4], float yy[4], float xy[4]) {
  auto at = [](const RowRef& u, int k) -> float { return k == 0 ? u.l : k == 5 ? u.r : u.c[k - 1]; };
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int k = 2 * p + 1;
    const float2 m0 = make_float2(at(u0, k), at(u0, k + 1));
    const float2 m1 = make_float2(at(u1, k), at(u1, k + 1));
    const float2 m2 = make_float2(at(u2, k), at(u2, k + 1));
    put(xx, p, __ffma2_rn(dup2(-2.f), m1, __fadd2_rn(m0, m2)));
    put(yy, p, __ffma2_rn(dup2(-2.f), m1, make_float2(at(u1, k - 1) + at(u1, k + 1), at(u1, k) + at(u1, k + 2))));
    const float2 a = make_float2(at(u2, k + 1) + at(u0, k - 1), at(u2, k + 2) + at(u0, k));
    const float2 b = make_float2(at(u2, k - 1) + at(u0, k + 1), at(u2, k) + at(u0, k + 2));
    put(xy, p, __fadd2_rn(a, neg2(b)));
  }
}

// New values of one own row (local row lr): px, py hold the previous level
// on entry and the new level on return.  The new row is stored into the
// next level and, on the CTA's first and last row, pushed into the
// neighbours' halo rows.  Same terms, order and rounding as row_step.
template <bool LAM, bool DENSE>
__device__ __forceinline__ void reg_row(const Tile& T, const KSr& ks, const StepCtx& x, const Rhs& rhs,
                                        int lr, int j, bool src_row, const RowRef& ax, const RowRef& ay,
                                        const RowRef& bx, const RowRef& by, const RowRef& dx,
                                        const RowRef& dy, float (&px)[4], float (&py)[4]) {
  const int ny = x.ny;
  const int s = lr + 1;
  Quad st;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    st.cx[q] = bx.c[q];
    st.cy[q] = by.c[q];
  }
  ref_stencils(ax, bx, dx, st.xx_x, st.yy_x, st.xy_x);
  ref_stencils(ay, by, dy, st.xx_y, st.yy_y, st.xy_y);
  // the load joins the operator sum before the update, as in row_step
  const bool src = !LAM && src_row;
  float4 fl = make_float4(0.f, 0.f, 0.f, 0.f);
  if (src) fl = *reinterpret_cast<const float4*>(rhs.F + lr * ny + j);
  float2 v2x[2], v2y[2];
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float2 lx, ly;
    lq2(ks, st, p, lx, ly);
    if (src) {  // L + amp F, one rounding
      if (rhs.src_comp == 0) lx = __ffma2_rn(dup2(rhs.amp), pair4(fl, p), lx);
      else ly = __ffma2_rn(dup2(rhs.amp), pair4(fl, p), ly);
    }
    v2x[p] = __fadd2_rn(__ffma2_rn(dup2(2.f), pair(st.cx, p), neg2(pair(px, p))), lx);
    v2y[p] = __fadd2_rn(__ffma2_rn(dup2(2.f), pair(st.cy, p), neg2(pair(py, p))), ly);
  }
  if (LAM && DENSE && rhs.gx != nullptr) {
    const float4 a4 = *reinterpret_cast<const float4*>(rhs.gx + (size_t)lr * ny + j);
    const float4 b4 = *reinterpret_cast<const float4*>(rhs.gy + (size_t)lr * ny + j);
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      v2x[p] = __ffma2_rn(dup2(rhs.gs), pair4(a4, p), v2x[p]);
      v2y[p] = __ffma2_rn(dup2(rhs.gs), pair4(b4, p), v2y[p]);
    }
  }
  put(px, 0, v2x[0]);
  put(px, 1, v2x[1]);
  put(py, 0, v2y[0]);
  put(py, 1, v2y[1]);
  const float4 nvx = f4(px), nvy = f4(py);
  *reinterpret_cast<float4*>(T.comp(x.nxt, 0) + T.at(s, j)) = nvx;
  *reinterpret_cast<float4*>(T.comp(x.nxt, 1) + T.at(s, j)) = nvy;
  if (lr == 0 && x.up_base) {  // into rank-1's bottom halo row
    const uint32_t o = x.nxt_off_b + 4u * (uint32_t)T.at(x.R + 1, j);
    st_async16(x.up_base + o, nvx, x.up_bar);
    st_async16(x.up_base + o + 4u * (uint32_t)T.plane, nvy, x.up_bar);
  }
  if (lr == x.rows - 1 && x.dn_base) {  // into rank+1's top halo row
    const uint32_t o = x.nxt_off_b + 4u * (uint32_t)T.at(0, j);
    st_async16(x.dn_base + o, nvx, x.dn_bar);
    st_async16(x.dn_base + o + 4u * (uint32_t)T.plane, nvy, x.dn_bar);
  }
}

// Window [j-1 .. j+4] of a shared-memory row as (left, quad, right).
struct HaloRow {
  float l, c[4], r;
};
__device__ __forceinline__ void load_halo(const float* __restrict__ p, int j, int ny, HaloRow& h) {
  const float4 m = *reinterpret_cast<const float4*>(p + j);
  h.l = (j >= 1) ? p[j - 1] : 0.f;
  h.c[0] = m.x;
  h.c[1] = m.y;
  h.c[2] = m.z;
  h.c[3] = m.w;
  h.r = (j + 4 < ny) ? p[j + 4] : 0.f;
}

// One ring step of the register-resident form.  (cx, cy): the thread's cells
// of cur; (px, py): of prev on entry, of nxt on return.  The rows that read
// a neighbour CTA's halo row (the CTA's first and last rows) run after the
// bounded wait for it, every other row before; threads with neither row do
// not wait.
template <bool LAM, bool DENSE, int RC>
__device__ __forceinline__ void reg_step(const Tile& T, const KSr& ks, const StepCtx& x, const Rhs& rhs,
                                         uint64_t* cur_bar, uint32_t parity, bool wait, int* err,
                                         const RegUnit& U, const float (&cx)[RC][4],
                                         const float (&cy)[RC][4], float (&px)[RC][4],
                                         float (&py)[RC][4]) {
  const int ny = x.ny, j = U.j, a = U.ra;
  const float* cur0 = T.comp(const_cast<float*>(x.cur), 0);
  const float* cur1 = T.comp(const_cast<float*>(x.cur), 1);
  float lx[RC], rx[RC], ly[RC], ry[RC];
#pragma unroll
  for (int k = 0; k < RC; ++k) {
    const int o = T.at(a + k + 1, 0);
    lx[k] = j >= 1 ? cur0[o + j - 1] : 0.f;
    ly[k] = j >= 1 ? cur1[o + j - 1] : 0.f;
    rx[k] = j + 4 < ny ? cur0[o + j + 4] : 0.f;
    ry[k] = j + 4 < ny ? cur1[o + j + 4] : 0.f;
  }
  HaloRow tx, ty, bx, by;  // rows a-1 and a+RC (halo coordinates a and a+RC+1)
  if (!U.top_ext) {
    load_halo(cur0 + T.at(a, 0), j, ny, tx);
    load_halo(cur1 + T.at(a, 0), j, ny, ty);
  }
  if (!U.bot_ext) {
    load_halo(cur0 + T.at(a + RC + 1, 0), j, ny, bx);
    load_halo(cur1 + T.at(a + RC + 1, 0), j, ny, by);
  }
  auto row = [&](int k) {
    const RowRef bxr{lx[k], cx[k], rx[k]}, byr{ly[k], cy[k], ry[k]};
    const RowRef axr = k == 0 ? RowRef{tx.l, tx.c, tx.r} : RowRef{lx[k - 1], cx[k - 1], rx[k - 1]};
    const RowRef ayr = k == 0 ? RowRef{ty.l, ty.c, ty.r} : RowRef{ly[k - 1], cy[k - 1], ry[k - 1]};
    const RowRef dxr = k == RC - 1 ? RowRef{bx.l, bx.c, bx.r} : RowRef{lx[k + 1], cx[k + 1], rx[k + 1]};
    const RowRef dyr = k == RC - 1 ? RowRef{by.l, by.c, by.r} : RowRef{ly[k + 1], cy[k + 1], ry[k + 1]};
    reg_row<LAM, DENSE>(T, ks, x, rhs, a + k, j, (U.src_rows >> k) & 1u, axr, ayr, bxr, byr, dxr, dyr,
                        px[k], py[k]);
  };
#pragma unroll
  for (int k = 0; k < RC; ++k)
    if (!(k == 0 && U.top_ext) && !(k == RC - 1 && U.bot_ext)) row(k);
  if (U.top_ext || U.bot_ext) {
    if (wait) halo_wait(cur_bar, parity, err);
    if (U.top_ext) {
      load_halo(cur0 + T.at(0, 0), j, ny, tx);
      load_halo(cur1 + T.at(0, 0), j, ny, ty);
    }
    if (U.bot_ext) {
      load_halo(cur0 + T.at(a + RC + 1, 0), j, ny, bx);
      load_halo(cur1 + T.at(a + RC + 1, 0), j, ny, by);
    }
    if (U.top_ext) row(0);
    if (U.bot_ext && (RC > 1 || !U.top_ext)) row(RC - 1);
  }
}

// Row window [j-1 .. j+4] of row i of a global plane (zero outside the grid).
__device__ __forceinline__ void load_grow6(const float* __restrict__ plane, int i, int j, int nx,
                                           int ny, float w[6]) {
  if (i < 0 || i >= nx) {
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = 0.f;
    return;
  }
  const float* p = plane + (size_t)i * ny;
  const float4 m = __ldg(reinterpret_cast<const float4*>(p + j));
  w[0] = (j >= 1) ? __ldg(p + j - 1) : 0.f;
  w[1] = m.x;
  w[2] = m.y;
  w[3] = m.z;
  w[4] = m.w;
  w[5] = (j + 4 < ny) ? __ldg(p + j + 4) : 0.f;
}

// Imaging of one 4 x 4 item of step n: sum over its cells of lam^{n+1} times
// the derivatives of A u^n with respect to the six constants.
__device__ __forceinline__ void img_item(const float* __restrict__ lam, const float* __restrict__ u,
                                         size_t N, int nx, int ny, int i0, int j, float acc[6]) {
  float vx[3][6], vy[3][6];
  load_grow6(u, i0 - 1, j, nx, ny, vx[0]);
  load_grow6(u + N, i0 - 1, j, nx, ny, vy[0]);
  load_grow6(u, i0, j, nx, ny, vx[1]);
  load_grow6(u + N, i0, j, nx, ny, vy[1]);
#pragma unroll
  for (int q4 = 0; q4 < 4; ++q4) {
    const int i = i0 + q4;
    if (i >= nx) break;
    load_grow6(u, i + 1, j, nx, ny, vx[2]);
    load_grow6(u + N, i + 1, j, nx, ny, vy[2]);
    Quad su;
    quad_stencils(vx, vy, su);
    const float4 lx4 = __ldg(reinterpret_cast<const float4*>(lam + (size_t)i * ny + j));
    const float4 ly4 = __ldg(reinterpret_cast<const float4*>(lam + N + (size_t)i * ny + j));
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float l1x = at4(lx4, q), l1y = at4(ly4, q);
      acc[0] += l1x * su.xx_x[q];
      acc[1] += l1y * su.yy_y[q];
      acc[2] += l1x * su.xy_y[q] + l1y * su.xy_x[q];
      acc[3] += l1x * (0.5f * su.xy_x[q] + su.xx_y[q]) + l1y * su.xx_x[q];
      acc[4] += l1x * su.yy_y[q] + l1y * (su.yy_x[q] + 0.5f * su.xy_y[q]);
      acc[5] += l1x * su.yy_x[q] + l1y * su.xx_y[q];
    }
    shift6(vx);
    shift6(vy);
  }
}

// FP64 block reduction of six per-thread sums into one row of partials.
__device__ __forceinline__ void block_reduce6(const double v6[6], double* __restrict__ row) {
  __shared__ double red[kResThreads / 32][6];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    double v = v6[t];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][t] = v;
  }
  __syncthreads();
  if (tid < 6) {
    double v = 0.0;
    for (int w = 0; w < kResThreads / 32; ++w) v += red[w][tid];
    row[tid] += v;
  }
}

// IMG role: the items (n, row group, column quad) of one shot spread over
// that shot's IMG CTAs; products summed in FP32 over an item's 16 cells, in
// FP64 from there on; one partial row per CTA, rows grouped by shot.
__device__ void imaging_role(const ResCommon& c, const ResImg& g, int shot, int cta, int ncta) {
  const size_t N = (size_t)c.nx * c.ny;
  const int ngr = (c.nx + 3) / 4, ncq = c.ny / 4;
  const int nn = g.n_hi - g.n_lo + 1;
  double acc64[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  // items it = first, first + stride, ... walked as (dn, gi, qc) digits of
  // radix (nn, ngr, ncq): an addition with carries per item, no division
  const int first = cta * kResThreads + threadIdx.x, stride = ncta * kResThreads;
  int qc = first % ncq, gi = (first / ncq) % ngr, dn = first / ncq / ngr;
  const int sq = stride % ncq, sg = (stride / ncq) % ngr, sd = stride / ncq / ngr;
  for (; dn < nn;) {
    const size_t slot = (size_t)dn * g.state_stride + (size_t)shot * 2 * N;
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    img_item(g.lbuf + slot, g.ubuf + slot, N, c.nx, c.ny, 4 * gi, 4 * qc, acc);
#pragma unroll
    for (int t = 0; t < 6; ++t) acc64[t] += (double)acc[t];
    qc += sq;
    if (qc >= ncq) { qc -= ncq; ++gi; }
    gi += sg;
    if (gi >= ngr) { gi -= ngr; ++dn; }
    dn += sd;
  }
  block_reduce6(acc64, g.partials + ((size_t)shot * ncta + cta) * 8);
}

// ---------------------------------------------------------------- kernel
// The thread issuing a CTA's bulk state copies (and waiting for them), and
// the first thread of the forward role's receiver gather: both in middle
// warps, away from the first and last warps, which compute the CTA's first
// and last rows (the chain through the neighbours) on square grids.
constexpr int kStoreTid = kResThreads / 2;
constexpr int kGatherTid0 = kResThreads / 4;

template <bool DENSE, int RC>
__global__ void __launch_bounds__(kResThreads, 1) resident_kernel(const ResCommon c, const ResFwd f,
                                                                   const ResLam a, const ResImg g,
                                                                   const ResRoles roles) {
  const int z = (int)blockIdx.z;
  if (roles.z_img >= 0 && z >= roles.z_img) {
    // IMG role: no cluster features, no shared state; blockIdx.y is the shot
    const int cta = (z - roles.z_img) * (int)gridDim.x + (int)blockIdx.x;
    const int ncta = roles.n_img_z * (int)gridDim.x;
    imaging_role(c, g, (int)blockIdx.y, cta, ncta);
    return;
  }
  extern __shared__ __align__(128) float smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int CL = c.CL;
  const int shot = blockIdx.y;
  const bool is_fwd = (z == roles.z_fwd);
  const int tid = threadIdx.x;
  const int nx = c.nx, ny = c.ny, R = c.R;
  const size_t N = (size_t)nx * ny;
  const int r0 = rank * R;
  const int rows = min(R, nx - r0);  // >= 1 by construction on the host
  Tile T{R, ny, rows, (R + 2) * ny};
  const int level_floats = 2 * T.plane;

  // ring of three levels: level l starts at smem + l * level_floats
  auto Lv = [&](int l) { return smem + l * level_floats; };
  float* F = smem + 3 * level_floats;   // FWD role: source load of the own rows [R][ny]
  int* rec_list = reinterpret_cast<int*>(F + R * ny);  // [kResMaxRec][2]
  int* rec_count = rec_list + 2 * kResMaxRec;
  uint64_t* bar = reinterpret_cast<uint64_t*>(rec_count + 4);  // [4], 8-byte aligned
  // bar[0..2]: halo rows of the ring levels; bar[3]: the initial state
  int* inj = reinterpret_cast<int*>(bar + 4);  // [kResMaxRec] receivers by owner thread
  int* inj_cnt = inj + kResMaxRec;             // [kResThreads]
  int* inj_pos = inj_cnt + kResThreads;        // [kResThreads]

  const Coef* K = c.coef + (size_t)shot * c.coef_stride;
  const KSr ks{K->k11, K->k22, K->kq12, K->k16, K->k26, K->k66, K->k16h, K->k26h};
  const float kappa = K->kappa;
  const size_t shot_off = (size_t)shot * 2 * N;

  // -------- initial state: zero the levels and the load, then load
  {
    float4* z4 = reinterpret_cast<float4*>(smem);  // ny % 4 == 0: whole float4s
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = tid; e < (3 * level_floats + R * ny) / 4; e += kResThreads) z4[e] = zero;
  }
  if (tid == 0) {
    *rec_count = 0;
    for (int l = 0; l < 4; ++l) mbar_init(&bar[l], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (is_fwd && c.bx > 0 && c.by > 0) {
    // the shot's load restricted to the own rows, kept in shared memory so the
    // update adds amp * F without touching global memory
    const int ox = c.src_origin[2 * shot], oy = c.src_origin[2 * shot + 1];
    for (int e = tid; e < c.bx * c.by; e += kResThreads) {
      const int sa = e / c.by, sb = e - sa * c.by;
      const int gi = ox + sa, gj = oy + sb;
      if (gi >= r0 && gi < r0 + rows && gj >= 0 && gj < ny)
        F[(gi - r0) * ny + gj] = c.src_map[(size_t)shot * c.bx * c.by + e];
    }
  }
  // receivers owned by this CTA
  if (c.nrec > 0) {
    for (int r = tid; r < c.nrec; r += kResThreads) {
      const int32_t idx = c.rec_idx[(size_t)shot * c.nrec + r];
      if (idx < 0 || (size_t)idx >= N) continue;
      const int gi = idx / ny;
      if (gi >= r0 && gi < r0 + rows) {
        const int slot = atomicAdd(rec_count, 1);
        if (slot < kResMaxRec) {
          rec_list[2 * slot] = (gi - r0 + 1) * ny + (idx - gi * ny);  // halo-coordinate offset
          rec_list[2 * slot + 1] = r;
        }
      }
    }
  }
  const float* init_cur = is_fwd ? f.init_cur : (a.first ? nullptr : a.lam_save);
  const float* init_prev = is_fwd ? f.init_prev : (a.first ? nullptr : a.lam_save + a.save_stride);
  // step 0 reads L[0] (with halo rows, from global memory) and L[2] (own
  // rows): one bulk copy per component and level (rows are contiguous in
  // both layouts; rows outside the grid stay zero), or element by element
  // when a source is not on a 16-byte boundary
  const bool bulk_init = (init_cur == nullptr || al16(init_cur)) && (init_prev == nullptr || al16(init_prev));
  if (bulk_init) {
    const int g_lo = max(r0 - 1, 0), g_hi = min(r0 + rows + 1, nx);  // rows of cur with its halo
    const uint32_t cur_bytes = (uint32_t)((size_t)(g_hi - g_lo) * ny * sizeof(float));
    const uint32_t prev_bytes = (uint32_t)((size_t)rows * ny * sizeof(float));
    const uint32_t total = (init_cur ? 2u * cur_bytes : 0u) + (init_prev ? 2u * prev_bytes : 0u);
    if (total > 0) {
      if (tid == 0) {
        fence_proxy_async();  // the zero stores above before the copies' writes
        mbar_arrive_expect_tx(&bar[3], total);
        for (int comp = 0; comp < 2; ++comp) {
          if (init_cur)
            bulk_g2s(T.comp(Lv(0), comp) + T.at(g_lo - r0 + 1, 0),
                     init_cur + shot_off + (size_t)comp * N + (size_t)g_lo * ny, cur_bytes, &bar[3]);
          if (init_prev)
            bulk_g2s(T.comp(Lv(2), comp) + T.at(1, 0), init_prev + shot_off + (size_t)comp * N + (size_t)r0 * ny,
                     prev_bytes, &bar[3]);
        }
      }
      halo_wait(&bar[3], 0u, c.err);
    }
  } else {
    for (int e = tid; e < 2 * (rows + 2) * ny; e += kResThreads) {
      const int comp = e / ((rows + 2) * ny);
      const int rem = e - comp * (rows + 2) * ny;
      const int s = rem / ny, j = rem - s * ny;
      const int gi = r0 + s - 1;
      if (gi < 0 || gi >= nx) continue;
      const size_t gidx = shot_off + (size_t)comp * N + (size_t)gi * ny + j;
      if (init_cur) T.comp(Lv(0), comp)[T.at(s, j)] = init_cur[gidx];
      if (init_prev && s >= 1 && s <= rows) T.comp(Lv(2), comp)[T.at(s, j)] = init_prev[gidx];
    }
  }
  __syncthreads();
  cluster.sync();  // every CTA initialised (levels, mbarriers) before any push

  const int nloc = min(*rec_count, kResMaxRec);
  const bool has_up = rank > 0, has_dn = rank < CL - 1;
  // bytes each ring step receives: both components of one row per neighbour
  const uint32_t halo_bytes = (uint32_t)((has_up ? 1 : 0) + (has_dn ? 1 : 0)) * 2u * (uint32_t)ny * 4u;
  const uint32_t base_b = smem_u32(smem);
  const Unit U = unit_of(rows, ny);
  StepCtx x;
  x.up_base = has_up ? map_rank(base_b, rank - 1) : 0u;
  x.dn_base = has_dn ? map_rank(base_b, rank + 1) : 0u;
  x.rows = rows;
  x.R = R;
  x.ny = ny;
  uint32_t parity_bits = 0u;  // bit l: phase parity of bar[l]
  // The levels of step t: cur is ring level cl = t % 3 (kept as a counter by
  // the step loops), prev cl - 1 and nxt cl + 1 (mod 3).  The neighbours'
  // mbarriers of a level are at the same offsets in their shared::cluster
  // windows as this CTA's (mapped once).
  const uint32_t up_bar0 = has_up ? map_rank(smem_u32(&bar[0]), rank - 1) : 0u;
  const uint32_t dn_bar0 = has_dn ? map_rank(smem_u32(&bar[0]), rank + 1) : 0u;
  int cl = 0;
  auto set_levels = [&]() {
    const int nl = cl == 2 ? 0 : cl + 1, pl = cl == 0 ? 2 : cl - 1;
    x.cur = Lv(cl);
    x.prev = Lv(pl);
    x.nxt = Lv(nl);
    x.nxt_off_b = (uint32_t)nl * (uint32_t)level_floats * 4u;
    x.up_bar = has_up ? up_bar0 + 8u * (uint32_t)nl : 0u;
    x.dn_bar = has_dn ? dn_bar0 + 8u * (uint32_t)nl : 0u;
  };
  auto next_level = [&]() { cl = cl == 2 ? 0 : cl + 1; };
  // this step's wait: the neighbours pushed cur's halo during their step t-1
  auto step_wait = [&](int t) -> bool { return t >= 1 && halo_bytes > 0; };
  auto expect_next = [&]() {  // halo of nxt arrives during the neighbours' step t
    if (tid == 0 && halo_bytes > 0) mbar_arrive_expect_tx(&bar[cl == 2 ? 0 : cl + 1], halo_bytes);
  };
  const uint32_t own_bytes = (uint32_t)((size_t)rows * ny * sizeof(float));
  // own rows of a level -> global state at dst (x plane, y plane at y_off)
  auto store_level = [&](const float* level, float* dst, ptrdiff_t y_off) {
    bulk_s2g(dst + (size_t)r0 * ny, T.comp(const_cast<float*>(level), 0) + T.at(1, 0), own_bytes);
    bulk_s2g(dst + y_off + (size_t)r0 * ny, T.comp(const_cast<float*>(level), 1) + T.at(1, 0),
             own_bytes);
  };
  int t_last = -1;

  // register-resident form of the adjoint role: the thread's own cells of
  // the two latest levels (A and B swap roles from one step to the next)
  constexpr int RCn = RC > 0 ? RC : 1;
  float Ax[RCn][4], Ay[RCn][4], Bx[RCn][4], By[RCn][4];
  RegUnit RU;
  RU.active = false;
  RU.j = 0;
  RU.ra = 0;
  RU.top_ext = RU.bot_ext = false;
  RU.src_rows = 0u;
  RU.rmask = 0u;
  if (RC > 0) {
    // units of exactly RC rows: thread tid takes column quad tid % (ny / 4)
    // and rows [RC * (tid / (ny / 4)), + RC); the host launches this form only
    // when every CTA's rows split into such chunks
    const int ncq = ny / 4, ch = tid / ncq;
    RU.j = 4 * (tid - ch * ncq);
    RU.ra = ch * RCn;
    RU.active = RU.ra < rows;
    RU.top_ext = RU.ra == 0;
    RU.bot_ext = RU.ra + RCn == rows;
    if (RU.active && !is_fwd) {
      own_load<RCn>(T, Lv(0), RU, Ax, Ay);  // cur of the first step
      own_load<RCn>(T, Lv(2), RU, Bx, By);  // prev of the first step
    }
  }

  if (is_fwd) {
    // ================================================================ FWD role
    const float* sig = c.src_signal + (size_t)shot * c.nt;
    float amp_next = (f.i0 < f.i1) ? sig[f.i0] : 0.f;
    Rhs rhs{F, 0.f, c.src_comp, nullptr, nullptr, 0.f};
    // i % stride and i / stride, kept as counters (no integer division in
    // the step loop)
    int st_r = f.i0 % c.stride, st_q = f.i0 / c.stride;
    // The state copies are the store thread's alone: its next state slot
    // and the checkpoint phases of i + 1, i + 2 as counters, the slots as
    // pointers stepped by additions.
    const int ck_k = f.ckpt != nullptr ? f.ck_k : 1;
    int c1_r = (f.i0 + 1) % ck_k, c1_q = (f.i0 + 1) / ck_k;
    int c2_r = (f.i0 + 2) % ck_k, c2_q = (f.i0 + 2) / ck_k;
    float* st_next = f.states ? f.states + shot_off : nullptr;
    // (slot c - 1 of checkpoint c: c1_q, c2_q >= 1 at every step that copies)
    float* ck_lev0 = f.ckpt ? f.ckpt + ((ptrdiff_t)(c1_q - 1) * 2 + 0) * (ptrdiff_t)f.state_stride + shot_off
                            : nullptr;
    float* ck_lev1 = f.ckpt ? f.ckpt + ((ptrdiff_t)(c2_q - 1) * 2 + 1) * (ptrdiff_t)f.state_stride + shot_off
                            : nullptr;
    const size_t ck_seg = 2 * f.state_stride;  // floats between checkpoints
    // The receivers this thread records (entries g, g + kResThreads, ...;
    // g counts from kGatherTid0 so the gather avoids the first warp, which
    // also computes the CTA's first row): shared-memory offsets and output
    // offsets at frame 0, in registers.
    constexpr int kGath = (kResMaxRec + kResThreads - 1) / kResThreads;
    const int g0 = (tid + kResThreads - kGatherTid0) % kResThreads;
    int goff[kGath];
    size_t gout[kGath];
    int ngath = 0;
#pragma unroll
    for (int h = 0; h < kGath; ++h) {
      const int e = g0 + h * kResThreads;
      goff[h] = e < nloc ? rec_list[2 * e] : 0;
      gout[h] = e < nloc ? (size_t)shot * c.nt_out * c.nrec + rec_list[2 * e + 1] : 0;
      if (e < nloc) ngath = h + 1;
    }
    // (the step as a lambda called from one loop: measured 8 % faster on
    // rot256 than the same body written inline in the loop)
    auto fwd_step = [&](int i) {
      const int t = i - f.i0;
      set_levels();
      expect_next();
      rhs.amp = amp_next * kappa;
      amp_next = (i + 1 < f.i1) ? sig[i + 1] : 0.f;  // in flight during this step
      const bool w = step_wait(t);
      ring_step<false, false>(T, ks, x, rhs, &bar[cl], (parity_bits >> cl) & 1u, w, c.err, U);
      if (w) parity_bits ^= 1u << cl;
      // bulk stores issued after the previous step read a level overwritten two
      // steps from now: make sure they are done reading before the barrier
      if (tid == kStoreTid) bulk_wait_read_all();
      __syncthreads();
      t_last = t;
      next_level();
      const bool rec_step = st_r == 0;
      const int frame = st_q;
      if (++st_r == c.stride) { st_r = 0; ++st_q; }
      if (tid == kStoreTid) {
        // u^{i+1} (own rows of nxt) to global memory through the bulk-copy engine
        float* dst[4] = {st_next, nullptr, nullptr, nullptr};
        ptrdiff_t dst_y[4] = {(ptrdiff_t)N, (ptrdiff_t)N, (ptrdiff_t)N, (ptrdiff_t)N};  // y plane offset
        if (st_next) st_next += f.state_stride;
        if (f.ckpt != nullptr) {
          if (c1_r == 0 && c1_q <= f.ck_nseg - 1) dst[1] = ck_lev0;
          if (c2_r == 0 && c2_q <= f.ck_nseg - 1) dst[2] = ck_lev1;
          if (++c1_r == ck_k) { c1_r = 0; ++c1_q; ck_lev0 += ck_seg; }
          if (++c2_r == ck_k) { c2_r = 0; ++c2_q; ck_lev1 += ck_seg; }
        }
        if (DENSE && rec_step && f.hist_x) {
          dst[3] = f.hist_x + ((size_t)shot * c.nt_out + frame) * N;
          dst_y[3] = f.hist_y - f.hist_x;  // the y history relative to the x history
        }
        if (dst[0] || dst[1] || dst[2] || dst[3]) {
          fence_proxy_async();
#pragma unroll
          for (int d = 0; d < 4; ++d)
            if (dst[d]) store_level(x.nxt, dst[d], dst_y[d]);
          bulk_commit();
        }
      }
      if (!DENSE && rec_step && ngath > 0 && f.tr_x) {
        const size_t fo = (size_t)frame * c.nrec;
#pragma unroll
        for (int h = 0; h < kGath; ++h) {
          if (h < ngath) {
            f.tr_x[gout[h] + fo] = T.comp(x.nxt, 0)[goff[h]];
            f.tr_y[gout[h] + fo] = T.comp(x.nxt, 1)[goff[h]];
          }
        }
      }
    };
    for (int i = f.i0; i < f.i1; ++i) fwd_step(i);
  } else {
    // ================================================================ LAM role
    const float gs = c.coef->gscale;  // one scale for every shot
    // residuals of the receivers this thread injects (entries tid + h * kResThreads),
    // loaded one recording step ahead when the launch's frames are not staged
    // in shared memory (below); generic form only
    constexpr int kRecPerThread = RC > 0 ? 1 : (kResMaxRec + kResThreads - 1) / kResThreads;
    float gnx[kRecPerThread], gny[kRecPerThread];
#pragma unroll
    for (int h = 0; h < kRecPerThread; ++h) { gnx[h] = 0.f; gny[h] = 0.f; }
    int next_src = a.m_hi - ((a.m_hi - 1) % c.stride);  // highest m <= m_hi with a frame
    auto load_g = [&](int m) {
      const int frame = (m - 1) / c.stride;
#pragma unroll
      for (int h = 0; h < kRecPerThread; ++h) {
        const int e = tid + h * kResThreads;
        if (e < nloc) {
          const size_t go = ((size_t)shot * c.nt_out + frame) * c.nrec + rec_list[2 * e + 1];
          gnx[h] = a.g_x[go];
          gny[h] = a.g_y[go];
        }
      }
    };
    // The residuals of every frame of this launch, gathered once into the
    // load area F (unused by this role): entry (frame - f_lo) * nloc + e, x
    // and y interleaved.  The per-step injection then reads shared memory
    // only; when they do not fit, each step loads the next frame's residuals.
    const int f_lo = (a.m_lo + c.stride - 1) / c.stride;  // frames f: f * stride in [m_lo, m_hi - 1]
    const int nfr = a.m_hi >= a.m_lo + 1 ? (a.m_hi - 1) / c.stride - f_lo + 1 : 0;
    const bool staged = !DENSE && nloc > 0 && nfr > 0 && (long long)nfr * nloc * 2 <= (long long)R * ny;
    if (staged) {
      for (int idx = tid; idx < nfr * nloc; idx += kResThreads) {
        const int fr = idx / nloc, e = idx - fr * nloc;
        const size_t go = ((size_t)shot * c.nt_out + f_lo + fr) * c.nrec + rec_list[2 * e + 1];
        F[2 * idx] = a.g_x[go];
        F[2 * idx + 1] = a.g_y[go];
      }
      __syncthreads();
    } else if (RC == 0 && !DENSE && next_src >= a.m_lo + 1) {
      load_g(next_src);
    }
    // The receivers of this CTA sorted by the thread that owns their cell
    // (counting sort); entry (cell bit << 16) | e.  Register-resident form:
    // each owner adds its cells' residuals to its own registers.  Generic
    // form with one unit per thread and the launch's residuals staged in
    // shared memory: each owner adds them to its own cells of lam^{m+2} in
    // shared memory before its step, which only it reads this step, so no
    // barrier is needed (the adds inside the row updates instead measured
    // slower on rot256: 174 against 159 us per reverse launch).
    const bool own_inj = RC == 0 && !DENSE && staged && U.items <= kResThreads;
    const int own_rows = RC > 0 ? RCn : U.rc;  // rows of a thread's unit
    int inj_beg = 0, inj_end = 0;
    if ((RC > 0 || own_inj) && !DENSE && nloc > 0) {
      const int ncq = ny / 4;
      auto owner_of = [&](int e, int& bit) {
        const int off = rec_list[2 * e];
        const int s = off / ny, jj = off - s * ny;  // halo row s = local row + 1
        const int lr = s - 1, ch = lr / own_rows;
        bit = 4 * (lr - ch * own_rows) + (jj & 3);
        return ch * ncq + (jj >> 2);
      };
      for (int k = tid; k < kResThreads; k += kResThreads) inj_cnt[k] = 0;
      __syncthreads();
      for (int e = tid; e < nloc; e += kResThreads) {
        int bit;
        atomicAdd(&inj_cnt[owner_of(e, bit)], 1);
      }
      __syncthreads();
      if (tid == 0) {  // exclusive prefix sum (once per launch)
        int s = 0;
        for (int k = 0; k < kResThreads; ++k) {
          const int v = inj_cnt[k];
          inj_pos[k] = s;
          s += v;
        }
      }
      __syncthreads();
      inj_beg = inj_pos[tid];
      inj_end = inj_beg + inj_cnt[tid];
      __syncthreads();
      for (int e = tid; e < nloc; e += kResThreads) {
        int bit;
        const int o = owner_of(e, bit);
        inj[atomicAdd(&inj_pos[o], 1)] = (bit << 16) | e;
      }
      __syncthreads();
      // each owner sorts its few entries by cell and marks its cells
      for (int p = inj_beg + 1; p < inj_end; ++p) {
        const int v = inj[p];
        int q = p - 1;
        while (q >= inj_beg && inj[q] > v) { inj[q + 1] = inj[q]; --q; }
        inj[q + 1] = v;
      }
      if (RC > 0)
        for (int p = inj_beg; p < inj_end; ++p) RU.rmask |= 1u << (inj[p] >> 16);
    }
    // lam^{m_hi+1} is the imaging partner of u^{m_hi}: store it first
    if (tid == kStoreTid && a.lbuf && a.store_init) {
      fence_proxy_async();
      store_level(Lv(0), a.lbuf + (size_t)(a.m_hi + 1 - a.slot_base) * a.state_stride + shot_off,
                  (ptrdiff_t)N);
      bulk_commit();
    }
    Rhs rhs{nullptr, 0.f, 0, nullptr, nullptr, gs};
    // (m - 1) % stride and (m - 1) / stride as counters stepping down with m
    int sm_r = (a.m_hi - 1) % c.stride, sm_q = (a.m_hi - 1) / c.stride;
    auto lam_step = [&](int m, const float (&Cx)[RCn][4], const float (&Cy)[RCn][4], float (&Px)[RCn][4],
                        float (&Py)[RCn][4]) {
      const int t = a.m_hi - m;  // cur = lam^{m+1}, prev = lam^{m+2}, nxt = lam^m
      set_levels();
      expect_next();
      const bool src_step = sm_r == 0;
      const int frame = sm_q;
      if (sm_r == 0) { sm_r = c.stride - 1; --sm_q; } else { --sm_r; }
      if (RC > 0 && !DENSE && src_step && RU.rmask != 0u) {
        // lam^m = (2 lam^{m+1} - lam^{m+2} + ...) + g: the owner subtracts g
        // from its register copy of lam^{m+2} (every receiver of a cell summed)
        int p = inj_beg;
#pragma unroll
        for (int cb = 0; cb < 4 * RCn; ++cb) {
          if ((RU.rmask >> cb) & 1u) {
            float gxs = 0.f, gys = 0.f;
            while (p < inj_end && (inj[p] >> 16) == cb) {
              const int e = inj[p] & 0xffff;
              if (staged) {
                const int si = (frame - f_lo) * nloc + e;
                gxs += F[2 * si];
                gys += F[2 * si + 1];
              } else {
                const size_t go = ((size_t)shot * c.nt_out + frame) * c.nrec + rec_list[2 * e + 1];
                gxs += a.g_x[go];
                gys += a.g_y[go];
              }
              ++p;
            }
            Px[cb >> 2][cb & 3] += -gs * gxs;
            Py[cb >> 2][cb & 3] += -gs * gys;
          }
        }
      } else if (own_inj) {
        // generic form, owner adds: lam^m = (2 lam^{m+1} - lam^{m+2} + ...) + g
        // with g subtracted from the owner's cells of lam^{m+2}, one receiver
        // after another (as the shared-memory atomic adds below)
        if (src_step && inj_end > inj_beg) {
          const float* gst = F + 2 * (ptrdiff_t)(frame - f_lo) * nloc;
          float* p0 = T.comp(const_cast<float*>(x.prev), 0);
          float* p1 = T.comp(const_cast<float*>(x.prev), 1);
          for (int p = inj_beg; p < inj_end; ++p) {
            const int e = inj[p] & 0xffff;
            const int off = rec_list[2 * e];
            p0[off] += -gs * gst[2 * e];
            p1[off] += -gs * gst[2 * e + 1];
          }
        }
      } else if (RC == 0 && !DENSE && src_step) {
        // generic form: subtract g from the own copy of lam^{m+2} in shared
        // memory, which only the owning thread reads this step
#pragma unroll
        for (int h = 0; h < kRecPerThread; ++h) {
          const int e = tid + h * kResThreads;
          if (e < nloc) {
            const int off = rec_list[2 * e];
            const int si = (frame - f_lo) * nloc + e;
            const float vx = staged ? F[2 * si] : gnx[h];
            const float vy = staged ? F[2 * si + 1] : gny[h];
            atomicAdd(&T.comp(const_cast<float*>(x.prev), 0)[off], -gs * vx);
            atomicAdd(&T.comp(const_cast<float*>(x.prev), 1)[off], -gs * vy);
          }
        }
        next_src = m - c.stride;
        if (!staged && next_src >= a.m_lo + 1) load_g(next_src);
        __syncthreads();
      }
      rhs.gx = nullptr;
      rhs.gy = nullptr;
      if (DENSE && src_step) {
        rhs.gx = a.g_x + ((size_t)shot * c.nt_out + frame) * N + (size_t)r0 * ny;
        rhs.gy = a.g_y + ((size_t)shot * c.nt_out + frame) * N + (size_t)r0 * ny;
      }
      const bool w = step_wait(t);
      if (RC > 0) {
        if (RU.active)
          reg_step<true, DENSE, RCn>(T, ks, x, rhs, &bar[cl], (parity_bits >> cl) & 1u, w, c.err, RU, Cx, Cy,
                                     Px, Py);
      } else
        ring_step<true, DENSE>(T, ks, x, rhs, &bar[cl], (parity_bits >> cl) & 1u, w, c.err, U);
      if (w) parity_bits ^= 1u << cl;
      if (tid == kStoreTid) bulk_wait_read_all();
      __syncthreads();
      t_last = t;
      next_level();
      if (tid == kStoreTid && a.lbuf && m - a.slot_base >= 0) {
        fence_proxy_async();
        store_level(x.nxt, a.lbuf + (size_t)(m - a.slot_base) * a.state_stride + shot_off,
                    (ptrdiff_t)N);
        bulk_commit();
      }
    };
    if constexpr (RC > 0) {
      int m = a.m_hi;
      for (; m - 1 >= a.m_lo + 1; m -= 2) {
        lam_step(m, Ax, Ay, Bx, By);      // cur A, prev B -> B holds lam^m
        lam_step(m - 1, Bx, By, Ax, Ay);  // cur B, prev A -> A holds lam^{m-1}
      }
      if (m >= a.m_lo + 1) lam_step(m, Ax, Ay, Bx, By);
    } else {
      for (int m = a.m_hi; m >= a.m_lo + 1; --m) lam_step(m, Ax, Ay, Bx, By);
    }
  }
  // The neighbours' last pushes land in this CTA's level of step t_last + 1:
  // wait for them before this CTA's shared memory goes away.
  if (t_last >= 0 && halo_bytes > 0)
    halo_wait(&bar[(t_last + 1) % 3], (parity_bits >> ((t_last + 1) % 3)) & 1u, c.err);
  if (tid == kStoreTid) bulk_wait_all();
  __syncthreads();
  if (!is_fwd && a.m_hi >= a.m_lo + 1 && al16(a.lam_save) && al16(a.lam_save + a.save_stride)) {
    // lam^{m_lo+1} (level of step t_last + 1) and lam^{m_lo+2} -> lam_save,
    // own rows by bulk copies
    if (tid == 0) {
      fence_proxy_async();
      store_level(Lv((t_last + 1) % 3), a.lam_save + shot_off, (ptrdiff_t)N);
      store_level(Lv(t_last % 3), a.lam_save + a.save_stride + shot_off, (ptrdiff_t)N);
      bulk_commit();
      bulk_wait_all();
    }
    __syncthreads();
  } else if (!is_fwd && a.m_hi >= a.m_lo + 1) {
    // lam^{m_lo+1} (level of step t_last + 1) and lam^{m_lo+2} -> lam_save
    float* last = Lv((t_last + 1) % 3);
    float* before = Lv(t_last % 3);
    for (int e = tid; e < 2 * rows * ny; e += kResThreads) {
      const int comp = e / (rows * ny);
      const int rem = e - comp * rows * ny;
      const int lr = rem / ny, j = rem - lr * ny;
      const size_t gidx = shot_off + (size_t)comp * N + (size_t)(r0 + lr) * ny + j;
      a.lam_save[gidx] = T.comp(last, comp)[T.at(lr + 1, j)];
      a.lam_save[a.save_stride + gidx] = T.comp(before, comp)[T.at(lr + 1, j)];
    }
  }
  cluster.sync();  // no CTA leaves while a neighbour may still address it
}

// ---------------------------------------------------------------- host side
size_t resident_smem_bytes(const ResCommon& c) {
  const size_t level = 2 * (size_t)(c.R + 2) * c.ny * sizeof(float);
  const size_t tail = (2 * kResMaxRec + 4) * sizeof(int) + 4 * sizeof(uint64_t) +
                      (kResMaxRec + 2 * kResThreads) * sizeof(int) + 16;
  return 3 * level + (size_t)c.R * c.ny * sizeof(float) + tail;
}

// Raise the kernel's dynamic shared-memory limit to at least `smem` (once per
// kernel and size; the limit only grows).
static cudaError_t configure(const void* fn, size_t smem) {
  static std::mutex mu;
  static std::vector<std::pair<const void*, size_t>> done;
  std::lock_guard<std::mutex> lock(mu);
  for (auto& kv : done)
    if (kv.first == fn && kv.second >= smem) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  for (auto& kv : done)
    if (kv.first == fn) { kv.second = smem; return cudaSuccess; }
  done.push_back({fn, smem});
  return cudaSuccess;
}

static int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
  }
  return n;
}

int resident_img_clusters(const ResCommon& c) {
  // IMG clusters per shot row of the grid: fill the SMs the FWD and LAM
  // clusters leave free, at least one, at most eight
  const int free_sm = sm_count() - 2 * c.S * c.CL;
  int z = free_sm / (c.CL * c.S);
  if (z < 1) z = 1;
  if (z > 8) z = 8;
  return z;
}

// Feasibility answers per (kernel, cluster size, shared memory): the
// attribute and occupancy queries run once, so later calls (for example
// during stream capture) make no CUDA runtime calls here.
struct FeasKey {
  bool dense;
  int CL;
  size_t smem;
};
static std::mutex g_feas_mu;
static std::vector<std::pair<FeasKey, bool>> g_feas;

static bool feasible_uncached(const ResCommon& c, bool dense, size_t smem);

constexpr size_t kResSmemLimit = 220 * 1024;

bool resident_possible(int mode, int nx, int ny) {
  if (mode != kModeScalar || ny % 4 != 0 || nx < 1) return false;
  ResCommon c{};
  c.ny = ny;
  c.R = (nx + 15) / 16;  // the most CTAs per cluster give the fewest rows per CTA
  return resident_smem_bytes(c) <= kResSmemLimit;
}

bool resident_feasible(const ResCommon& c, bool dense) {
  if (c.CL < 1 || c.CL > 16 || c.ny % 4 != 0 || c.nrec > kResMaxRec) return false;
  if ((c.CL - 1) * c.R >= c.nx) return false;  // every CTA owns >= 1 row
  const size_t smem = resident_smem_bytes(c);
  if (smem > kResSmemLimit) return false;
  std::lock_guard<std::mutex> lock(g_feas_mu);
  for (const auto& kv : g_feas)
    if (kv.first.dense == dense && kv.first.CL == c.CL && kv.first.smem == smem) return kv.second;
  const bool ok = feasible_uncached(c, dense, smem);
  g_feas.push_back({FeasKey{dense, c.CL, smem}, ok});
  return ok;
}

// Rows per chunk of the register-resident form for this problem (the same
// split as unit_of for a CTA of R rows): 1, 2 or 4, or 0 when a thread would
// hold more than one unit or more than four rows (the generic form runs).
static int resident_rc(const ResCommon& c) {
  const int ncq = c.ny / 4;
  if (ncq < 1 || ncq > kResThreads) return 0;
  const int nchunk = kResThreads / ncq;
  const int rc = (c.R + nchunk - 1) / nchunk;
  // (4-row chunks measured slower in this form than in the generic one:
  // rot256 adjoint launches 214 vs 161 us)
  if (rc != 1 && rc != 2) return 0;
  // every CTA's rows (R, and the last CTA's remainder) in whole chunks
  const int last = c.nx - (c.CL - 1) * c.R;
  return (c.R % rc == 0 && last % rc == 0) ? rc : 0;
}

static const void* resident_fn(bool dense, int rc) {
  switch (rc) {
    case 1: return dense ? (const void*)resident_kernel<true, 1> : (const void*)resident_kernel<false, 1>;
    case 2: return dense ? (const void*)resident_kernel<true, 2> : (const void*)resident_kernel<false, 2>;
    default: return dense ? (const void*)resident_kernel<true, 0> : (const void*)resident_kernel<false, 0>;
  }
}

static bool feasible_uncached(const ResCommon& c, bool dense, size_t smem) {
  const void* fn = resident_fn(dense, resident_rc(c));
  if (configure(fn, smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.CL, 1, 1);
  cfg.blockDim = dim3(kResThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return clusters >= 1;
}

cudaError_t launch_resident(const ResCommon& c, const ResFwd& f, const ResLam& a, const ResImg& g,
                            bool run_fwd, bool run_lam, bool run_img, bool dense, cudaStream_t st) {
  if (!run_fwd && !run_lam && !run_img) return cudaSuccess;
  const size_t smem = resident_smem_bytes(c);
  const int rcf = resident_rc(c);
  const void* fn = resident_fn(dense, rcf);
  cudaError_t e = configure(fn, smem);
  if (e != cudaSuccess) return e;
  ResRoles roles{-1, -1, -1, 0};
  int z = 0;
  if (run_lam) roles.z_lam = z++;
  if (run_fwd) roles.z_fwd = z++;
  if (run_img) {
    roles.z_img = z;
    roles.n_img_z = resident_img_clusters(c);
    z += roles.n_img_z;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.CL, c.S, z);
  cfg.blockDim = dim3(kResThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int cls = (run_lam || run_img) ? kProfAdjoint : kProfForward;
  const double cells = (double)c.S * c.nx * c.ny;
  const double bytes =
      cells * ((run_fwd ? alg_bytes_forward(kModeScalar) * (f.i1 - f.i0) : 0.0) +
               (run_lam ? 24.0 * (a.m_hi - a.m_lo) : 0.0) +   // lam recursion: 3 x 8 B
               (run_img ? 16.0 * (g.n_hi - g.n_lo + 1) : 0.0));  // imaging: read lam, u
  return tracked_launch(cls, st, [&] {
    switch (rcf * 2 + (dense ? 1 : 0)) {
      case 2: cudaLaunchKernelEx(&cfg, resident_kernel<false, 1>, c, f, a, g, roles); break;
      case 3: cudaLaunchKernelEx(&cfg, resident_kernel<true, 1>, c, f, a, g, roles); break;
      case 4: cudaLaunchKernelEx(&cfg, resident_kernel<false, 2>, c, f, a, g, roles); break;
      case 5: cudaLaunchKernelEx(&cfg, resident_kernel<true, 2>, c, f, a, g, roles); break;
      case 1: cudaLaunchKernelEx(&cfg, resident_kernel<true, 0>, c, f, a, g, roles); break;
      default: cudaLaunchKernelEx(&cfg, resident_kernel<false, 0>, c, f, a, g, roles); break;
    }
  }, bytes);
}

}  // namespace ernn
