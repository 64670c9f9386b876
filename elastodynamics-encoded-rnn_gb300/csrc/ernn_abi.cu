// C ABI entry points of libernn_gb300.so (declared in include/ernn.h) and the
// host-side time-loop driver: step schedule, checkpoint/recompute plan,
// workspace layout.  Every launch goes on the caller's stream; nothing here
// synchronises the host or allocates device memory.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstring>

#include "ernn.h"
#include "ernn_launch.h"
#include "ernn_resident.h"
#include "ernn_tma.h"

namespace ernn {
namespace {

constexpr size_t kAlign = 256;
constexpr double kPi = 3.14159265358979323846;
// segment length of the resident reverse pass when the tape keeps every state
constexpr int kResStoreAllSegment = 128;
inline size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Workspace plan of one problem.
struct Plan {
  int S, nx, ny, nt, k, nseg, nt_out, nblocks, npart, kres;
  int ncoef;  // coefficient blocks: nshots with ERNN_FLAG_SHOT_CONSTANTS, else 1
  bool store_all;
  size_t N, state_bytes;
  // tape
  size_t t_coef, t_A, t_B, t_store, t_total_tape, t_total_notape;
  // adjoint scratch
  size_t s_coef, s_LA, s_LB, s_seg, s_lbuf, s_gacc, s_part, s_tflags, s_total;
  // instances on a canvas: tile table (tape and scratch), a zero state (scratch)
  bool inst;
  size_t inst_bytes, t_inst, s_inst, s_zero;
};

// Upper bound of the tile-table entries of any placement of S instances on
// an nx x ny canvas (each instance's tiling has at most one partial tile row
// and column).
inline size_t inst_table_bound(int nx, int ny, int S) {
  return ((size_t)(nx + kInstTileRows - 1) / kInstTileRows + S) * ((size_t)(ny + 63) / 64 + S);
}

Plan make_plan(const ErnnProblem& p) {
  Plan pl{};
  pl.S = p.nshots; pl.nx = p.nx; pl.ny = p.ny; pl.nt = p.nt;
  pl.k = p.ckpt_k < p.nt ? p.ckpt_k : p.nt;
  pl.nseg = (p.nt + pl.k - 1) / pl.k;
  pl.store_all = (pl.nseg == 1);
  pl.nt_out = (p.nt + p.stride - 1) / p.stride;
  pl.N = (size_t)p.nx * p.ny;
  pl.inst = (p.flags & ERNN_FLAG_INSTANCES) != 0;
  // instances share the canvas's one state plane
  pl.state_bytes = align_up((size_t)(pl.inst ? 1 : p.nshots) * 2 * pl.N * sizeof(float));
  const dim3 g = step_grid(p.nx, p.ny, pl.inst ? 1 : p.nshots);
  pl.nblocks = (int)(g.x * g.y * g.z);
  pl.ncoef = (p.flags & (ERNN_FLAG_SHOT_CONSTANTS | ERNN_FLAG_INSTANCES)) ? p.nshots : 1;
  pl.inst_bytes = pl.inst ? align_up(inst_table_bound(p.nx, p.ny, p.nshots) * sizeof(int4)) +
                                align_up((size_t)2 * p.nshots * sizeof(int4))
                          : 0;
  size_t off = 0;
  pl.t_coef = off; off += align_up((size_t)pl.ncoef * sizeof(Coef));
  pl.t_inst = off; off += pl.inst_bytes;
  pl.t_A = off; off += pl.state_bytes;
  pl.t_B = off; off += pl.state_bytes;
  pl.t_total_notape = off;
  pl.t_store = off;
  if (pl.store_all) off += (size_t)p.nt * pl.state_bytes;           // u^1..u^nt
  else off += (size_t)(pl.nseg - 1) * 2 * pl.state_bytes;          // (u^{jk}, u^{jk-1})
  pl.t_total_tape = off;
  off = 0;
  pl.s_coef = off; off += align_up((size_t)pl.ncoef * sizeof(Coef));
  pl.s_inst = off; off += pl.inst_bytes;
  pl.s_zero = off; if (pl.inst) off += pl.state_bytes;  // u^0 = u^{-1} = 0 of the first segment
  pl.s_LA = off; off += pl.state_bytes;
  pl.s_LB = off; off += pl.state_bytes;
  // two recompute segments: the cluster-resident path recomputes segment j-1
  // while the adjoint consumes segment j
  // (instances: the tiled path only, one segment)
  pl.s_seg = off; if (!pl.store_all) off += (size_t)(pl.inst ? 1 : 2) * pl.k * pl.state_bytes;
  // lam buffers of the resident reverse pass: two segments of kres steps,
  // only where that path can run
  pl.kres = pl.store_all ? (p.nt < kResStoreAllSegment ? p.nt : kResStoreAllSegment) : pl.k;
  if (!resident_possible(p.mode, p.nx, p.ny) || pl.inst) pl.kres = 0;
  pl.s_lbuf = off; off += (size_t)2 * pl.kres * pl.state_bytes;
  pl.s_gacc = off;
  if (p.mode == kModeDField) off += align_up((size_t)p.nshots * pl.N * sizeof(float));
  if (p.mode == kModeFields) off += align_up((size_t)p.nshots * 6 * pl.N * sizeof(float));
  pl.s_part = off;
  // partial-sum rows: plain per-step path one per block; resident path one
  // per imaging CTA (at most 8 clusters of 16 per shot); tiled path one per
  // CTA, kTiledRowsPerShot per shot with per-shot constants
  pl.npart = pl.nblocks > p.nshots * 16 * 8 ? pl.nblocks : p.nshots * 16 * 8;
  if (pl.ncoef > 1 && pl.npart < p.nshots * kTiledRowsPerShot) pl.npart = p.nshots * kTiledRowsPerShot;
  if (p.mode == kModeScalar) off += align_up((size_t)pl.npart * 8 * sizeof(double));
  // receiver table of the tiled adjoint: one byte per (shot, tile), sized for
  // its smallest tiles (64 x 16)
  pl.s_tflags = off;
  if (p.record == kRecordReceivers)
    off += align_up(pl.inst ? inst_table_bound(p.nx, p.ny, p.nshots) : tma_tiles(p.nx, p.ny, p.nshots, 16));
  pl.s_total = off;
  return pl;
}

int validate(const ErnnProblem* p) {
  if (p == nullptr) return ERNN_ERR_INVALID;
  if (p->nshots < 1 || p->nshots > 65535 || p->nx < 1 || p->ny < 1 || p->nt < 1 ||
      p->stride < 1 || p->ckpt_k < 1)
    return ERNN_ERR_INVALID;
  if ((int64_t)p->nx * p->ny >= ((int64_t)1 << 31) || p->nx > 2000000) return ERNN_ERR_INVALID;
  if (p->mode < kModeScalar || p->mode > kModeFields) return ERNN_ERR_INVALID;
  if (p->record != kRecordFields && p->record != kRecordReceivers) return ERNN_ERR_INVALID;
  if (p->record == kRecordReceivers && p->nrec < 1) return ERNN_ERR_INVALID;
  if (p->src_comp != 0 && p->src_comp != 1) return ERNN_ERR_INVALID;
  if (p->src_bx < 0 || p->src_by < 0) return ERNN_ERR_INVALID;
  if (p->path < ERNN_PATH_AUTO || p->path > ERNN_PATH_TILED) return ERNN_ERR_INVALID;
  if ((p->flags & ~(ERNN_FLAG_SHOT_CONSTANTS | ERNN_FLAG_INSTANCES | ERNN_FLAG_TALL_TILES)) != 0)
    return ERNN_ERR_INVALID;
  if ((p->flags & ERNN_FLAG_SHOT_CONSTANTS) && p->mode != kModeScalar) return ERNN_ERR_INVALID;
  if ((p->flags & ERNN_FLAG_INSTANCES) &&
      (p->mode != kModeScalar || p->record != kRecordReceivers || p->nshots > kMaxInstances ||
       p->nx >= 65536 || p->ny >= 65536))
    return ERNN_ERR_INVALID;
  if (!(p->h > 0.0) || !(p->dt > 0.0) || !std::isfinite(p->h) || !std::isfinite(p->dt))
    return ERNN_ERR_INVALID;
  // Sizes that the plan forms in 64-bit (states of the tape and scratch: at
  // most nt + 2 ckpt_k + 2 resident segments + a few) and in 32-bit (blocks
  // of one plain step launch) must not wrap: such a problem is refused
  // instead of being given a workspace size that is too small.
  const double state_bytes =
      (double)((p->flags & ERNN_FLAG_INSTANCES) ? 1 : p->nshots) * 2.0 * (double)p->nx * p->ny * 4.0;
  if (state_bytes * (3.0 * (double)p->nt + 16.0) >= 4.0e18) return ERNN_ERR_INVALID;
  if ((double)p->nshots * ((p->nx + 7) / 8) * ((p->ny + 31) / 32) >= 2.0e9) return ERNN_ERR_INVALID;
  return ERNN_OK;
}

int validate_inputs(const ErnnProblem* p, const ErnnInputs* in) {
  if (in == nullptr || in->C == nullptr || in->rho == nullptr || in->src_signal == nullptr)
    return ERNN_ERR_INVALID;
  if (p->mode == kModeDField && in->D == nullptr) return ERNN_ERR_INVALID;
  if ((size_t)p->src_bx * p->src_by > 0 && (in->src_map == nullptr || in->src_origin == nullptr))
    return ERNN_ERR_INVALID;
  if (p->record == kRecordReceivers && in->rec_idx == nullptr) return ERNN_ERR_INVALID;
  return ERNN_OK;
}

inline char* at(void* base, size_t off) { return static_cast<char*>(base) + off; }
inline float* fat(void* base, size_t off) { return reinterpret_cast<float*>(at(base, off)); }

#define ERNN_CUDA(expr)                      \
  do {                                       \
    if ((expr) != cudaSuccess) return ERNN_ERR_CUDA; \
  } while (0)

FwdStep base_fwd(const ErnnProblem& p, const ErnnInputs& in, const Coef* coef, int nt_out) {
  FwdStep a;
  std::memset(&a, 0, sizeof(a));
  a.nx = p.nx; a.ny = p.ny; a.S = p.nshots; a.nt = p.nt;
  a.frame = -1; a.gframe = -1; a.nt_out = nt_out;
  a.coef = coef;
  // one coefficient block per shot (per-shot constants) or per instance
  a.coef_stride = (p.flags & (ERNN_FLAG_SHOT_CONSTANTS | ERNN_FLAG_INSTANCES)) ? 1 : 0;
  a.field = (p.mode == kModeFields) ? in.C : in.D;
  a.src_signal = in.src_signal;
  a.src_map = in.src_map;
  a.src_origin = in.src_origin;
  a.bx = p.src_bx; a.by = p.src_by; a.src_comp = p.src_comp;
  a.rec_idx = in.rec_idx;
  a.nrec = p.nrec;
  return a;
}

std::atomic<int32_t> g_last_path{ERNN_PATH_AUTO};

// Tiled per-step kernels: requested (ERNN_PATH_TILED, an error when the
// problem is not eligible) or chosen by ERNN_PATH_AUTO when eligible and one
// step has at least four 64 x 32 tiles per SM.  The tiled kernels are
// persistent (2-3 CTAs of 72-111 KB shared memory per SM, each streaming
// several tiles); below that size the plain per-step kernels, many small
// CTAs per SM, hide latency better and share the GPU better with other
// streams' work.
int use_tiled(const ErnnProblem& p, int* tiled) {
  *tiled = 0;
  if (p.path == ERNN_PATH_STEP) return ERNN_OK;
  const bool ok = tma_eligible(p.mode, p.nx, p.ny, p.nshots);
  if (p.path == ERNN_PATH_TILED) {
    if (!ok) return ERNN_ERR_UNSUPPORTED;
    *tiled = 1;
    return ERNN_OK;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return ERNN_ERR_CUDA;
  *tiled = ok && tma_tiles(p.nx, p.ny, p.nshots) >= 4 * (size_t)sms;
  return ERNN_OK;
}

// Cluster-resident configuration: CL CTAs of R rows each.  Returns false when
// the problem does not fit the path (mode, alignment, receivers, memory).
bool pick_resident(const ErnnProblem& p, const ErnnInputs& in, Coef* coef, ResCommon& rc) {
  if (!resident_possible(p.mode, p.nx, p.ny)) return false;  // (the plan reserved no lam buffers)
  if (p.record == kRecordReceivers && p.nrec > kResMaxRec) return false;
  rc.nx = p.nx; rc.ny = p.ny; rc.S = p.nshots; rc.nt = p.nt; rc.stride = p.stride;
  rc.nt_out = (p.nt + p.stride - 1) / p.stride;
  rc.coef = coef;
  rc.coef_stride = (p.flags & ERNN_FLAG_SHOT_CONSTANTS) ? 1 : 0;
  rc.src_signal = in.src_signal; rc.src_map = in.src_map; rc.src_origin = in.src_origin;
  rc.bx = p.src_bx; rc.by = p.src_by; rc.src_comp = p.src_comp;
  rc.rec_idx = (p.record == kRecordReceivers) ? in.rec_idx : nullptr;
  rc.nrec = (p.record == kRecordReceivers) ? p.nrec : 0;
  rc.err = &coef->err;
  for (int CL = 16; CL >= 1; CL /= 2) {
    if (CL > p.nx) continue;
    rc.CL = CL;
    rc.R = (p.nx + CL - 1) / CL;
    if ((CL - 1) * rc.R >= p.nx) continue;
    if (resident_feasible(rc, p.record == kRecordFields)) return true;
  }
  return false;
}

int resident_forward(const ErnnProblem& p, const Plan& pl, ResCommon& rc, float* out_ux,
                     float* out_uy, void* tape, int with_tape, cudaStream_t st) {
  ResFwd f;
  std::memset(&f, 0, sizeof(f));
  f.i0 = 0; f.i1 = p.nt;
  f.state_stride = pl.state_bytes / sizeof(float);
  if (with_tape && pl.store_all) f.states = fat(tape, pl.t_store);
  if (with_tape && !pl.store_all) {
    f.ckpt = fat(tape, pl.t_store);
    f.ck_k = pl.k;
    f.ck_nseg = pl.nseg;
  }
  const bool dense = (p.record == kRecordFields);
  if (dense) { f.hist_x = out_ux; f.hist_y = out_uy; }
  else { f.tr_x = out_ux; f.tr_y = out_uy; }
  ResLam a;
  std::memset(&a, 0, sizeof(a));
  ResImg g;
  std::memset(&g, 0, sizeof(g));
  ERNN_CUDA(launch_resident(rc, f, a, g, true, false, false, dense, st));
  return ERNN_OK;
}

// Reverse pass of the resident path, in segments of ks steps, one launch per
// segment j (from the last): LAM runs the adjoint over segment j and stores
// every lam into lbuf[j & 1]; FWD recomputes segment j from its checkpoint
// into ubuf[j & 1] (not needed when the tape holds every state); IMG forms the
// imaging sums of segment j + 1 from the buffers of the previous launch.
int resident_adjoint(const ErnnProblem& p, const Plan& pl, ResCommon& rc, const float* g_ux,
                     const float* g_uy, void* tape, void* scratch, double* partials,
                     int* img_rows, cudaStream_t st) {
  const size_t ss = pl.state_bytes / sizeof(float);
  const bool dense = (p.record == kRecordFields);
  const int ks = pl.kres;
  const int nseg = (p.nt + ks - 1) / ks;
  auto lbuf = [&](int j) { return fat(scratch, pl.s_lbuf + (size_t)(j & 1) * ks * pl.state_bytes); };
  auto ubuf = [&](int j) -> float* {
    if (pl.store_all) return fat(tape, pl.t_store + (size_t)j * ks * pl.state_bytes);  // u^{jk+1}..
    return fat(scratch, pl.s_seg + (size_t)(j & 1) * pl.k * pl.state_bytes);
  };
  auto ck = [&](int j, int lev) -> const float* {
    if (j == 0) return nullptr;
    if (lev == 1 && j * pl.k - 1 == 0) return nullptr;  // u^0 = 0 (k == 1)
    return fat(tape, pl.t_store + ((size_t)(j - 1) * 2 + lev) * pl.state_bytes);
  };
  ResLam a;
  std::memset(&a, 0, sizeof(a));
  a.lam_save = fat(scratch, pl.s_LA);
  a.save_stride = ss;  // LB follows LA
  a.g_x = g_ux; a.g_y = g_uy;
  a.state_stride = ss;
  ResFwd f;
  std::memset(&f, 0, sizeof(f));
  f.state_stride = ss;
  ResImg g;
  std::memset(&g, 0, sizeof(g));
  g.state_stride = ss;
  g.partials = partials;
  *img_rows = resident_img_clusters(rc) * rc.S * rc.CL;
  for (int j = nseg - 1; j >= -1; --j) {
    const bool run_lam = j >= 0;
    bool run_fwd = false;
    if (run_lam) {
      a.m_hi = (j + 1) * ks < p.nt ? (j + 1) * ks : p.nt;
      a.m_lo = j * ks;
      a.first = (j == nseg - 1) ? 1 : 0;
      a.lbuf = lbuf(j);
      a.slot_base = j * ks + 2;
      a.store_init = (a.m_hi <= p.nt - 1) ? 1 : 0;
      if (!pl.store_all) {  // recompute u^{jk+1} .. u^{min((j+1)k, nt-1)}
        f.i0 = j * pl.k;
        f.i1 = (j + 1) * pl.k < p.nt - 1 ? (j + 1) * pl.k : p.nt - 1;
        f.init_cur = ck(j, 0);
        f.init_prev = ck(j, 1);
        f.states = ubuf(j);
        run_fwd = f.i1 > f.i0;
      }
    }
    const int jj = j + 1;  // segment imaged in this launch
    g.n_lo = jj * ks + 1;
    g.n_hi = (jj + 1) * ks < p.nt - 1 ? (jj + 1) * ks : p.nt - 1;
    const bool run_img = jj <= nseg - 1 && g.n_hi >= g.n_lo;
    if (run_img) {
      g.lbuf = lbuf(jj);
      g.ubuf = ubuf(jj);
    }
    ERNN_CUDA(launch_resident(rc, f, a, g, run_fwd, run_lam, run_img, dense, st));
  }
  return ERNN_OK;
}

// Instances of a canvas problem (ERNN_FLAG_INSTANCES), checked and ordered
// by decreasing step count; upto[g] = tiles of the first g of that order.
struct InstPlan {
  InstDesc d;
  int upto[kMaxInstances + 1];
  // tiles of forward (or recompute) step i: instances with nt > i
  int fwd_tiles(int i) const {
    int g = 0;
    while (g < d.count && d.nt[g] > i) ++g;
    return upto[g];
  }
  // tiles of adjoint step m: instances with nt >= m
  int adj_tiles(int m) const {
    int g = 0;
    while (g < d.count && d.nt[g] >= m) ++g;
    return upto[g];
  }
};

int plan_instances(const ErnnProblem& p, const ErnnInstances* in, InstPlan* ip) {
  if (!(p.flags & ERNN_FLAG_INSTANCES) || in == nullptr || in->count != p.nshots || in->x0 == nullptr ||
      in->y0 == nullptr || in->nx == nullptr || in->ny == nullptr || in->nt == nullptr)
    return ERNN_ERR_INVALID;
  const int S = in->count;
  for (int k = 0; k < S; ++k) {
    const int x0 = in->x0[k], y0 = in->y0[k], nx = in->nx[k], ny = in->ny[k], nt = in->nt[k];
    if (x0 < 0 || y0 < 0 || nx < 1 || ny < 4 || y0 % 4 != 0 || ny % 4 != 0 || (int64_t)x0 + nx > p.nx ||
        (int64_t)y0 + ny > p.ny || nt < 1 || nt > p.nt)  // (64-bit sums: no wrap past the canvas)
      return ERNN_ERR_INVALID;
  }
  // regions at least one cell apart: those cells stay zero, the instances'
  // ghost rings
  for (int a = 0; a < S; ++a)
    for (int b = a + 1; b < S; ++b) {
      const bool apart = in->x0[a] + in->nx[a] + 1 <= in->x0[b] || in->x0[b] + in->nx[b] + 1 <= in->x0[a] ||
                         in->y0[a] + in->ny[a] + 1 <= in->y0[b] || in->y0[b] + in->ny[b] + 1 <= in->y0[a];
      if (!apart) return ERNN_ERR_INVALID;
    }
  int order[kMaxInstances];
  for (int k = 0; k < S; ++k) order[k] = k;
  std::stable_sort(order, order + S, [&](int u, int v) { return in->nt[u] > in->nt[v]; });
  ip->d.count = S;
  ip->upto[0] = 0;
  for (int g = 0; g < S; ++g) {
    const int k = order[g];
    ip->d.id[g] = k;
    ip->d.x0[g] = in->x0[k];
    ip->d.y0[g] = in->y0[k];
    ip->d.nx[g] = in->nx[k];
    ip->d.ny[g] = in->ny[k];
    ip->d.nt[g] = in->nt[k];
    ip->d.base[g] = ip->upto[g];
    ip->upto[g + 1] = ip->upto[g] + inst_tiles(in->nx[k], in->ny[k]);
  }
  return ERNN_OK;
}

}  // namespace

void record_last_path(int32_t path) { g_last_path.store(path, std::memory_order_relaxed); }

}  // namespace ernn

using namespace ernn;

extern "C" {

int ernn_abi_version(void) { return ERNN_ABI_VERSION; }

const char* ernn_error_string(int code) {
  switch (code) {
    case ERNN_OK: return "ok";
    case ERNN_ERR_INVALID: return "invalid argument (null pointer, size or enum out of range)";
    case ERNN_ERR_WORKSPACE: return "workspace smaller than the size query returned";
    case ERNN_ERR_CUDA: return "CUDA runtime call failed";
    case ERNN_ERR_UNSTABLE: return "leapfrog stability bound violated for these constants";
    case ERNN_ERR_TIMEOUT: return "bounded device-side wait timed out";
    case ERNN_ERR_UNSUPPORTED: return "request not supported by this library";
    default: return "unknown error code";
  }
}

int ernn_validate(const ErnnProblem* p) { return validate(p); }

size_t ernn_tape_bytes(const ErnnProblem* p, int with_tape) {
  if (validate(p) != ERNN_OK) return 0;
  const Plan pl = make_plan(*p);
  return with_tape ? pl.t_total_tape : pl.t_total_notape;
}

size_t ernn_adjoint_scratch_bytes(const ErnnProblem* p) {
  if (validate(p) != ERNN_OK) return 0;
  return make_plan(*p).s_total;
}

int ernn_check_stability(const double* C, double rho, double h, double dt, double* courant) {
  if (C == nullptr || !(rho > 0.0) || !(h > 0.0) || !(dt > 0.0)) return ERNN_ERR_INVALID;
  // Symbol of -(h^2) A on the Fourier mode exp(i(tx*i + ty*j)):
  //   a = 4 sin^2(tx/2), b = 4 sin^2(ty/2), d = sin(tx) sin(ty)
  //   Mxx = C11 a + C66 b + 2 C16 d,  Myy = C66 a + C22 b + 2 C26 d,
  //   Mxy = C16 a + C26 b + (C12 + C66) d.
  // Leapfrog is stable when every eigenvalue of (dt^2 / (rho h^2)) M lies in [0, 4].
  const double q = dt * dt / (rho * h * h);
  const int n = 128;
  double worst = 0.0;
  bool indefinite = false;
  for (int u = 0; u <= n; ++u) {
    for (int v = 0; v <= n; ++v) {
      const double tx = kPi * u / n, ty = kPi * v / n;
      const double a = 4.0 * std::sin(tx / 2) * std::sin(tx / 2);
      const double b = 4.0 * std::sin(ty / 2) * std::sin(ty / 2);
      for (int sgn = -1; sgn <= 1; sgn += 2) {
        const double d = sgn * std::sin(tx) * std::sin(ty);
        const double mxx = C[0] * a + C[5] * b + 2 * C[3] * d;
        const double myy = C[5] * a + C[1] * b + 2 * C[4] * d;
        const double mxy = C[3] * a + C[4] * b + (C[2] + C[5]) * d;
        const double tr = mxx + myy, det = mxx * myy - mxy * mxy;
        const double disc = std::sqrt(std::fmax(tr * tr / 4 - det, 0.0));
        const double lmax = tr / 2 + disc, lmin = tr / 2 - disc;
        if (lmin < -1e-9 * std::fabs(lmax)) indefinite = true;
        if (q * lmax / 4.0 > worst) worst = q * lmax / 4.0;
      }
    }
  }
  if (courant) *courant = worst;
  return (worst > 1.0 || indefinite) ? ERNN_ERR_UNSTABLE : ERNN_OK;
}

int ernn_operator(int32_t nshots, int32_t nx, int32_t ny, int32_t mode, double h, const float* C,
                  const float* D, const float* rho, const float* ux, const float* uy,
                  const float* fx, const float* fy, float* Lux, float* Luy, void* stream) {
  if (nshots < 1 || nx < 1 || ny < 1 || mode < 0 || mode > 2 || !(h > 0.0)) return ERNN_ERR_INVALID;
  if (C == nullptr || rho == nullptr || ux == nullptr || uy == nullptr || Lux == nullptr ||
      Luy == nullptr || (mode == kModeDField && D == nullptr))
    return ERNN_ERR_INVALID;
  ERNN_CUDA(launch_operator(nshots, nx, ny, mode, h, C, D, rho, ux, uy, fx, fy, Lux, Luy,
                            (cudaStream_t)stream));
  return ERNN_OK;
}

// Tile rows of the tiled kernels: 32 with ERNN_FLAG_TALL_TILES and always in
// the D-field mode (its forward measured faster with them: 8 x 512^2 shots,
// 81.3 -> 75.6 ms per inversion iteration), else 16.
static int tile_rows_of(const ErnnProblem& p) {
  return ((p.flags & ERNN_FLAG_TALL_TILES) || p.mode == kModeDField) ? 32 : 16;
}

// The forward time loop of ernn_forward and, with an instance plan `ip`, of
// ernn_forward_instances.
static int forward_impl(const ErnnProblem* p, const ErnnInputs* in, const InstPlan* ip, float* out_ux,
                        float* out_uy, void* tape, size_t tape_bytes, int with_tape, void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  if ((rc = validate_inputs(p, in))) return rc;
  if (out_ux == nullptr || out_uy == nullptr || tape == nullptr) return ERNN_ERR_INVALID;
  if ((ip != nullptr) != ((p->flags & ERNN_FLAG_INSTANCES) != 0)) return ERNN_ERR_INVALID;
  const Plan pl = make_plan(*p);
  if (tape_bytes < (with_tape ? pl.t_total_tape : pl.t_total_notape)) return ERNN_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  Coef* coef = reinterpret_cast<Coef*>(at(tape, pl.t_coef));
  ERNN_CUDA(launch_coef(p->mode, in->C, in->rho, p->h, p->dt, coef, st, pl.ncoef));

  InstTiles itab{nullptr, nullptr, 0};
  if (ip != nullptr) {
    // instances: the tiled kernels over the tile table only.  A and B start
    // at zero (B stands for u^0); the stored states need only the instances'
    // ghost rings zeroed (the cells between the regions are never written,
    // and outside the regions the kernels read only the rings); trace frames
    // past an instance's steps are zero
    if (p->path != ERNN_PATH_AUTO && p->path != ERNN_PATH_TILED) return ERNN_ERR_UNSUPPORTED;
    if (!tma_eligible(p->mode, p->nx, p->ny, 1)) return ERNN_ERR_UNSUPPORTED;
    itab.tiles = reinterpret_cast<int4*>(at(tape, pl.t_inst));
    itab.box = reinterpret_cast<int4*>(at(tape, pl.t_inst + align_up(inst_table_bound(p->nx, p->ny, p->nshots) *
                                                                       sizeof(int4))));
    ERNN_CUDA(launch_inst_table(ip->d, const_cast<int4*>(itab.tiles), const_cast<int4*>(itab.box), st));
    ERNN_CUDA(cudaMemsetAsync(at(tape, pl.t_A), 0, 2 * pl.state_bytes, st));  // A and B are adjacent
    if (with_tape) {
      const int nstore = pl.store_all ? p->nt : 2 * (pl.nseg - 1);
      ERNN_CUDA(launch_inst_ring_zero(fat(tape, pl.t_store), pl.state_bytes / sizeof(float), nstore, p->nx, p->ny,
                                      itab.box, p->nshots, st));
    }
    const size_t tr_bytes = (size_t)p->nshots * pl.nt_out * p->nrec * sizeof(float);
    ERNN_CUDA(cudaMemsetAsync(out_ux, 0, tr_bytes, st));
    ERNN_CUDA(cudaMemsetAsync(out_uy, 0, tr_bytes, st));
  }

  if (ip == nullptr && (p->path == ERNN_PATH_AUTO || p->path == ERNN_PATH_RESIDENT)) {
    ResCommon res;
    if (pick_resident(*p, *in, coef, res)) {
      g_last_path.store(ERNN_PATH_RESIDENT, std::memory_order_relaxed);
      return resident_forward(*p, pl, res, out_ux, out_uy, tape, with_tape, st);
    }
    if (p->path == ERNN_PATH_RESIDENT) return ERNN_ERR_UNSUPPORTED;
  }
  int tiled = 0;
  if (ip != nullptr) tiled = 1;
  else if ((rc = use_tiled(*p, &tiled))) return rc;
  g_last_path.store(tiled ? ERNN_PATH_TILED : ERNN_PATH_STEP, std::memory_order_relaxed);
  auto fwd_step = [&](const FwdStep& s) {
    return tiled ? launch_tma_fwd(p->mode, s, &coef->err, st) : launch_fwd_step(p->mode, s, st);
  };

  const bool store_all = with_tape && pl.store_all;
  float* A = fat(tape, pl.t_A);
  float* B = fat(tape, pl.t_B);
  auto stored = [&](int n) { return fat(tape, pl.t_store + (size_t)(n - 1) * pl.state_bytes); };
  auto ck = [&](int j, int lev) {  // checkpoint j >= 1: lev 0 = u^{jk}, lev 1 = u^{jk-1}
    return fat(tape, pl.t_store + ((size_t)(j - 1) * 2 + lev) * pl.state_bytes);
  };
  const bool receivers = (p->record == kRecordReceivers);
  FwdStep a = base_fwd(*p, *in, coef, pl.nt_out);
  a.inst = itab;
  a.tile_rows = tile_rows_of(*p);
  const float* last = nullptr;
  for (int i = 0; i < p->nt; ++i) {
    if (store_all) {
      a.out = stored(i + 1);
      a.cur = i >= 1 ? stored(i) : nullptr;
      a.prev = i >= 2 ? stored(i - 1) : nullptr;
    } else {
      a.out = (i % 2 == 0) ? A : B;
      a.cur = i == 0 ? nullptr : ((i % 2 == 0) ? B : A);
      a.prev = i <= 1 ? nullptr : a.out;
    }
    if (ip != nullptr) {
      // u^0 = 0: B (zeroed, first written at step 1) stands for it
      if (a.cur == nullptr) a.cur = B;
      a.inst.ntiles = ip->fwd_tiles(i);
    }
    a.i = i;
    a.copy0 = a.copy1 = nullptr;
    if (with_tape && !pl.store_all) {
      if ((i + 1) % pl.k == 0 && (i + 1) / pl.k <= pl.nseg - 1) a.copy0 = ck((i + 1) / pl.k, 0);
      if ((i + 2) % pl.k == 0 && (i + 2) / pl.k <= pl.nseg - 1) a.copy1 = ck((i + 2) / pl.k, 1);
    }
    a.frame = -1;
    a.gframe = -1;
    if (!receivers) {
      if (i % p->stride == 0) { a.frame = i / p->stride; a.hist_x = out_ux; a.hist_y = out_uy; }
    } else if (i >= 1 && (i - 1) % p->stride == 0) {
      a.gframe = (i - 1) / p->stride; a.tr_x = out_ux; a.tr_y = out_uy;
    }
    a.chained = i > 0;  // step 0 follows the coefficient kernel
    ERNN_CUDA(fwd_step(a));
    last = a.out;
  }
  if (receivers && (p->nt - 1) % p->stride == 0) {
    ERNN_CUDA(launch_gather(last, p->nx, p->ny, p->nshots, in->rec_idx, p->nrec,
                            (p->nt - 1) / p->stride, pl.nt_out, out_ux, out_uy, st, itab.box, p->nt));
  }
  return ERNN_OK;
}

int ernn_forward(const ErnnProblem* p, const ErnnInputs* in, float* out_ux, float* out_uy,
                 void* tape, size_t tape_bytes, int with_tape, void* stream) {
  return forward_impl(p, in, nullptr, out_ux, out_uy, tape, tape_bytes, with_tape, stream);
}

int ernn_forward_instances(const ErnnProblem* p, const ErnnInputs* in, const ErnnInstances* inst,
                           float* out_ux, float* out_uy, void* tape, size_t tape_bytes, int with_tape,
                           void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  InstPlan ip;
  if ((rc = plan_instances(*p, inst, &ip))) return rc;
  return forward_impl(p, in, &ip, out_ux, out_uy, tape, tape_bytes, with_tape, stream);
}

// The adjoint of ernn_adjoint and, with an instance plan `ip`, of
// ernn_adjoint_instances.
static int adjoint_impl(const ErnnProblem* p, const ErnnInputs* in, const InstPlan* ip, const float* g_ux,
                        const float* g_uy, const void* tape_c, size_t tape_bytes, void* scratch,
                        size_t scratch_bytes, double* grad_C, float* grad_field, void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  if ((rc = validate_inputs(p, in))) return rc;
  if ((ip != nullptr) != ((p->flags & ERNN_FLAG_INSTANCES) != 0)) return ERNN_ERR_INVALID;
  if (g_ux == nullptr || g_uy == nullptr || tape_c == nullptr || scratch == nullptr)
    return ERNN_ERR_INVALID;
  if (p->mode == kModeScalar && grad_C == nullptr) return ERNN_ERR_INVALID;
  if (p->mode != kModeScalar && grad_field == nullptr) return ERNN_ERR_INVALID;
  const Plan pl = make_plan(*p);
  if (tape_bytes < pl.t_total_tape || scratch_bytes < pl.s_total) return ERNN_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  void* tape = const_cast<void*>(tape_c);  // read only below

  Coef* coef = reinterpret_cast<Coef*>(at(scratch, pl.s_coef));
  ERNN_CUDA(launch_coef(p->mode, in->C, in->rho, p->h, p->dt, coef, st, pl.ncoef));
  const size_t gcount = (size_t)p->nshots * pl.nt_out *
                        (p->record == kRecordFields ? pl.N : (size_t)p->nrec);
  ERNN_CUDA(launch_gscale(g_ux, g_uy, gcount, coef, st, pl.ncoef));
  float* LA = fat(scratch, pl.s_LA);
  float* LB = fat(scratch, pl.s_LB);
  ERNN_CUDA(cudaMemsetAsync(LA, 0, 2 * pl.state_bytes, st));  // LA and LB are adjacent
  float* gacc = fat(scratch, pl.s_gacc);
  double* partials = reinterpret_cast<double*>(at(scratch, pl.s_part));
  if (p->mode != kModeScalar) ERNN_CUDA(cudaMemsetAsync(gacc, 0, pl.s_part - pl.s_gacc, st));
  else ERNN_CUDA(cudaMemsetAsync(partials, 0, pl.s_tflags - pl.s_part, st));

  InstTiles itab{nullptr, nullptr, 0};
  if (ip != nullptr) {
    // instances: the tiled kernels over the tile table only; the zero state
    // starts at zero, the recompute segment's states need only the
    // instances' ghost rings zeroed (as the stored states of the forward)
    if (p->path != ERNN_PATH_AUTO && p->path != ERNN_PATH_TILED) return ERNN_ERR_UNSUPPORTED;
    if (!tma_eligible(p->mode, p->nx, p->ny, 1)) return ERNN_ERR_UNSUPPORTED;
    itab.tiles = reinterpret_cast<int4*>(at(scratch, pl.s_inst));
    itab.box = reinterpret_cast<int4*>(at(scratch, pl.s_inst + align_up(inst_table_bound(p->nx, p->ny, p->nshots) *
                                                                          sizeof(int4))));
    ERNN_CUDA(launch_inst_table(ip->d, const_cast<int4*>(itab.tiles), const_cast<int4*>(itab.box), st));
    ERNN_CUDA(cudaMemsetAsync(at(scratch, pl.s_zero), 0, pl.state_bytes, st));
    if (!pl.store_all)
      ERNN_CUDA(launch_inst_ring_zero(fat(scratch, pl.s_seg), pl.state_bytes / sizeof(float), pl.k, p->nx, p->ny,
                                      itab.box, p->nshots, st));
  }

  if (ip == nullptr && (p->path == ERNN_PATH_AUTO || p->path == ERNN_PATH_RESIDENT)) {
    ResCommon res;
    if (pick_resident(*p, *in, coef, res)) {
      g_last_path.store(ERNN_PATH_RESIDENT, std::memory_order_relaxed);
      int img_rows = 0;
      if ((rc = resident_adjoint(*p, pl, res, g_ux, g_uy, tape, scratch, partials, &img_rows, st)))
        return rc;
      // imaging rows are grouped by shot
      if (pl.ncoef > 1) ERNN_CUDA(launch_finalize_scalar(partials, img_rows / p->nshots, coef, grad_C, st,
                                                         p->nshots, 1));
      else ERNN_CUDA(launch_finalize_scalar(partials, img_rows, coef, grad_C, st));
      return ERNN_OK;
    }
    if (p->path == ERNN_PATH_RESIDENT) return ERNN_ERR_UNSUPPORTED;
  }
  int tiled = 0;
  if (ip != nullptr) tiled = 1;
  else if ((rc = use_tiled(*p, &tiled))) return rc;
  g_last_path.store(tiled ? ERNN_PATH_TILED : ERNN_PATH_STEP, std::memory_order_relaxed);

  auto stored = [&](int n) { return fat(tape, pl.t_store + (size_t)(n - 1) * pl.state_bytes); };
  const float* zero_state = ip != nullptr ? fat(scratch, pl.s_zero) : nullptr;
  auto ck = [&](int j, int lev) -> const float* {
    if (j == 0) return lev == 0 ? zero_state : nullptr;  // u^0 = 0 (given as a state with instances)
    if (lev == 1 && j * pl.k - 1 == 0) return nullptr;  // u^0 = 0 (k == 1)
    return fat(tape, pl.t_store + ((size_t)(j - 1) * 2 + lev) * pl.state_bytes);
  };
  auto seg = [&](int slot) { return fat(scratch, pl.s_seg + (size_t)slot * pl.state_bytes); };

  AdjStep b;
  std::memset(&b, 0, sizeof(b));
  b.nx = p->nx; b.ny = p->ny; b.S = p->nshots;
  b.coef = coef;
  b.field = (p->mode == kModeFields) ? in->C : in->D;
  b.g_x = g_ux; b.g_y = g_uy;
  b.nt_out = pl.nt_out; b.record = p->record; b.nrec = p->nrec; b.rec_idx = in->rec_idx;
  b.coef_stride = pl.ncoef > 1 ? 1 : 0;
  b.partials = partials;
  b.gacc = gacc;
  b.tile_flags = nullptr;
  b.inst = itab;
  b.tile_rows = tile_rows_of(*p);
  if (tiled && p->record == kRecordReceivers) {
    uint8_t* flags = reinterpret_cast<uint8_t*>(at(scratch, pl.s_tflags));
    if (ip != nullptr)
      ERNN_CUDA(launch_inst_tile_flags(in->rec_idx, p->nshots, p->nrec, p->ny, itab.box, flags,
                                       ip->upto[ip->d.count], st));
    else
      ERNN_CUDA(launch_tile_flags(p->mode, in->rec_idx, p->nshots, p->nrec, p->nx, p->ny, flags, st,
                                  b.tile_rows));
    b.tile_flags = flags;
  }

  // per-shot gradients need one row layout for the whole call: the tiled
  // kernel only if every step takes it (same buffers every step)
  if (tiled && pl.ncoef > 1) {
    AdjStep probe = b;
    probe.out = LA; probe.cur = LB; probe.prev = LA;
    probe.u = pl.store_all ? stored(1) : seg(0);
    if (!tma_adj_would_run(p->mode, probe)) {
      tiled = 0;
      g_last_path.store(ERNN_PATH_STEP, std::memory_order_relaxed);
    }
  }
  const bool tiled_adj = tiled != 0;
  // every step launch after the first of the loop below follows a step kernel
  bool chained = false;
  auto adj_step = [&](int m, const float* um) -> int {
    const int idx = p->nt - m;
    b.m = m;
    if (ip != nullptr) b.inst.ntiles = ip->adj_tiles(m);
    b.out = (idx % 2 == 0) ? LA : LB;
    b.cur = (idx % 2 == 0) ? LB : LA;
    b.prev = b.out;
    b.u = (m <= p->nt - 1) ? um : nullptr;
    b.frame = ((m - 1) % p->stride == 0) ? (m - 1) / p->stride : -1;
    b.chained = chained ? 1 : 0;
    chained = true;
    const cudaError_t e = tiled ? launch_tma_adj(p->mode, b, &coef->err, st) : launch_adj_step(p->mode, b, st);
    return e == cudaSuccess ? ERNN_OK : ERNN_ERR_CUDA;
  };

  if (pl.store_all) {
    for (int m = p->nt; m >= 1; --m)
      if ((rc = adj_step(m, stored(m)))) return rc;
  } else {
    FwdStep a = base_fwd(*p, *in, coef, pl.nt_out);
    a.inst = itab;
    a.tile_rows = b.tile_rows;
    for (int j = pl.nseg - 1; j >= 0; --j) {
      const int i0 = j * pl.k, i1 = (j + 1) * pl.k < p->nt ? (j + 1) * pl.k : p->nt;
      // recompute u^{i0+1} .. u^{i1} into the segment buffer; u^{nt} is never
      // imaged, so the last segment stops one step short
      const int iend = i1 < p->nt ? i1 : p->nt - 1;
      // on the tiled path, pairs of steps go through the two-step kernel
      for (int i = i0; i < iend;) {
        a.i = i;
        a.out = seg(i - i0);
        a.cur = (i == i0) ? ck(j, 0) : seg(i - i0 - 1);
        a.prev = (i == i0) ? ck(j, 1) : (i == i0 + 1 ? ck(j, 0) : seg(i - i0 - 2));
        a.chained = chained ? 1 : 0;
        chained = true;
        if (ip != nullptr) a.inst.ntiles = ip->fwd_tiles(i);
        // (a pair of steps takes the tiles of the first step: an instance
        // ending after step i runs both of them, one ending at i + 1 takes
        // the pair only when it has step i + 1)
        a.out2 = (tiled && i + 1 < iend && (ip == nullptr || ip->fwd_tiles(i + 1) == a.inst.ntiles))
                     ? seg(i + 1 - i0)
                     : nullptr;
        if (a.out2 != nullptr && tma_fwd2_would_run(p->mode, a)) {
          ERNN_CUDA(launch_tma_fwd2(p->mode, a, &coef->err, st));
          i += 2;
          continue;
        }
        a.out2 = nullptr;
        ERNN_CUDA(tiled ? launch_tma_fwd(p->mode, a, &coef->err, st) : launch_fwd_step(p->mode, a, st));
        ++i;
      }
      for (int m = i1; m >= i0 + 1; --m)
        if ((rc = adj_step(m, seg(m - 1 - i0)))) return rc;
    }
  }
  if (p->mode == kModeScalar && pl.ncoef > 1) {
    // per-shot gradients: the tiled kernel keeps kTiledRowsPerShot rows per
    // shot, the plain kernel one row per block (blocks of a shot contiguous)
    const int rows = tiled_adj ? kTiledRowsPerShot : pl.nblocks / p->nshots;
    ERNN_CUDA(launch_finalize_scalar(partials, rows, coef, grad_C, st, p->nshots, 1));
  } else if (p->mode == kModeScalar) {
    ERNN_CUDA(launch_finalize_scalar(partials, pl.nblocks, coef, grad_C, st));
  } else {
    ERNN_CUDA(launch_finalize_fields(p->mode, gacc, p->nshots, (int)pl.N, coef, grad_field, st));
  }
  return ERNN_OK;
}

int ernn_adjoint(const ErnnProblem* p, const ErnnInputs* in, const float* g_ux,
                 const float* g_uy, const void* tape_c, size_t tape_bytes, void* scratch,
                 size_t scratch_bytes, double* grad_C, float* grad_field, void* stream) {
  return adjoint_impl(p, in, nullptr, g_ux, g_uy, tape_c, tape_bytes, scratch, scratch_bytes, grad_C,
                      grad_field, stream);
}

int ernn_adjoint_instances(const ErnnProblem* p, const ErnnInputs* in, const ErnnInstances* inst,
                           const float* g_ux, const float* g_uy, const void* tape, size_t tape_bytes,
                           void* scratch, size_t scratch_bytes, double* grad_C, void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  InstPlan ip;
  if ((rc = plan_instances(*p, inst, &ip))) return rc;
  return adjoint_impl(p, in, &ip, g_ux, g_uy, tape, tape_bytes, scratch, scratch_bytes, grad_C, nullptr,
                      stream);
}

uint64_t ernn_launch_count(void) { return launches(); }

int ernn_device_status(const ErnnProblem* p, const void* workspace, int is_scratch,
                       int32_t* status_host, void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  if (workspace == nullptr || status_host == nullptr || (is_scratch != 0 && is_scratch != 1))
    return ERNN_ERR_INVALID;
  const Plan pl = make_plan(*p);
  const char* w = static_cast<const char*>(workspace) + (is_scratch ? pl.s_coef : pl.t_coef) +
                  offsetof(Coef, err);
  ERNN_CUDA(cudaMemcpyAsync(status_host, w, sizeof(int32_t), cudaMemcpyDeviceToHost,
                            (cudaStream_t)stream));
  return ERNN_OK;
}

int ernn_wait_selftest(int32_t* status_host, void* stream) {
  if (status_host == nullptr) return ERNN_ERR_INVALID;
  int v = -1;
  ERNN_CUDA(wait_selftest(&v, (cudaStream_t)stream));
  *status_host = v;
  return ERNN_OK;
}

int32_t ernn_last_path(void) { return g_last_path.load(std::memory_order_relaxed); }

int ernn_set_launch_overlap(int on) {
  const int was = launch_overlap_setting() ? 1 : 0;
  set_launch_overlap(on != 0);
  return was;
}

int ernn_profile_enable(int enable) {
  profile_enable(enable != 0);
  return ERNN_OK;
}

int ernn_profile_read(double* ms3, uint64_t* launches3, double* alg_bytes3) {
  if (ms3 == nullptr || launches3 == nullptr) return ERNN_ERR_INVALID;
  return profile_read(ms3, launches3, alg_bytes3) == cudaSuccess ? ERNN_OK : ERNN_ERR_CUDA;
}

}  // extern "C"
