// Allocation-free forward entry point (ernn_forward_static in include/ernn.h).
//
// Some callers of this library cannot call cudaMalloc (or any allocating
// routine) around a propagation: code that runs while another framework is
// capturing a CUDA graph on the stream, real-time loops in which the implicit
// device synchronisation of cudaMalloc/cudaFree is not acceptable, and thin
// FFI hosts that carry no device allocator of their own.  They still pass
// their inputs and outputs, but the two-level wavefield and the coefficient
// block that ernn_forward keeps in the caller's tape live here in a
// file-scope device array instead.
//
// The array is kStaticScratchBytes (8 MiB) on every GPU that loads the
// library and is held until the process exits.  All calls share it: calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.  Every word a
// call reads is written earlier in the same call (the coefficient block by
// the first kernel, each state level by the step that produces it), so
// nothing needs clearing between calls.
#include <cstring>
#include <mutex>

#include "ernn.h"
#include "ernn_launch.h"

namespace ernn {
namespace {

constexpr size_t kStaticScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// In host code g_static_scratch names a host-side stand-in, not device
// memory: the device address comes from cudaGetSymbolAddress, once per device
// with that device current, cached here.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return ERNN_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return ERNN_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || p == nullptr)
      return ERNN_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return ERNN_OK;
}

constexpr size_t kAlignStatic = 256;
inline size_t align_static(size_t v) { return (v + kAlignStatic - 1) / kAlignStatic * kAlignStatic; }

}  // namespace
}  // namespace ernn

using namespace ernn;

extern "C" int ernn_forward_static(const ErnnProblem* p, const ErnnInputs* in, float* out_ux,
                                   float* out_uy, void* stream) {
  int rc = ernn_validate(p);
  if (rc != ERNN_OK) return rc;
  if (in == nullptr || in->C == nullptr || in->rho == nullptr || in->src_signal == nullptr ||
      out_ux == nullptr || out_uy == nullptr)
    return ERNN_ERR_INVALID;
  if (p->mode == kModeDField && in->D == nullptr) return ERNN_ERR_INVALID;
  if ((size_t)p->src_bx * p->src_by > 0 && (in->src_map == nullptr || in->src_origin == nullptr))
    return ERNN_ERR_INVALID;
  if (p->record == kRecordReceivers && in->rec_idx == nullptr) return ERNN_ERR_INVALID;
  // the per-step kernels are the only ones this entry runs: an explicit
  // request for the resident or tiled kernels cannot be served
  if (p->path != ERNN_PATH_AUTO && p->path != ERNN_PATH_STEP) return ERNN_ERR_UNSUPPORTED;
  // coefficient block(s), then two state levels of nshots x 2 x nx x ny floats
  const size_t N = (size_t)p->nx * p->ny;
  const size_t state_bytes = align_static((size_t)p->nshots * 2 * N * sizeof(float));
  const int ncoef = (p->flags & ERNN_FLAG_SHOT_CONSTANTS) ? p->nshots : 1;
  const size_t coef_bytes = align_static((size_t)ncoef * sizeof(Coef));
  if (coef_bytes + 2 * state_bytes > kStaticScratchBytes) return ERNN_ERR_WORKSPACE;

  void* base = nullptr;
  if ((rc = scratch_for_current_device(&base)) != ERNN_OK) return rc;
  char* b = static_cast<char*>(base);
  Coef* coef = reinterpret_cast<Coef*>(b);
  float* A = reinterpret_cast<float*>(b + coef_bytes);
  float* B = reinterpret_cast<float*>(b + coef_bytes + state_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  record_last_path(ERNN_PATH_STEP);
  if (launch_coef(p->mode, in->C, in->rho, p->h, p->dt, coef, st, ncoef) != cudaSuccess) return ERNN_ERR_CUDA;

  const int nt_out = (p->nt + p->stride - 1) / p->stride;
  const bool receivers = (p->record == kRecordReceivers);
  FwdStep a;
  std::memset(&a, 0, sizeof(a));
  a.nx = p->nx; a.ny = p->ny; a.S = p->nshots; a.nt = p->nt;
  a.nt_out = nt_out;
  a.coef = coef;
  a.coef_stride = ncoef > 1 ? 1 : 0;
  a.field = (p->mode == kModeFields) ? in->C : in->D;
  a.src_signal = in->src_signal;
  a.src_map = in->src_map;
  a.src_origin = in->src_origin;
  a.bx = p->src_bx; a.by = p->src_by; a.src_comp = p->src_comp;
  a.rec_idx = in->rec_idx;
  a.nrec = p->nrec;
  const float* last = nullptr;
  for (int i = 0; i < p->nt; ++i) {
    // u^{i+1} overwrites u^{i-1}: A holds even steps' outputs, B odd ones
    a.out = (i % 2 == 0) ? A : B;
    a.cur = i == 0 ? nullptr : ((i % 2 == 0) ? B : A);
    a.prev = i <= 1 ? nullptr : a.out;
    a.i = i;
    a.frame = -1;
    a.gframe = -1;
    if (!receivers) {
      if (i % p->stride == 0) { a.frame = i / p->stride; a.hist_x = out_ux; a.hist_y = out_uy; }
    } else if (i >= 1 && (i - 1) % p->stride == 0) {
      a.gframe = (i - 1) / p->stride; a.tr_x = out_ux; a.tr_y = out_uy;
    }
    a.chained = i > 0;  // step 0 follows the coefficient kernel
    if (launch_fwd_step(p->mode, a, st) != cudaSuccess) return ERNN_ERR_CUDA;
    last = a.out;
  }
  if (receivers && (p->nt - 1) % p->stride == 0) {
    if (launch_gather(last, p->nx, p->ny, p->nshots, in->rec_idx, p->nrec, (p->nt - 1) / p->stride,
                      nt_out, out_ux, out_uy, st) != cudaSuccess)
      return ERNN_ERR_CUDA;
  }
  return ERNN_OK;
}
