// Host/device interface of the cluster-resident time loop (ernn_resident.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "ernn_common.cuh"

namespace ernn {

constexpr int kResThreads = 256;  // threads per CTA (each owns 4 x 4-cell items)
constexpr int kResMaxRec = 1024;  // receivers one CTA can own

struct ResCommon {
  int nx, ny, S, nt, stride, nt_out;
  int R, CL;              // rows per CTA, CTAs per cluster (one cluster per shot and role)
  const Coef* coef;
  const float* src_signal;
  const float* src_map;
  const int32_t* src_origin;
  int bx, by, src_comp;
  const int32_t* rec_idx;
  int nrec;
  int* err;               // device error word (ERNN_ERR_TIMEOUT on a timed-out wait)
};

// Forward role: steps i0 .. i1-1 from (u^{i0}, u^{i0-1}).
struct ResFwd {
  int i0, i1;
  const float* init_cur;   // u^{i0}  [S][2][N] or nullptr (zero)
  const float* init_prev;  // u^{i0-1} or nullptr
  float* states;           // u^{i+1} -> states + (i - i0) * state_stride, or nullptr
  size_t state_stride;     // floats between consecutive stored states
  float* ckpt;             // checkpoint pairs (segmented forward pass) or nullptr
  int ck_k, ck_nseg;
  float* hist_x;           // dense history (S, nt_out, N) or nullptr
  float* hist_y;
  float* tr_x;             // receiver traces (S, nt_out, nrec) or nullptr
  float* tr_y;
};

// Adjoint role: m = m_hi down to m_lo + 1, imaging against u^m.
struct ResAdj {
  int m_hi, m_lo;
  const float* u_states;   // u^m at u_states + (m - u_base) * state_stride
  int u_base;
  size_t state_stride;
  float* lam_save;         // level 0: lam^{m+1}, level 1: lam^{m+2} (in and out)
  size_t save_stride;      // floats between the two levels
  int first;               // 1: start from lam = 0
  const float* g_x;
  const float* g_y;
  double* partials;        // [S][CL][8]
};

size_t resident_smem_bytes(const ResCommon& c, bool with_adjoint);
bool resident_feasible(const ResCommon& c, bool dense);
cudaError_t launch_resident(const ResCommon& c, const ResFwd& f, const ResAdj& a, bool run_fwd,
                            bool run_adj, bool dense, cudaStream_t st);

}  // namespace ernn
