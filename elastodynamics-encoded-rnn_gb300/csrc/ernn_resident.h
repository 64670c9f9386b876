// Host/device interface of the cluster-resident time loop (ernn_resident.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "ernn_common.cuh"

namespace ernn {

constexpr int kResThreads = 256;  // threads per CTA (each owns 4 x 4-cell items; 512 measured slower)
constexpr int kResMaxRec = 1024;  // receivers one CTA can own

struct ResCommon {
  int nx, ny, S, nt, stride, nt_out;
  int R, CL;              // rows per CTA, CTAs per cluster (one cluster per shot and role)
  const Coef* coef;
  int coef_stride;        // 0: one coefficient block; 1: one per shot (coef + shot)
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

// LAM role: m = m_hi down to m_lo + 1 of the adjoint recursion.
struct ResLam {
  int m_hi, m_lo;
  float* lam_save;         // level 0: lam^{m+1}, level 1: lam^{m+2} (in and out)
  size_t save_stride;      // floats between the two levels
  int first;               // 1: start from lam = 0
  const float* g_x;
  const float* g_y;
  float* lbuf;             // lam^m -> lbuf + (m - slot_base) * state_stride (slots >= 0), or nullptr
  int slot_base;
  int store_init;          // also store lam^{m_hi+1} into slot m_hi + 1 - slot_base
  size_t state_stride;
};

// IMG role: imaging pairs (lam^{n+1}, u^n) for n = n_lo .. n_hi, slot n - n_lo.
struct ResImg {
  int n_lo, n_hi;
  const float* lbuf;
  const float* ubuf;
  size_t state_stride;
  double* partials;        // [shot][IMG CTAs of the shot][8]
};

// blockIdx.z of each role (-1: absent); IMG occupies n_img_z planes from z_img.
struct ResRoles {
  int z_fwd, z_lam, z_img, n_img_z;
};

size_t resident_smem_bytes(const ResCommon& c);
// Whether any cluster size can hold a shot of this grid (the adjoint scratch
// reserves the path's lam buffers only then).
bool resident_possible(int mode, int nx, int ny);
bool resident_feasible(const ResCommon& c, bool dense);
// IMG clusters along z for one launch (total IMG CTAs = this x S x CL)
int resident_img_clusters(const ResCommon& c);
cudaError_t launch_resident(const ResCommon& c, const ResFwd& f, const ResLam& a, const ResImg& g,
                            bool run_fwd, bool run_lam, bool run_img, bool dense, cudaStream_t st);

}  // namespace ernn
