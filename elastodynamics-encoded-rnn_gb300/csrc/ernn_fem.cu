// FEM data generator step (sm_103a): the explicit time loop that produces
// the reference's training wavefields (Parameter_inversion/FEM_generate_data.py:
// mesh :117-185, lumped mass :330-342, element operator :345-457, central
// differences with fixed edges :474-499, 0.7-scaled frames :525-526, 901-930).
//
// The mesh is the structured triangular one of the generator: nodes on an
// nx x ny grid, each cell split along the diagonal n0-n2 when (ci + cj) is
// even and along n1-n3 when odd.  Its elements therefore come in four shapes
// with constant strain (one B matrix per shape), and every interior node
// sees the same 8 (node parity even) or 4 (odd) triangles.  Instead of
// gathering elements and scattering forces with atomics, one thread per node
// gathers the strains of its adjacent triangles from the 3 x 3 neighbourhood
// of displacements, forms their stresses and sums the node's share of each
// element force: one pass per step reading u^n (neighbourhood), u^{n-1}, the
// load, writing u^{n+1} and, on recording steps, the scaled frame.
// Edge nodes are fixed at zero (their forces are never needed).
//
// State layout: [i][j] with j (y) fastest, the layout of the saved frames
// (nt_out, nx, ny); node (i, j) is the generator's node j*nx + i.
#include <cmath>
#include <cstring>

#include "ernn.h"
#include "ernn_launch.h"

namespace ernn {
namespace {

// Element shapes: 0 = even cell [n0, n1, n2], 1 = even [n0, n2, n3],
// 2 = odd [n0, n1, n3], 3 = odd [n1, n2, n3]; corners n0 = (0, 0),
// n1 = (1, 0), n2 = (1, 1), n3 = (0, 1) in (i, j) offsets within the cell.
struct FemConsts {
  float bx[4][3], by[4][3];  // dN/dx, dN/dy of the three nodes of each shape
  float fh;                  // |det J| x (3 Gauss points x weight 1/6)
  float C11, C22, C12, C16, C26, C66;
  float m_even, m_odd;       // lumped mass of interior nodes (8 or 4 triangles)
  float dt2, rho_inv, scale;
};

struct FemStep {
  int nx, ny, n;
  const float* cur_x; const float* cur_y;
  const float* prev_x; const float* prev_y;
  float* out_x; float* out_y;
  const float* load;    // (nx, ny)
  const float* signal;  // (nt)
  const float* cf;      // per-node constants, 6 planes (nx, ny), or nullptr
  float* frame_x;       // (nx, ny) slice of the frames, or nullptr
  float* frame_y;
};

// Contribution of one triangle of shape T, in the cell whose corner (0, 0)
// sits at offset (oi, oj) from the node, to the node's force; the node is
// the triangle's vertex `a`.  u[1 + di][1 + dj] is the neighbourhood.
// FIELDS: the element's constants are those of the grid node nearest its
// centroid (Damage_inversion/FEM_generate_data.py:1002-1017): centroids sit
// at (2/3, 1/3), (1/3, 2/3), (1/3, 1/3), (2/3, 2/3) of the cell for shapes
// 0..3, so that node is the cell corner (1, 0), (0, 1), (0, 0), (1, 1).
template <bool FIELDS, int T, int OI, int OJ, int A>
__device__ __forceinline__ void tri(const FemConsts& k, const FemStep& s, size_t o,
                                    const float ux[3][3], const float uy[3][3], float& fx, float& fy) {
  constexpr int vi[4][3] = {{0, 1, 1}, {0, 1, 0}, {0, 1, 0}, {1, 1, 0}};
  constexpr int vj[4][3] = {{0, 0, 1}, {0, 1, 1}, {0, 0, 1}, {0, 1, 1}};
  constexpr int ci[4] = {1, 0, 0, 1}, cj[4] = {0, 1, 0, 1};
  float C11 = k.C11, C22 = k.C22, C12 = k.C12, C16 = k.C16, C26 = k.C26, C66 = k.C66;
  if (FIELDS) {
    const size_t N = (size_t)s.nx * s.ny;
    const size_t e = o + (size_t)((OI + ci[T]) * s.ny + (OJ + cj[T]));
    C11 = __ldg(s.cf + e);
    C22 = __ldg(s.cf + N + e);
    C12 = __ldg(s.cf + 2 * N + e);
    C16 = __ldg(s.cf + 3 * N + e);
    C26 = __ldg(s.cf + 4 * N + e);
    C66 = __ldg(s.cf + 5 * N + e);
  }
  float exx = 0.f, eyy = 0.f, gxy = 0.f;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const float vx = ux[1 + OI + vi[T][b]][1 + OJ + vj[T][b]];
    const float vy = uy[1 + OI + vi[T][b]][1 + OJ + vj[T][b]];
    exx += k.bx[T][b] * vx;
    eyy += k.by[T][b] * vy;
    gxy += k.by[T][b] * vx + k.bx[T][b] * vy;
  }
  const float sxx = C11 * exx + C12 * eyy + C16 * gxy;
  const float syy = C12 * exx + C22 * eyy + C26 * gxy;
  const float txy = C16 * exx + C26 * eyy + C66 * gxy;
  fx += k.fh * (k.bx[T][A] * sxx + k.by[T][A] * txy);
  fy += k.fh * (k.by[T][A] * syy + k.bx[T][A] * txy);
}

template <bool FIELDS>
__global__ void __launch_bounds__(256) fem_step_kernel(const FemStep s, const FemConsts k) {
  grid_dep_trigger();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= s.nx || j >= s.ny) return;
  const int ny = s.ny;
  const size_t o = (size_t)i * ny + j;
  const bool interior = i > 0 && i < s.nx - 1 && j > 0 && j < ny - 1;
  // the load term needs no state: formed before the wait
  const float lf = interior ? s.signal[s.n] * s.load[o] * k.rho_inv : 0.f;
  grid_dep_wait();  // levels of the previous launch complete from here on
  float vx = 0.f, vy = 0.f;
  if (interior) {
    float ux[3][3], uy[3][3];
#pragma unroll
    for (int di = 0; di < 3; ++di)
#pragma unroll
      for (int dj = 0; dj < 3; ++dj) {
        const size_t q = o + (size_t)(di - 1) * ny + (dj - 1);
        ux[di][dj] = s.cur_x[q];
        uy[di][dj] = s.cur_y[q];
      }
    float fx = 0.f, fy = 0.f;
    float m;
    // cells around the node: A = (i-1, j-1) (node is its n2), B = (i, j-1)
    // (n3), C = (i-1, j) (n1), D = (i, j) (n0); A and D have the node's
    // parity, B and C the other
    if (((i + j) & 1) == 0) {
      tri<FIELDS, 0, -1, -1, 2>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 1, -1, -1, 1>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 2, 0, -1, 2>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 3, 0, -1, 2>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 2, -1, 0, 1>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 3, -1, 0, 0>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 0, 0, 0, 0>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 1, 0, 0, 0>(k, s, o, ux, uy, fx, fy);
      m = k.m_even;
    } else {
      tri<FIELDS, 3, -1, -1, 1>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 1, 0, -1, 2>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 0, -1, 0, 1>(k, s, o, ux, uy, fx, fy);
      tri<FIELDS, 2, 0, 0, 0>(k, s, o, ux, uy, fx, fy);
      m = k.m_odd;
    }
    const float fext = lf * m;
    vx = 2.f * ux[1][1] - s.prev_x[o] - k.dt2 * fx / m;
    vy = 2.f * uy[1][1] - s.prev_y[o] + k.dt2 * (fext - fy) / m;
  }
  s.out_x[o] = vx;
  s.out_y[o] = vy;
  if (s.frame_x != nullptr) {
    s.frame_x[o] = k.scale * vx;
    s.frame_y[o] = k.scale * vy;
  }
}

FemConsts fem_consts(const ErnnFemProblem& p) {
  FemConsts k;
  std::memset(&k, 0, sizeof(k));
  // corner coordinates of the four shapes (units of dx, dy)
  const int vi[4][3] = {{0, 1, 1}, {0, 1, 0}, {0, 1, 0}, {1, 1, 0}};
  const int vj[4][3] = {{0, 0, 1}, {0, 1, 1}, {0, 0, 1}, {0, 1, 1}};
  const double dxi[3] = {-1.0, 1.0, 0.0}, deta[3] = {-1.0, 0.0, 1.0};
  double det = 0.0;
  for (int t = 0; t < 4; ++t) {
    const double J00 = (vi[t][1] - vi[t][0]) * p.dx, J01 = (vi[t][2] - vi[t][0]) * p.dx;
    const double J10 = (vj[t][1] - vj[t][0]) * p.dy, J11 = (vj[t][2] - vj[t][0]) * p.dy;
    det = J00 * J11 - J01 * J10;
    // J^-1, rounded to float as the generator moves it to float32
    const float i00 = (float)(J11 / det), i01 = (float)(-J01 / det);
    const float i10 = (float)(-J10 / det), i11 = (float)(J00 / det);
    for (int a = 0; a < 3; ++a) {
      k.bx[t][a] = i00 * (float)dxi[a] + i10 * (float)deta[a];
      k.by[t][a] = i01 * (float)dxi[a] + i11 * (float)deta[a];
    }
  }
  // every shape has |det J| = dx dy; three Gauss points of weight 1/6
  const float w = (float)(1.0 / 6.0);
  const float f1 = (float)std::fabs(det) * w;
  k.fh = f1 + f1 + f1;
  k.C11 = (float)p.C[0]; k.C22 = (float)p.C[1]; k.C12 = (float)p.C[2];
  k.C16 = (float)p.C[3]; k.C26 = (float)p.C[4]; k.C66 = (float)p.C[5];
  // lumped mass: rho * (dx dy / 2) / 3 added once per adjacent triangle, in float
  const float mnode = (float)(p.rho * (p.dx * p.dy / 2.0) / 3.0);
  float m = 0.f;
  for (int c = 0; c < 8; ++c) {
    m += mnode;
    if (c == 3) k.m_odd = m;
  }
  k.m_even = m;
  k.dt2 = (float)(p.dt * p.dt);
  k.rho_inv = (float)(1.0 / p.rho);
  k.scale = (float)p.out_scale;
  return k;
}

constexpr size_t kFemAlign = 256;
inline size_t fem_align(size_t v) { return (v + kFemAlign - 1) / kFemAlign * kFemAlign; }

}  // namespace
}  // namespace ernn

using namespace ernn;

extern "C" size_t ernn_fem_workspace_bytes(const ErnnFemProblem* p) {
  if (p == nullptr || p->nx < 2 || p->ny < 2) return 0;
  return 6 * fem_align((size_t)p->nx * p->ny * sizeof(float));
}

extern "C" int ernn_fem_forward(const ErnnFemProblem* p, const float* load, const float* signal,
                                const float* C_fields, float* frames_x, float* frames_y,
                                void* workspace, size_t workspace_bytes, void* stream) {
  // (the per-level launch takes 8 node rows per block along grid y: at most 65535 blocks)
  if (p == nullptr || p->nx < 2 || p->ny < 2 || p->nt < 1 || p->stride < 1 ||
      (int64_t)p->nx * p->ny >= ((int64_t)1 << 31) || (p->nx + 7) / 8 > 65535)
    return ERNN_ERR_INVALID;
  if (!(p->dx > 0.0) || !(p->dy > 0.0) || !(p->dt > 0.0) || !(p->rho > 0.0) ||
      !std::isfinite(p->dx) || !std::isfinite(p->dy) || !std::isfinite(p->dt) ||
      !std::isfinite(p->out_scale))
    return ERNN_ERR_INVALID;
  if (load == nullptr || signal == nullptr || frames_x == nullptr || frames_y == nullptr ||
      workspace == nullptr)
    return ERNN_ERR_INVALID;
  if (workspace_bytes < ernn_fem_workspace_bytes(p)) return ERNN_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t N = (size_t)p->nx * p->ny;
  const size_t lev = fem_align(N * sizeof(float));
  char* w = static_cast<char*>(workspace);
  float* ux[3];
  float* uy[3];
  for (int l = 0; l < 3; ++l) {
    ux[l] = reinterpret_cast<float*>(w + (2 * l) * lev);
    uy[l] = reinterpret_cast<float*>(w + (2 * l + 1) * lev);
  }
  // levels 0 and 1 are zero (slot n % 3 holds u^n)
  if (cudaMemsetAsync(w, 0, 4 * lev, st) != cudaSuccess) return ERNN_ERR_CUDA;
  const int nt_out = (p->nt + p->stride - 1) / p->stride;
  // frames of the levels that are never computed (0, and 1 when stride is 1)
  for (int f = 0; f < nt_out && f * p->stride <= 1; ++f) {
    if (cudaMemsetAsync(frames_x + (size_t)f * N, 0, N * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(frames_y + (size_t)f * N, 0, N * sizeof(float), st) != cudaSuccess)
      return ERNN_ERR_CUDA;
  }
  const FemConsts k = fem_consts(*p);
  const dim3 block(32, 8, 1);
  const dim3 grid((p->ny + 31) / 32, (p->nx + 7) / 8, 1);
  FemStep s;
  std::memset(&s, 0, sizeof(s));
  s.nx = p->nx; s.ny = p->ny;
  s.load = load;
  s.signal = signal;
  s.cf = C_fields;
  for (int n = 1; n < p->nt - 1; ++n) {
    s.n = n;
    s.cur_x = ux[n % 3]; s.cur_y = uy[n % 3];
    s.prev_x = ux[(n + 2) % 3]; s.prev_y = uy[(n + 2) % 3];
    s.out_x = ux[(n + 1) % 3]; s.out_y = uy[(n + 1) % 3];
    if ((n + 1) % p->stride == 0) {
      const size_t f = (size_t)((n + 1) / p->stride) * N;
      s.frame_x = frames_x + f;
      s.frame_y = frames_y + f;
    } else {
      s.frame_x = s.frame_y = nullptr;
    }
    const bool chained = n > 1;  // the previous launch is the previous level's
    const cudaError_t e = tracked_launch(kProfForward, st, [&] {
      if (C_fields != nullptr) launch_step_kernel(fem_step_kernel<true>, grid, block, 0, st, chained, s, k);
      else launch_step_kernel(fem_step_kernel<false>, grid, block, 0, st, chained, s, k);
    }, (double)N * (C_fields != nullptr ? 52.0 : 28.0));
    if (e != cudaSuccess) return ERNN_ERR_CUDA;
  }
  return ERNN_OK;
}
