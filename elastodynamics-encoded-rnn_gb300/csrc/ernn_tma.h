// Tiled per-step kernels (ernn_tma.cu): one launch per time step, persistent
// CTAs streaming 64-column tiles through TMA loads.  Internal to the library.
#pragma once

#include "ernn_launch.h"

namespace ernn {

// Scalar constants or a degradation map, ny % 4 == 0 (rows of 16-byte
// multiples for the copy engine), and the driver exposes the tensor-map
// encoder.
bool tma_eligible(int mode, int nx, int ny, int S);
// Partial-sum rows reserved per shot by the tiled adjoint with per-shot
// constants (its grid never exceeds this many CTAs).
constexpr int kTiledRowsPerShot = 1024;
// Number of 64-column tiles of `tile_rows` rows of one step over all shots.
size_t tma_tiles(int nx, int ny, int S, int tile_rows = 32);
// Tile rows of the tiled adjoint for a mode: SCALAR 16, or 32 when
// tile_rows == 32 (ERNN_FLAG_TALL_TILES); DFIELD 32.
int tma_adj_tile_rows(int mode, int tile_rows = 0);
// Same contract as launch_fwd_step / launch_adj_step (SCALAR or DFIELD
// mode); `err` is the call's device error word.
cudaError_t launch_tma_fwd(int mode, const FwdStep& a, int* err, cudaStream_t st);
// Two steps in one launch (u^{i+1} into a.out, u^{i+2} into a.out2) when
// tma_fwd2_would_run: scalar constants, u^i given, no frames, copies or
// receiver gathers in either step; cudaErrorNotSupported otherwise.
bool tma_fwd2_would_run(int mode, const FwdStep& a);
cudaError_t launch_tma_fwd2(int mode, const FwdStep& a, int* err, cudaStream_t st);
cudaError_t launch_tma_adj(int mode, const AdjStep& a, int* err, cudaStream_t st);
// Whether launch_tma_adj takes the tiled kernel for steps shaped like `a`
// (buffers on 16-byte boundaries, tensor maps encodable) rather than falling
// back to the plain kernel.
bool tma_adj_would_run(int mode, const AdjStep& a);
// Per-call receiver table of the tiled adjoint of `mode`
// (tma_tiles(nx, ny, S, tma_adj_tile_rows(mode, tile_rows)) bytes at `flags`).
cudaError_t launch_tile_flags(int mode, const int32_t* rec_idx, int S, int nrec, int nx, int ny,
                              uint8_t* flags, cudaStream_t st, int tile_rows = 0);
// Instances on a canvas (ERNN_FLAG_INSTANCES).  The instance table passed
// by value to the kernel that writes the tile table: instances in the order
// of decreasing step count, each with its caller-side index.
constexpr int kMaxInstances = 256;
constexpr int kInstTileRows = 16;  // tile rows of every instance kernel (scalar constants)
struct InstDesc {
  int count;
  int id[kMaxInstances], x0[kMaxInstances], y0[kMaxInstances], nx[kMaxInstances];
  int ny[kMaxInstances], nt[kMaxInstances], base[kMaxInstances];
};
// Tiles of one instance of nx x ny cells.
__host__ __device__ inline int inst_tiles(int nx, int ny) {
  return ((nx + kInstTileRows - 1) / kInstTileRows) * ((ny + 63) / 64);
}
// Writes the tile table (sum of inst_tiles entries, in the order of d) and
// the per-instance boxes (2 x S int4) described in InstTiles.
cudaError_t launch_inst_table(const InstDesc& d, int4* tiles, int4* box, cudaStream_t st);
// Zeroes the one-cell ghost ring around every instance region (box[2 k]) in
// `nslots` canvas states of slot_floats floats from `base` (both components
// of each).  The kernels read a state outside the instance regions only
// there: cells further out feed only cells that are never stored, and the
// imaging masks them by selection, so a recompute segment or checkpoint
// buffer needs its rings zeroed, not the whole canvas.
cudaError_t launch_inst_ring_zero(float* base, size_t slot_floats, int nslots, int nx, int ny, const int4* box,
                                  int count, cudaStream_t st);
// Receiver table of the instance tile table: flags[t] = 1 where the tile's
// instance has a receiver in it (ntiles bytes).
cudaError_t launch_inst_tile_flags(const int32_t* rec_idx, int S, int nrec, int ny, const int4* box,
                                   uint8_t* flags, int ntiles, cudaStream_t st);

// Runs one bounded wait that cannot complete and copies the error word it
// records into *status_host; synchronises `st`.
cudaError_t wait_selftest(int* status_host, cudaStream_t st);

}  // namespace ernn
