/*
 * ernn.h — C ABI of the GB300 ERNN propagation library (libernn_gb300.so).
 *
 * The library advances the 2D anisotropic elastic displacement field of the
 * Elastodynamics-Encoded RNN with a fused sm_103a stencil kernel per step and
 * returns the exact discrete gradient through a hand-written reverse-time
 * adjoint with checkpoint recomputation.
 *
 * Conventions shared by every entry point:
 *   - Grid (nx, ny), row-major with y contiguous: cell (i, j) is at i*ny + j,
 *     the layout of the reference's (1, nx, ny) tensors.
 *   - The constants are ordered C11, C22, C12, C16, C26, C66 (x-y plane of the
 *     reference; the x-z names C11, C33, C13, C15, C35, C55 map one to one).
 *   - Every pointer argument is DEVICE memory unless its comment says host.
 *     The caller allocates everything; the library allocates nothing.
 *   - `stream` is a cudaStream_t passed as void*; all work is enqueued on it,
 *     nothing synchronises the host.
 *   - Return value: ERNN_OK (0) or a positive error code; ernn_error_string()
 *     describes it.  Nothing aborts or traps.
 *
 * The reference exposes this path as Python functions and an nn.Module; each
 * entry point below names the reference code it stands in for (paths inside
 * the reference project).
 */
#ifndef ERNN_H_
#define ERNN_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ERNN_ABI_VERSION 1

enum {
  ERNN_OK = 0,
  ERNN_ERR_INVALID = 1,     /* bad argument: null pointer, size or enum */
  ERNN_ERR_WORKSPACE = 2,   /* workspace smaller than the query returned */
  ERNN_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  ERNN_ERR_UNSTABLE = 4,    /* leapfrog stability bound violated */
  ERNN_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  ERNN_ERR_UNSUPPORTED = 6  /* valid request this library cannot serve */
};

enum {
  ERNN_MODE_SCALAR = 0, /* six scalar constants */
  ERNN_MODE_DFIELD = 1, /* C_ij(x) = (1 - D(x)) C0_ij: scalar C0 and a degradation map D */
  ERNN_MODE_FIELDS = 2  /* six per-cell constant planes */
};

enum {
  ERNN_RECORD_FIELDS = 0,   /* dense history (S, nt_out, nx, ny) per component */
  ERNN_RECORD_RECEIVERS = 1 /* receiver traces (S, nt_out, nrec) per component */
};

enum {
  ERNN_PATH_AUTO = 0,     /* cluster-resident when the problem fits, else tiled when
                             eligible, else per-step */
  ERNN_PATH_STEP = 1,     /* one fused kernel launch per time step (any size, any mode) */
  ERNN_PATH_RESIDENT = 2, /* one thread-block cluster per shot holds the state in
                             distributed shared memory for all steps (scalar constants,
                             ny % 4 == 0, state small enough); ERNN_ERR_UNSUPPORTED otherwise */
  ERNN_PATH_TILED = 3     /* one launch per time step of persistent CTAs that stream
                             64-column tiles (16 rows; 32 for the degradation-map
                             adjoint) through TMA loads (scalar constants or a
                             degradation map, ny % 4 == 0); ERNN_ERR_UNSUPPORTED
                             otherwise */
};

/* Problem flags. */
enum {
  /* SCALAR mode: every shot has its own constants and density — C is
   * nshots x 6, rho nshots, grad_C nshots x 6 — so independent inversions
   * of one grid size and step count advance in the same launches */
  ERNN_FLAG_SHOT_CONSTANTS = 1,
  /* Independent instances of uneven grid sizes and step counts on one
   * canvas (ernn_forward_instances / ernn_adjoint_instances): nx x ny is the
   * canvas, holding ONE state plane; nshots is the number of instances, each
   * a rectangular region of the canvas with its own constants (C nshots x 6,
   * rho nshots, as ERNN_FLAG_SHOT_CONSTANTS), source (src_signal nshots x nt,
   * src_map, src_origin in canvas cells), receivers (rec_idx: canvas cell
   * indices) and step count; nt is the largest step count.  SCALAR mode,
   * RECORD_RECEIVERS, tiled kernels (ERNN_PATH_AUTO or _TILED). */
  ERNN_FLAG_INSTANCES = 2,
  /* Tiled kernels: 64 x 32 tiles for the forward steps and the scalar
   * adjoint instead of 64 x 16 (a tenth fewer halo rows per cell, one CTA
   * fewer per SM); a tile geometry the autotuner measures.  Results are the
   * same up to FP32 rounding of the imaging sums' grouping.  The D-field
   * mode takes 64 x 32 tiles with or without the flag (its adjoint always
   * did; its forward measured faster so: 8 x 512^2 shots, 81.3 -> 75.6 ms
   * per inversion iteration). */
  ERNN_FLAG_TALL_TILES = 4
};

/* One propagation problem.  Plain data; identical layout in C, C++, ctypes. */
typedef struct ErnnProblem {
  int32_t nshots;   /* independent shots sharing the medium (batched) */
  int32_t nx, ny;   /* grid */
  int32_t nt;       /* time steps */
  int32_t stride;   /* frame k records u^{k*stride+1} (step i records when i % stride == 0) */
  int32_t mode;     /* ERNN_MODE_* */
  int32_t record;   /* ERNN_RECORD_* */
  int32_t nrec;     /* receivers per shot (ERNN_RECORD_RECEIVERS) */
  int32_t src_comp; /* 0: force along x, 1: force along y */
  int32_t src_bx, src_by; /* source map box size in cells */
  int32_t ckpt_k;   /* checkpoint interval in steps; >= nt keeps every state */
  int32_t path;     /* ERNN_PATH_*: which kernels run the time loop */
  int32_t flags;    /* ERNN_FLAG_* bits; others must be 0 */
  double h;         /* grid spacing [m] */
  double dt;        /* time step [s] */
} ErnnProblem;

/* Inputs shared by the forward and the adjoint (all device pointers). */
typedef struct ErnnInputs {
  const float* C;            /* SCALAR, DFIELD: 6 floats (nshots x 6 with
                                ERNN_FLAG_SHOT_CONSTANTS); FIELDS: 6 planes of nx*ny */
  const float* D;            /* DFIELD: nx*ny; otherwise NULL */
  const float* rho;          /* 1 float (nshots with ERNN_FLAG_SHOT_CONSTANTS), density [kg/m^3] */
  const float* src_signal;   /* nshots*nt: force amplitude of step i */
  const float* src_map;      /* nshots*src_bx*src_by: spatial load inside the box */
  const int32_t* src_origin; /* nshots*2: (x0, y0) of each shot's box; may lie partly outside */
  const int32_t* rec_idx;    /* nshots*nrec flat cell indices; NULL unless RECEIVERS */
} ErnnInputs;

/* ABI version of the loaded library (ERNN_ABI_VERSION). */
int ernn_abi_version(void);

/* Static description of an error code. */
const char* ernn_error_string(int code);

/* Validate a problem on the host; ERNN_OK or ERNN_ERR_INVALID. */
int ernn_validate(const ErnnProblem* p);

/* Bytes of the tape: state the forward writes and the adjoint reads
 * (checkpoints or, when ckpt_k >= nt, every state).  With with_tape == 0 the
 * forward only needs the two-level state and no tape. (host call) */
size_t ernn_tape_bytes(const ErnnProblem* p, int with_tape);

/* Bytes of scratch the adjoint needs besides the tape (recompute segment,
 * gradient accumulators, FP64 partial sums). (host call) */
size_t ernn_adjoint_scratch_bytes(const ErnnProblem* p);

/* Leapfrog stability of the scheme for scalar constants (host call, host
 * pointers): *courant receives max over wavenumbers of the largest
 * eigenvalue of -(dt^2/rho) A(k) divided by 4 (the scheme is stable for
 * values <= 1).  Returns ERNN_ERR_UNSTABLE when it exceeds 1.
 * No counterpart in the reference, which does not check stability. */
int ernn_check_stability(const double* C6_host, double rho, double h, double dt, double* courant);

/* One application of the operator, ((A u + f) / rho) for nshots fields.
 * Stands in for _general_anisotropic_elastic_operator_with_force
 * (Parameter_inversion/Inversion_adam.py:54-106) and, with mode FIELDS, its
 * spatially varying variant (Damage_inversion/Inversion_adam.py:100-176; that
 * one adds force.transpose(1, 2), so pass the transposed force to reproduce
 * it).  ux, uy, fx, fy, Lux, Luy: (nshots, nx, ny); fx, fy may be NULL. */
int ernn_operator(int32_t nshots, int32_t nx, int32_t ny, int32_t mode, double h,
                  const float* C, const float* D, const float* rho, const float* ux,
                  const float* uy, const float* fx, const float* fy, float* Lux, float* Luy,
                  void* stream);

/* Forward time loop.  Stands in for CFRPWaveSimulatorRicker.forward
 * (Parameter_inversion/Inversion_adam.py:240-307) and
 * SpatiallyVaryingAnisotropicSimulator.forward
 * (Damage_inversion/Inversion_adam.py:331-393), batched over shots.
 * out_ux, out_uy: (nshots, nt_out, nx, ny) for RECORD_FIELDS or
 * (nshots, nt_out, nrec) for RECORD_RECEIVERS, nt_out = ceil(nt / stride).
 * tape: ernn_tape_bytes(p, with_tape) bytes; keep it unchanged until
 * ernn_adjoint when with_tape != 0. */
int ernn_forward(const ErnnProblem* p, const ErnnInputs* in, float* out_ux, float* out_uy,
                 void* tape, size_t tape_bytes, int with_tape, void* stream);

/* Reverse-time adjoint: the gradient that loss.backward() produces through
 * the forward loop (Parameter_inversion/Inversion_adam.py:447,
 * Damage_inversion/Inversion_adam.py:511).
 * g_ux, g_uy: dL/d(out_ux, out_uy), same shapes as the forward outputs.
 * tape: the tape of the matching ernn_forward(with_tape = 1) call.
 * scratch: ernn_adjoint_scratch_bytes(p) bytes.
 * grad_C: SCALAR: 6 doubles dL/dC (FP64 reduction over cells, steps, shots),
 *         nshots x 6 with ERNN_FLAG_SHOT_CONSTANTS (each shot's own constants);
 *         other modes: may be NULL.
 * grad_field: FIELDS: 6 planes dL/dC_ij(x) (float); DFIELD: nx*ny dL/dD(x);
 *             SCALAR: may be NULL. */
int ernn_adjoint(const ErnnProblem* p, const ErnnInputs* in, const float* g_ux,
                 const float* g_uy, const void* tape, size_t tape_bytes, void* scratch,
                 size_t scratch_bytes, double* grad_C, float* grad_field, void* stream);

/* Forward time loop that allocates nothing, for callers that cannot call
 * cudaMalloc: code running while another framework captures a CUDA graph on
 * the stream, real-time loops that cannot afford the device synchronisation
 * of an allocation, FFI hosts without a device allocator.  Same problem,
 * inputs, outputs and results as ernn_forward(with_tape = 0) on the per-step
 * kernels; the two-level wavefield lives in an 8 MiB file-scope device array
 * that every GPU loading the library keeps until exit.  Problems needing
 * more than that (the coefficient blocks, 64 B each, + 2 x nshots x 2 x nx x ny x 4 B, each rounded up to
 * 256 B) are rejected with ERNN_ERR_WORKSPACE.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current: make it before any stream capture; `stream` must belong to the
 * current device.  All calls share the array, so calls that overlap on the
 * GPU race; serialise them.  Produces no tape: there is no adjoint for it.
 * No counterpart in the reference. */
int ernn_forward_static(const ErnnProblem* p, const ErnnInputs* in, float* out_ux, float* out_uy,
                        void* stream);

/* ---------------------------------------------------------------------------
 * Many independent inversions of uneven grid sizes and step counts advancing
 * in one launch sequence (a problem with ERNN_FLAG_INSTANCES).  The caller
 * places each instance in a region of the canvas: regions at least one row
 * and four columns apart (the cells between them, never written, are the
 * instances' zero ghost rings), y0 and ny multiples of 4.  Every time step is
 * one launch over a table of all instances' 64 x 16 tiles, ordered by step
 * count, of which a step takes the prefix of instances still running: an
 * instance with nt_k steps takes part in forward steps i < nt_k and adjoint
 * steps m <= nt_k, on the same time axis, so checkpoint segments are shared.
 * Instance k's trace frames beyond its own ceil(nt_k / stride) are zero.
 * The reference runs one inversion per loop (batch of one,
 * Parameter_inversion/Inversion_adam.py:252); no counterpart there. */
#define ERNN_MAX_INSTANCES 256

typedef struct ErnnInstances {
  int32_t count;        /* instances: the problem's nshots (<= ERNN_MAX_INSTANCES) */
  const int32_t* x0;    /* host: count first rows of the regions */
  const int32_t* y0;    /* host: count first columns (multiples of 4) */
  const int32_t* nx;    /* host: count region rows */
  const int32_t* ny;    /* host: count region columns (multiples of 4) */
  const int32_t* nt;    /* host: count step counts, 1 .. problem nt */
} ErnnInstances;

/* Forward time loop of every instance (tape: ernn_tape_bytes of the canvas
 * problem).  Outputs: traces (nshots, nt_out, nrec) per component. */
int ernn_forward_instances(const ErnnProblem* p, const ErnnInputs* in, const ErnnInstances* inst,
                           float* out_ux, float* out_uy, void* tape, size_t tape_bytes, int with_tape,
                           void* stream);

/* Adjoint of every instance: grad_C nshots x 6 (each instance's constants),
 * FP64 sums over its cells and steps. */
int ernn_adjoint_instances(const ErnnProblem* p, const ErnnInputs* in, const ErnnInstances* inst,
                           const float* g_ux, const float* g_uy, const void* tape, size_t tape_bytes,
                           void* scratch, size_t scratch_bytes, double* grad_C, void* stream);

/* ---------------------------------------------------------------------------
 * FEM data generator (the step before the ERNN path): the explicit
 * finite-element time loop that produces the reference's training
 * wavefields, solve_2d_anisotropic_wave_fem_ricker_fixed
 * (Parameter_inversion/FEM_generate_data.py:196-590) — structured
 * checkerboard triangular mesh, lumped mass, constant-strain elements with
 * three Gauss points, central differences, edges fixed at zero, frames scaled
 * by out_scale (0.7 there).  The host keeps the generator's dt / nt choice
 * (its CFL adjustment) and computes the nodal load and the time factors. */
typedef struct ErnnFemProblem {
  int32_t nx, ny;   /* nodes along x and y */
  int32_t nt;       /* time levels 0 .. nt-1 (u^0 = u^1 = 0) */
  int32_t stride;   /* frame k holds level k*stride; nt_out = ceil(nt / stride) */
  double dx, dy;    /* node spacing (Lx / (nx-1), Ly / (ny-1)) */
  double dt, rho;
  double C[6];      /* C11, C22, C12, C16, C26, C66 */
  double out_scale; /* factor applied to the frames */
} ErnnFemProblem;

/* Device workspace of ernn_fem_forward: three time levels of two components. */
size_t ernn_fem_workspace_bytes(const ErnnFemProblem* p);

/* load: (nx, ny) nodal Gaussian (y fastest), signal: (nt) time factors,
 * C_fields: NULL (the constants of p->C everywhere) or 6 planes (nx, ny) of
 * per-node constants, each element taking those of the node nearest its
 * centroid (the damaged-plate generator, Damage_inversion/FEM_generate_data.py:
 * 1002-1017); frames_x / frames_y: (nt_out, nx, ny) outputs; all device
 * memory, enqueued on `stream`.  Replaces the time loop of
 * Parameter_inversion/FEM_generate_data.py:474-499 (Damage_inversion/...:1093-1117)
 * and the frame extraction of :519-526 / :926-930. */
int ernn_fem_forward(const ErnnFemProblem* p, const float* load, const float* signal,
                     const float* C_fields, float* frames_x, float* frames_y, void* workspace,
                     size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Misfit (the step between the forward and the adjoint): the loss of
 * predicted against observed series and its gradient, which is the adjoint
 * source.  Series are laid out series x frames x nx x ny floats, as the
 * histories (S, nt_out, nx, ny) of ernn_forward (traces (S, nt_out, nrec):
 * nx = 1, ny = nrec).  Counted: frames 0, frame_stride, ... and within them
 * cells (i, j) with i and j multiples of space_stride; count = series x
 * ceil(frames / frame_stride) x ceil(nx / space_stride) x ceil(ny / space_stride).
 *   loss = wx * sum((px - ox)^2) / count + wy * sum((py - oy)^2) / count
 * over the counted elements, with predictions and observations in the same
 * layout.  This is compute_loss of Parameter_inversion/Inversion_adam.py:358-391
 * (wx = wy = 1, [:, ::ts, ::ss, ::ss] of both, :339-342) and the data term of
 * Damage_inversion/Inversion_adam.py:441-463 (wx = 5, wy = 1, [:, ::ts] of
 * both, :420-422). */
typedef struct ErnnSeries {
  int64_t series;        /* series (shots) */
  int64_t frames;        /* frames per series */
  int32_t nx, ny;        /* frame shape, ny contiguous */
  int32_t frame_stride;  /* >= 1 */
  int32_t space_stride;  /* >= 1 */
  double wx, wy;         /* weights of the two components, >= 0 */
} ErnnSeries;

/* Device workspace of ernn_misfit (block partials; fixed size). */
size_t ernn_misfit_workspace_bytes(void);

/* loss: 3 device doubles <- (loss, mean square of x, mean square of y).
 * Differences in FP32, sums in FP64, fixed summation order (reproducible).
 * Enqueued on `stream`; ERNN_ERR_INVALID for a bad layout or weights. */
int ernn_misfit(const ErnnSeries* s, const float* px, const float* py, const float* ox,
                const float* oy, double* loss, void* workspace, size_t workspace_bytes,
                void* stream);

/* Gradient of the three outputs of ernn_misfit against the upstream
 * gradients grad_loss = 3 device doubles (g0, g1, g2) of (loss, mean square
 * x, mean square y), or NULL for (1, 0, 0):
 *   gx = 2 (wx g0 + g1) (px - ox) / count on counted elements, 0 elsewhere
 *   gy = 2 (wy g0 + g2) (py - oy) / count
 * over the whole series x frames x nx x ny layout. */
int ernn_misfit_grad(const ErnnSeries* s, const float* px, const float* py, const float* ox,
                     const float* oy, const double* grad_loss, float* gx, float* gy, void* stream);

/* ---------------------------------------------------------------------------
 * Fused Adam step over every parameter tensor of an optimiser in one launch
 * (torch.optim.Adam of the inversion loops, Parameter_inversion/Inversion_adam.py:421-447,
 * Damage_inversion/Inversion_adam.py:477-514; no amsgrad).  Per element, t =
 * step count after this step:
 *   g = grad + weight_decay p;  m += (1 - beta1)(g - m);  v = beta2 v + (1 - beta2) g^2
 *   p += -lr / (1 - beta1^t) * m / (sqrt(v) / sqrt(1 - beta2^t) + eps)
 * FP32 state, bias corrections in FP64.  The step count is device state, so
 * a CUDA graph that captured the call advances it on every replay. */
typedef struct ErnnAdamTensor {
  float* param;          /* n floats, updated in place */
  const float* grad;     /* n floats */
  float* exp_avg;        /* n floats, zero before the first step */
  float* exp_avg_sq;     /* n floats, zero before the first step */
  int64_t n;
} ErnnAdamTensor;

typedef struct ErnnAdamHyper {
  double lr, beta1, beta2, eps, weight_decay;
} ErnnAdamHyper;

/* tensors: DEVICE array of ntensors descriptors; max_numel: the largest n;
 * h: host; state: 2 device int32 (step count, then a ticket that must be 0
 * before the first call; both zero-initialised by the caller). */
int ernn_adam_step(const ErnnAdamTensor* tensors, int32_t ntensors, int64_t max_numel,
                   const ErnnAdamHyper* h, int32_t* state, void* stream);

/* Number of kernels this library has launched since it was loaded. (host call)
 * Diagnostic; no counterpart in the reference. */
uint64_t ernn_launch_count(void);

/* Device-side status of the last call that used `workspace`: the tape of
 * ernn_forward (is_scratch == 0) or the scratch of ernn_adjoint
 * (is_scratch == 1), for problem `p`.  Enqueues on `stream` a 4-byte
 * device-to-host copy into *status_host (pinned host memory keeps it
 * asynchronous); once the stream has passed it, the word is ERNN_OK, or
 * ERNN_ERR_TIMEOUT when a bounded device-side wait of that call gave up (its
 * outputs are then not valid).  No counterpart in the reference. */
int ernn_device_status(const ErnnProblem* p, const void* workspace, int is_scratch,
                       int32_t* status_host, void* stream);

/* Failure path of the device-side waits, without a fault: one CTA waits on a
 * barrier that nothing completes, with the same bounded wait as the
 * propagation kernels, gives up after about a second and records
 * ERNN_ERR_TIMEOUT; that word is copied into *status_host and `stream` is
 * synchronised.  The context stays usable.  No counterpart in the reference. */
int ernn_wait_selftest(int32_t* status_host, void* stream);

/* ERNN_PATH_STEP, _RESIDENT or _TILED: the kernels that ran the time loop of
 * the last ernn_forward / ernn_adjoint call of this process (ERNN_PATH_AUTO
 * before any call). (host call)  Diagnostic; no counterpart in the reference. */
int32_t ernn_last_path(void);

/* Launch overlap of consecutive time-step kernels on the per-step and tiled
 * paths and of the FEM generator's levels (programmatic dependent launch: a
 * step kernel is scheduled while the previous one drains, loads its
 * step-independent inputs, then waits for the previous step's state).  On by
 * default; results are bitwise the same either way.  Returns the previous
 * setting. (host call)  No counterpart in the reference. */
int ernn_set_launch_overlap(int on);

/* Diagnostic kernel timing (no counterpart in the reference): while enabled,
 * every launch of the library is bracketed by CUDA events on its stream.
 * enable != 0 starts a new measurement (totals reset). (host call) */
int ernn_profile_enable(int enable);

/* Totals since ernn_profile_enable(1), per kernel class
 * [0: forward time loop, 1: adjoint time loop, 2: everything else]: device
 * time in milliseconds (ms3[3], host), launch counts (launches3[3], host) and
 * the algorithmic DRAM bytes of the work those launches did (alg_bytes3[3],
 * host, may be NULL).  Waits for the recorded events. (host call) */
int ernn_profile_read(double* ms3, uint64_t* launches3, double* alg_bytes3);

#ifdef __cplusplus
}
#endif

#endif /* ERNN_H_ */
