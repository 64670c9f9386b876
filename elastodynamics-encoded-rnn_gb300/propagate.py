"""torch.autograd.Function over the CUDA library: forward time loop + hand adjoint.

ErnnPropagate replaces the reference's Python time loop
(Parameter_inversion/Inversion_adam.py:240-307,
Damage_inversion/Inversion_adam.py:331-393) and the autograd backward through
it (Inversion_adam.py:447).  Inputs are the physical constants (already
clamped by the caller, as get_material_params does), so any parameterisation
upstream keeps working with loss.backward() and torch.optim unchanged.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import torch

from . import _lib

MODE_SCALAR, MODE_DFIELD, MODE_FIELDS = _lib.MODE_SCALAR, _lib.MODE_DFIELD, _lib.MODE_FIELDS
RECORD_FIELDS, RECORD_RECEIVERS = _lib.RECORD_FIELDS, _lib.RECORD_RECEIVERS


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class Instances:
    """Independent instances on one canvas: instance k occupies rows
    [x0[k], x0[k] + nx[k]) and columns [y0[k], y0[k] + ny[k]) of the canvas
    grid and runs nt[k] steps (y0 and ny multiples of 4, regions at least one
    cell apart).  With it a Geometry's grid is the canvas, its shots are the
    instances (sources and receivers in canvas cells), nt is max(nt) and the
    constants are (S, 6) with rho (S,)."""
    x0: list
    y0: list
    nx: list
    ny: list
    nt: list

    def __post_init__(self):
        self._arrays = [(ctypes.c_int32 * len(v))(*[int(x) for x in v])
                        for v in (self.x0, self.y0, self.nx, self.ny, self.nt)]

    @property
    def count(self) -> int:
        return len(self.nt)

    def c_struct(self) -> _lib.ErnnInstances:
        P = ctypes.POINTER(ctypes.c_int32)
        return _lib.ErnnInstances(self.count, *[ctypes.cast(a, P) for a in self._arrays])


@dataclass
class Geometry:
    """Static description of one propagation: grid, time axis, sources, receivers.

    src_signal: (S, nt) float32 force amplitude per step and shot.
    src_map:    (S, bx, by) float32 spatial load inside each shot's box.
    src_origin: (S, 2) int32 box origin (x0, y0) per shot.
    rec_idx:    (S, R) int32 flat receiver cells (i*ny + j), or None for the
                dense history of the reference.
    ckpt_k:     checkpoint interval in steps (>= nt keeps every state).
    path:       PATH_AUTO (cluster-resident when the problem fits, else the
                tiled TMA kernels when eligible, else one plain kernel per
                step), PATH_STEP, PATH_RESIDENT or PATH_TILED.
    tile_rows:  tile rows of the tiled kernels, 16 or 32 (autotune.tune
                measures both).
    """
    nx: int
    ny: int
    nt: int
    h: float
    dt: float
    src_signal: torch.Tensor
    src_map: torch.Tensor
    src_origin: torch.Tensor
    stride: int = 1
    src_comp: int = 1
    rec_idx: torch.Tensor | None = None
    ckpt_k: int | None = None
    path: int = _lib.PATH_AUTO
    instances: Instances | None = None
    tile_rows: int = 16  # tiled kernels: 16 (64 x 16 tiles) or 32 (64 x 32, ERNN_FLAG_TALL_TILES)
    _checked: bool = field(default=False, repr=False)

    @property
    def nshots(self) -> int:
        return int(self.src_signal.shape[0])

    @property
    def nt_out(self) -> int:
        return (self.nt + self.stride - 1) // self.stride

    @property
    def record(self) -> int:
        return RECORD_FIELDS if self.rec_idx is None else RECORD_RECEIVERS

    def problem(self, mode: int, flags: int = 0) -> _lib.ErnnProblem:
        nrec = 0 if self.rec_idx is None else int(self.rec_idx.shape[1])
        if self.tile_rows == 32:
            flags |= _lib.FLAG_TALL_TILES
        k = self.ckpt_k if self.ckpt_k is not None else self.nt
        return _lib.ErnnProblem(self.nshots, self.nx, self.ny, self.nt, self.stride, mode,
                                self.record, nrec, self.src_comp, int(self.src_map.shape[1]),
                                int(self.src_map.shape[2]), int(max(1, k)), int(self.path),
                                int(flags), float(self.h), float(self.dt))

    def out_shape(self):
        if self.rec_idx is None:
            return (self.nshots, self.nt_out, self.nx, self.ny)
        return (self.nshots, self.nt_out, int(self.rec_idx.shape[1]))

    def check(self, device) -> None:
        """Host-side validation, once: shapes, dtypes, devices, receiver range."""
        if self._checked:
            return
        S = self.nshots
        if self.src_signal.shape != (S, self.nt):
            raise ValueError(f"src_signal must be (S, nt) = ({S}, {self.nt})")
        if self.src_map.dim() != 3 or self.src_map.shape[0] != S:
            raise ValueError("src_map must be (S, bx, by)")
        if tuple(self.src_origin.shape) != (S, 2):
            raise ValueError("src_origin must be (S, 2)")
        for name in ("src_signal", "src_map"):
            t = getattr(self, name)
            if t.dtype != torch.float32 or not t.is_contiguous() or t.device != device:
                raise ValueError(f"{name} must be contiguous float32 on {device}")
        if self.src_origin.dtype != torch.int32 or self.src_origin.device != device:
            raise ValueError(f"src_origin must be int32 on {device}")
        if self.rec_idx is not None:
            r = self.rec_idx
            if r.dim() != 2 or r.shape[0] != S or r.dtype != torch.int32 or r.device != device:
                raise ValueError(f"rec_idx must be (S, R) int32 on {device}")
            lo, hi = int(r.min()), int(r.max())
            if lo < 0 or hi >= self.nx * self.ny:
                raise ValueError("receiver index outside the grid")
        if self.instances is not None and self.instances.count != S:
            raise ValueError("one instance per shot")
        flags = _lib.FLAG_INSTANCES if self.instances is not None else 0
        rc = _lib.load().ernn_validate(ctypes.byref(self.problem(MODE_SCALAR, flags)))
        _lib.check("ernn_validate", rc)
        self._checked = True


def choose_ckpt_k(geom: Geometry, mode: int, device, budget_fraction: float = 0.4, flags: int = 0) -> int:
    """Checkpoint interval for a problem: keep every state when the tape fits in
    `budget_fraction` of the free device memory (no recomputation), otherwise the
    largest interval whose checkpoints plus recompute segment fit, starting from
    the memory-optimal sqrt(2 nt)."""
    lib = _lib.load()
    free, _ = torch.cuda.mem_get_info(device)
    budget = budget_fraction * free
    nt = geom.nt

    def need(k):
        p = geom.problem(mode, flags)
        p.ckpt_k = k
        return lib.ernn_tape_bytes(ctypes.byref(p), 1) + lib.ernn_adjoint_scratch_bytes(ctypes.byref(p))

    if need(nt) <= budget:
        return nt
    k = max(1, int(round((2 * nt) ** 0.5)))
    best = k
    while k < nt and need(k) <= budget:
        best = k
        k *= 2
    return best


def _inputs(geom: Geometry, C, D, rho) -> _lib.ErnnInputs:
    return _lib.ErnnInputs(_ptr(C), _ptr(D), _ptr(rho), _ptr(geom.src_signal),
                           _ptr(geom.src_map), _ptr(geom.src_origin), _ptr(geom.rec_idx))


def _mode_of(C: torch.Tensor, D) -> int:
    if D is not None:
        return MODE_DFIELD
    return MODE_SCALAR if C.dim() == 1 else MODE_FIELDS


def _require_cuda(*ts):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise RuntimeError("the ERNN propagation runs only on a CUDA device through "
                               "libernn_gb300.so; there is no CPU path")


class _DeviceStatus:
    """Error words of the device-side waits (ERNN_ERR_TIMEOUT when a bounded
    wait gave up), read back without stalling the stream: after each call a
    4-byte copy into pinned memory is enqueued with an event behind it, and the
    word is examined once the event has completed — at the next call, or in
    check_device_status(), which waits for it.  Calls made while a CUDA graph
    is being captured are not tracked."""

    def __init__(self):
        self.pending = []

    def enqueue(self, fn: str, prob, workspace: torch.Tensor, is_scratch: int) -> None:
        if torch.cuda.is_current_stream_capturing():
            return
        buf = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        rc = _lib.load().ernn_device_status(ctypes.byref(prob), _ptr(workspace), is_scratch,
                                            ctypes.c_void_p(buf.data_ptr()), _stream())
        _lib.check("ernn_device_status", rc)
        ev = torch.cuda.Event()
        ev.record()
        self.pending.append((fn, buf, ev))

    def poll(self, wait: bool = False) -> None:
        if not self.pending or torch.cuda.is_current_stream_capturing():
            return  # event queries are not allowed while a graph is being captured
        keep = []
        for fn, buf, ev in self.pending:
            if wait:
                ev.synchronize()
            elif not ev.query():
                keep.append((fn, buf, ev))
                continue
            code = int(buf[0])
            if code != 0:
                self.pending = []
                raise _lib.ErnnError(fn + " (device-side)", code,
                                     _lib.load().ernn_error_string(code).decode())
        self.pending = keep


_STATUS = _DeviceStatus()


def check_device_status() -> None:
    """Wait for the status words of all earlier calls and raise ErnnError if a
    bounded device-side wait of any of them gave up."""
    _STATUS.poll(wait=True)


class ErnnPropagate(torch.autograd.Function):
    """(C, D, rho) -> (out_ux, out_uy) through the fused CUDA time loop.

    C:   (6,) scalar constants (SCALAR, or C0 of DFIELD), (S, 6) per-shot
         constants (SCALAR: independent media advancing together, with rho (S,)),
         or (6, nx, ny) planes (FIELDS).
    D:   (nx, ny) degradation map or None.
    rho: 0-dim density, or (S,) with per-shot constants.
    Returns the dense history (S, nt_out, nx, ny) per component, or receiver
    traces (S, nt_out, R), frame k holding u^{k*stride+1}.
    Gradients: dL/dC (FP64 reduction, returned as float32; (S, 6) with
    per-shot constants) in SCALAR mode, dL/dC(x) in FIELDS mode, dL/dD(x) in
    DFIELD mode (C0 gets none).
    """

    @staticmethod
    def forward(ctx, C, D, rho, geom: Geometry, keep_tape: bool = True):
        _require_cuda(C, D, rho)
        dev = C.device
        per_shot = D is None and C.dim() == 2 and C.shape[-1] == 6
        mode = MODE_SCALAR if per_shot else _mode_of(C, D)
        inst = geom.instances
        if inst is not None and not per_shot:
            raise ValueError("instances take (S, 6) constants with rho (S,)")
        flags = _lib.FLAG_INSTANCES if inst is not None else (_lib.FLAG_SHOT_CONSTANTS if per_shot else 0)
        C = C.detach().to(torch.float32).contiguous()
        D = None if D is None else D.detach().to(torch.float32).contiguous()
        rho = rho.detach().to(torch.float32).reshape(-1).contiguous()
        if per_shot:
            if tuple(C.shape) != (geom.nshots, 6) or tuple(rho.shape) != (geom.nshots,):
                raise ValueError("per-shot constants must be (S, 6) with rho (S,)")
        elif mode == MODE_FIELDS and tuple(C.shape) != (6, geom.nx, geom.ny):
            raise ValueError("per-cell constants must be (6, nx, ny)")
        elif mode != MODE_FIELDS and tuple(C.shape) != (6,):
            raise ValueError("scalar constants must be (6,)")
        if not per_shot and rho.numel() != 1:
            raise ValueError("rho must be a scalar")
        if D is not None and tuple(D.shape) != (geom.nx, geom.ny):
            raise ValueError("D must be (nx, ny)")
        geom.check(dev)
        _STATUS.poll()
        lib = _lib.load()
        if geom.ckpt_k is None:
            geom.ckpt_k = choose_ckpt_k(geom, mode, dev, flags=flags)
        prob = geom.problem(mode, flags)
        want_grad = bool(keep_tape and (ctx.needs_input_grad[0] or ctx.needs_input_grad[1]))
        tape_bytes = lib.ernn_tape_bytes(ctypes.byref(prob), int(want_grad))
        with torch.cuda.device(dev):
            tape = torch.empty(tape_bytes, dtype=torch.uint8, device=dev)
            out_ux = torch.empty(geom.out_shape(), dtype=torch.float32, device=dev)
            out_uy = torch.empty(geom.out_shape(), dtype=torch.float32, device=dev)
            ins = _inputs(geom, C, D, rho)
            if inst is not None:
                ist = inst.c_struct()
                rc = lib.ernn_forward_instances(ctypes.byref(prob), ctypes.byref(ins), ctypes.byref(ist),
                                                _ptr(out_ux), _ptr(out_uy), _ptr(tape),
                                                ctypes.c_size_t(tape_bytes), int(want_grad), _stream())
                _lib.check("ernn_forward_instances", rc)
            else:
                rc = lib.ernn_forward(ctypes.byref(prob), ctypes.byref(ins), _ptr(out_ux),
                                      _ptr(out_uy), _ptr(tape), ctypes.c_size_t(tape_bytes),
                                      int(want_grad), _stream())
                _lib.check("ernn_forward", rc)
            _STATUS.enqueue("ernn_forward", prob, tape, 0)
        ctx.mode = mode
        # the problem as the tape was laid out: a later change of the geometry
        # (its checkpoint interval, say) must not change how backward reads it
        ctx.prob = _lib.ErnnProblem.from_buffer_copy(prob)
        ctx.out_shape = geom.out_shape()
        ctx.srcs = (geom.src_signal, geom.src_map, geom.src_origin, geom.rec_idx)
        ctx.inst = inst
        ctx.tape = tape if want_grad else None
        ctx.save_for_backward(C, D, rho)
        return out_ux, out_uy

    @staticmethod
    def backward(ctx, g_ux, g_uy):
        C, D, rho = ctx.saved_tensors
        mode = ctx.mode
        if ctx.tape is None:
            return None, None, None, None, None
        dev = C.device
        shape = ctx.out_shape
        g_ux = torch.zeros(shape, device=dev) if g_ux is None else g_ux.to(torch.float32).contiguous()
        g_uy = torch.zeros(shape, device=dev) if g_uy is None else g_uy.to(torch.float32).contiguous()
        lib = _lib.load()
        prob = ctx.prob
        scratch_bytes = lib.ernn_adjoint_scratch_bytes(ctypes.byref(prob))
        with torch.cuda.device(dev):
            scratch = torch.empty(scratch_bytes, dtype=torch.uint8, device=dev)
            grad_C64 = torch.empty(tuple(C.shape), dtype=torch.float64, device=dev) \
                if mode == MODE_SCALAR else None
            if mode == MODE_FIELDS:
                grad_field = torch.empty((6, prob.nx, prob.ny), dtype=torch.float32, device=dev)
            elif mode == MODE_DFIELD:
                grad_field = torch.empty((prob.nx, prob.ny), dtype=torch.float32, device=dev)
            else:
                grad_field = None
            sig, smap, sorg, rec = ctx.srcs
            ins = _lib.ErnnInputs(_ptr(C), _ptr(D), _ptr(rho), _ptr(sig), _ptr(smap), _ptr(sorg), _ptr(rec))
            if ctx.inst is not None:
                ist = ctx.inst.c_struct()
                rc = lib.ernn_adjoint_instances(ctypes.byref(prob), ctypes.byref(ins), ctypes.byref(ist),
                                                _ptr(g_ux), _ptr(g_uy), _ptr(ctx.tape),
                                                ctypes.c_size_t(ctx.tape.numel()), _ptr(scratch),
                                                ctypes.c_size_t(scratch_bytes), _ptr(grad_C64), _stream())
                _lib.check("ernn_adjoint_instances", rc)
            else:
                rc = lib.ernn_adjoint(ctypes.byref(prob), ctypes.byref(ins), _ptr(g_ux), _ptr(g_uy),
                                      _ptr(ctx.tape), ctypes.c_size_t(ctx.tape.numel()),
                                      _ptr(scratch), ctypes.c_size_t(scratch_bytes), _ptr(grad_C64),
                                      _ptr(grad_field), _stream())
                _lib.check("ernn_adjoint", rc)
            _STATUS.enqueue("ernn_adjoint", prob, scratch, 1)
        if mode == MODE_SCALAR:
            return grad_C64.to(torch.float32), None, None, None, None
        if mode == MODE_FIELDS:
            return grad_field, None, None, None, None
        return None, grad_field, None, None, None


def propagate(C, rho, geom: Geometry, D=None):
    """Functional form of ErnnPropagate.  The forward keeps a tape for the
    adjoint only when grad mode is on and C or D requires a gradient."""
    keep = torch.is_grad_enabled() and any(
        t is not None and t.requires_grad for t in (C, D))
    return ErnnPropagate.apply(C, D, rho, geom, keep)


def elastic_operator_with_force(ux, uy, C11, C22, C12, C16, C26, C66, h, force_x, force_y, rho):
    """((A u + f) / rho) for (S, nx, ny) fields on the GPU, the values of
    _general_anisotropic_elastic_operator_with_force
    (Parameter_inversion/Inversion_adam.py:54-106).  Constants are 0-dim
    (scalar mode) or (1, nx, ny) planes; with planes the force is added as given
    (the reference's spatially varying variant adds force.transpose(1, 2),
    Damage_inversion/Inversion_adam.py:169-174 — transpose it before calling to
    reproduce that).  Forward values only: no autograd graph is recorded."""
    _require_cuda(ux, uy)
    dev = ux.device
    S, nx, ny = ux.shape
    consts = [torch.as_tensor(c, device=dev, dtype=torch.float32) for c in
              (C11, C22, C12, C16, C26, C66)]
    if consts[0].dim() == 0:
        C = torch.stack(consts).contiguous()
        mode = MODE_SCALAR
    else:
        C = torch.cat([c.reshape(1, nx, ny) for c in consts]).contiguous()
        mode = MODE_FIELDS
    ux = ux.detach().to(torch.float32).contiguous()
    uy = uy.detach().to(torch.float32).contiguous()
    fx = None if force_x is None else torch.as_tensor(force_x, device=dev).to(torch.float32).expand(S, nx, ny).contiguous()
    fy = None if force_y is None else torch.as_tensor(force_y, device=dev).to(torch.float32).expand(S, nx, ny).contiguous()
    rho_t = torch.as_tensor(rho, device=dev, dtype=torch.float32).reshape(1).contiguous()
    Lux = torch.empty_like(ux)
    Luy = torch.empty_like(uy)
    lib = _lib.load()
    with torch.cuda.device(dev):
        rc = lib.ernn_operator(S, nx, ny, mode, float(h), _ptr(C), None, _ptr(rho_t), _ptr(ux),
                               _ptr(uy), _ptr(fx), _ptr(fy), _ptr(Lux), _ptr(Luy), _stream())
    _lib.check("ernn_operator", rc)
    return Lux, Luy
