"""ctypes front end of the C oracle (test infrastructure only).

ORACLE: this module is the oracle the CUDA path is compared against.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import it.

It restates the reference's forward time loop
(Parameter_inversion/Inversion_adam.py:240-307), its operator
(Inversion_adam.py:54-106, Damage_inversion/Inversion_adam.py:100-176) and the
gradient autograd returns for it (Inversion_adam.py:447), in FP32 or FP64.
Parity is pinned against golden vectors generated from the reference module
itself (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build_oracle

MODE_SCALAR, MODE_DFIELD, MODE_FIELDS = 0, 1, 2
RECORD_FIELDS, RECORD_RECEIVERS = 0, 1


class _Problem(ctypes.Structure):
    _fields_ = [
        ("nshots", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("nt", ctypes.c_int32), ("stride", ctypes.c_int32), ("mode", ctypes.c_int32),
        ("record", ctypes.c_int32), ("nrec", ctypes.c_int32), ("src_comp", ctypes.c_int32),
        ("src_bx", ctypes.c_int32), ("src_by", ctypes.c_int32), ("ref_f32_sum", ctypes.c_int32),
        ("h", ctypes.c_double), ("dt", ctypes.c_double),
    ]


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        _LIB = ctypes.CDLL(path)
    return _LIB


@dataclass
class Case:
    """One propagation problem in plain numpy arrays.

    C: (6,) scalar constants (C11, C22, C12, C16, C26, C66) for MODE_SCALAR and
       the undamaged C0 for MODE_DFIELD; (6, nx, ny) planes for MODE_FIELDS.
    D: (nx, ny) degradation map for MODE_DFIELD.
    src_signal: (S, nt); src_map: (S, bx, by); src_origin: (S, 2) int.
    rec_idx: (S, R) flat cell indices x*ny + y (record == RECORD_RECEIVERS).
    """
    nx: int
    ny: int
    nt: int
    h: float
    dt: float
    rho: float
    C: np.ndarray
    src_signal: np.ndarray
    src_map: np.ndarray
    src_origin: np.ndarray
    stride: int = 1
    mode: int = MODE_SCALAR
    record: int = RECORD_FIELDS
    rec_idx: np.ndarray | None = None
    D: np.ndarray | None = None
    src_comp: int = 1
    # form C12 + C66 in float32 as the reference does (its constants are float32
    # tensors even in its FP64 run); 0 gives a pure FP64 scheme
    ref_f32_sum: int = 1

    @property
    def nshots(self) -> int:
        return int(self.src_signal.shape[0])

    @property
    def nt_out(self) -> int:
        return (self.nt + self.stride - 1) // self.stride

    def problem(self) -> _Problem:
        bx, by = int(self.src_map.shape[1]), int(self.src_map.shape[2])
        nrec = 0 if self.rec_idx is None else int(self.rec_idx.shape[1])
        return _Problem(self.nshots, self.nx, self.ny, self.nt, self.stride, self.mode,
                        self.record, nrec, self.src_comp, bx, by, self.ref_f32_sum, float(self.h),
                        float(self.dt))

    def out_shape(self):
        if self.record == RECORD_FIELDS:
            return (self.nshots, self.nt_out, self.nx, self.ny)
        return (self.nshots, self.nt_out, int(self.rec_idx.shape[1]))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _arr(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


def forward(case: Case, precision: str = "f64", keep_states: bool = False):
    """Run the forward loop.  Returns (out_ux, out_uy, states or None)."""
    dt = np.float64 if precision == "f64" else np.float32
    fn = getattr(_lib(), f"oracle_forward_{precision}")
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_Problem)] + [ctypes.c_void_p] * 6 + [real] + [ctypes.c_void_p] * 3
    C, D = _arr(case.C, dt), _arr(case.D, dt)
    sig, smap = _arr(case.src_signal, dt), _arr(case.src_map, dt)
    org = _arr(case.src_origin, np.int32)
    rec = _arr(case.rec_idx, np.int32)
    out_ux = np.zeros(case.out_shape(), dt)
    out_uy = np.zeros(case.out_shape(), dt)
    states = None
    if keep_states:
        states = np.zeros((case.nt + 1, case.nshots, 2, case.nx, case.ny), dt)
    p = case.problem()
    rc = fn(ctypes.byref(p), _ptr(C), _ptr(D), _ptr(sig), _ptr(smap), _ptr(org), _ptr(rec),
            real(case.rho), _ptr(out_ux), _ptr(out_uy), _ptr(states))
    if rc != 0:
        raise ValueError(f"oracle_forward failed with code {rc}")
    return out_ux, out_uy, states


def adjoint(case: Case, states: np.ndarray, g_ux: np.ndarray, g_uy: np.ndarray,
            precision: str = "f64"):
    """Exact discrete adjoint.  Returns dL/dC (6,) or (6, nx, ny), and dL/dD for MODE_DFIELD."""
    dt = np.float64 if precision == "f64" else np.float32
    fn = getattr(_lib(), f"oracle_adjoint_{precision}")
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_Problem), ctypes.c_void_p, ctypes.c_void_p, real] + \
        [ctypes.c_void_p] * 6
    C, D = _arr(case.C, dt), _arr(case.D, dt)
    rec = _arr(case.rec_idx, np.int32)
    st = _arr(states, dt)
    gx, gy = _arr(g_ux, dt), _arr(g_uy, dt)
    if case.mode == MODE_FIELDS:
        gC = np.zeros((6, case.nx, case.ny), np.float64)
    else:
        gC = np.zeros(6, np.float64)
    gD = np.zeros((case.nx, case.ny), np.float64) if case.mode == MODE_DFIELD else None
    p = case.problem()
    rc = fn(ctypes.byref(p), _ptr(C), _ptr(D), real(case.rho), _ptr(rec), _ptr(st), _ptr(gx),
            _ptr(gy), _ptr(gC), _ptr(gD))
    if rc != 0:
        raise ValueError(f"oracle_adjoint failed with code {rc}")
    return gC, gD


def forward_ckpt(case: Case, k: int, precision: str = "f64"):
    """Forward loop keeping checkpoint pairs every k steps instead of every
    state.  Returns (out_ux, out_uy, ckpt) for adjoint_ckpt."""
    dt = np.float64 if precision == "f64" else np.float32
    fn = getattr(_lib(), f"oracle_forward_ckpt_{precision}")
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_Problem)] + [ctypes.c_void_p] * 6 + [real, ctypes.c_int] + \
        [ctypes.c_void_p] * 3
    C, D = _arr(case.C, dt), _arr(case.D, dt)
    sig, smap = _arr(case.src_signal, dt), _arr(case.src_map, dt)
    org = _arr(case.src_origin, np.int32)
    rec = _arr(case.rec_idx, np.int32)
    out_ux = np.zeros(case.out_shape(), dt)
    out_uy = np.zeros(case.out_shape(), dt)
    nseg = (case.nt + k - 1) // k
    ckpt = np.zeros((nseg, case.nshots, 2, 2, case.nx, case.ny), dt)
    p = case.problem()
    rc = fn(ctypes.byref(p), _ptr(C), _ptr(D), _ptr(sig), _ptr(smap), _ptr(org), _ptr(rec),
            real(case.rho), int(k), _ptr(out_ux), _ptr(out_uy), _ptr(ckpt))
    if rc != 0:
        raise ValueError(f"oracle_forward_ckpt failed with code {rc}")
    return out_ux, out_uy, ckpt


def adjoint_ckpt(case: Case, k: int, ckpt: np.ndarray, g_ux: np.ndarray, g_uy: np.ndarray,
                 precision: str = "f64"):
    """The exact discrete adjoint recomputing each k-step segment from the
    checkpoints of forward_ckpt.  Returns what adjoint() returns."""
    dt = np.float64 if precision == "f64" else np.float32
    fn = getattr(_lib(), f"oracle_adjoint_ckpt_{precision}")
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_Problem)] + [ctypes.c_void_p] * 6 + [real, ctypes.c_int] + \
        [ctypes.c_void_p] * 5
    C, D = _arr(case.C, dt), _arr(case.D, dt)
    sig, smap = _arr(case.src_signal, dt), _arr(case.src_map, dt)
    org = _arr(case.src_origin, np.int32)
    rec = _arr(case.rec_idx, np.int32)
    ck = _arr(ckpt, dt)
    gx, gy = _arr(g_ux, dt), _arr(g_uy, dt)
    if case.mode == MODE_FIELDS:
        gC = np.zeros((6, case.nx, case.ny), np.float64)
    else:
        gC = np.zeros(6, np.float64)
    gD = np.zeros((case.nx, case.ny), np.float64) if case.mode == MODE_DFIELD else None
    p = case.problem()
    rc = fn(ctypes.byref(p), _ptr(C), _ptr(D), _ptr(sig), _ptr(smap), _ptr(org), _ptr(rec),
            real(case.rho), int(k), _ptr(ck), _ptr(gx), _ptr(gy), _ptr(gC), _ptr(gD))
    if rc != 0:
        raise ValueError(f"oracle_adjoint_ckpt failed with code {rc}")
    return gC, gD


def operator(nx, ny, h, C, ux, uy, fx=None, fy=None, rho=1.0, mode=MODE_SCALAR, D=None,
             precision="f64", ref_f32_sum=1):
    """One application of the elastic operator: returns (Lux, Luy) = ((A u + f) / rho)."""
    dt = np.float64 if precision == "f64" else np.float32
    fn = getattr(_lib(), f"oracle_operator_{precision}")
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_Problem)] + [ctypes.c_void_p] * 6 + [real] + [ctypes.c_void_p] * 2
    p = _Problem(1, nx, ny, 1, 1, mode, 0, 0, 1, 0, 0, ref_f32_sum, float(h), 1.0)
    C, D = _arr(C, dt), _arr(D, dt)
    ux, uy, fx, fy = (_arr(a, dt) for a in (ux, uy, fx, fy))
    Lux = np.zeros((nx, ny), dt)
    Luy = np.zeros((nx, ny), dt)
    rc = fn(ctypes.byref(p), _ptr(C), _ptr(D), _ptr(ux), _ptr(uy), _ptr(fx), _ptr(fy), real(rho),
            _ptr(Lux), _ptr(Luy))
    if rc != 0:
        raise ValueError(f"oracle_operator failed with code {rc}")
    return Lux, Luy


def history_grad(pred: np.ndarray, target: np.ndarray, ts: int, ss: int, weight: float = 1.0):
    """d/dpred of weight * mean((pred[:, ::ts, ::ss, ::ss] - target[:, ::ts, ::ss, ::ss])^2),
    the per-component loss of Parameter_inversion/Inversion_adam.py:358-391 (ss=1 and
    weight 5 or 1 give Damage_inversion/Inversion_adam.py:441-450)."""
    g = np.zeros_like(pred, dtype=np.float64)
    sel = pred[:, ::ts, ::ss, ::ss].astype(np.float64)
    tgt = target[:, ::ts, ::ss, ::ss].astype(np.float64)
    n = sel.size
    g[:, ::ts, ::ss, ::ss] = weight * 2.0 * (sel - tgt) / n
    return g
