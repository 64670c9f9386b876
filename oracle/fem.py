"""ctypes front end of the FEM generator oracle (test infrastructure only).

ORACLE: the oracle the CUDA FEM kernels are compared against; only tests/
and __graft_entry__.smoke() import it.  The C restatement
(oracle/fem_oracle.c) follows Parameter_inversion/FEM_generate_data.py:117-527;
its parity is pinned by tests/golden/fem*.npz from the reference solver.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .oracle import _lib


class _FemProblem(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nt", ctypes.c_int32),
                ("stride", ctypes.c_int32), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("dt", ctypes.c_double), ("rho", ctypes.c_double), ("C", ctypes.c_double * 6),
                ("out_scale", ctypes.c_double)]


def fem_forward(nx, ny, nt, dx, dy, dt, rho, C, load, signal, stride=1, out_scale=0.7,
                precision="f64", C_fields=None):
    """Frames (nt_out, nx, ny) of both components, frame k = out_scale * u^{k*stride}.
    `load` is the nodal Gaussian as an (nx, ny) array, `signal` the (nt,) time
    factors, `C_fields` None or (6, nx, ny) per-node constants (damaged plate)."""
    real = np.float32 if precision == "f32" else np.float64
    p = _FemProblem(nx, ny, nt, stride, dx, dy, dt, rho, (ctypes.c_double * 6)(*[float(c) for c in C]),
                    out_scale)
    node_load = np.ascontiguousarray(np.asarray(load, dtype=real).T).reshape(-1)  # node j*nx + i
    sig = np.ascontiguousarray(signal, dtype=real)
    nt_out = (nt + stride - 1) // stride
    fx = np.zeros((nt_out, nx, ny), dtype=real)
    fy = np.zeros((nt_out, nx, ny), dtype=real)
    fn = getattr(_lib(), f"oracle_fem_forward_{precision}")
    fn.restype = ctypes.c_int
    cf = None if C_fields is None else np.ascontiguousarray(C_fields, dtype=real)
    fn.argtypes = [ctypes.POINTER(_FemProblem)] + [ctypes.c_void_p] * 5
    rc = fn(ctypes.byref(p), node_load.ctypes.data_as(ctypes.c_void_p), sig.ctypes.data_as(ctypes.c_void_p),
            None if cf is None else cf.ctypes.data_as(ctypes.c_void_p),
            fx.ctypes.data_as(ctypes.c_void_p), fy.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(f"oracle_fem_forward failed ({rc})")
    return fx, fy
