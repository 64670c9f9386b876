"""ctypes binding of libernn_gb300.so (the C ABI of include/ernn.h).

The library is the only compute path: if it cannot be loaded, every call
raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

MODE_SCALAR, MODE_DFIELD, MODE_FIELDS = 0, 1, 2
RECORD_FIELDS, RECORD_RECEIVERS = 0, 1
PATH_AUTO, PATH_STEP, PATH_RESIDENT, PATH_TILED = 0, 1, 2, 3
FLAG_SHOT_CONSTANTS = 1
FLAG_INSTANCES = 2
FLAG_TALL_TILES = 4

ERRORS = {
    0: "ok", 1: "invalid argument", 2: "workspace too small", 3: "CUDA runtime error",
    4: "unstable time step", 5: "device wait timed out", 6: "unsupported",
}


class ErnnProblem(ctypes.Structure):
    """Mirror of struct ErnnProblem (include/ernn.h)."""
    _fields_ = [
        ("nshots", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("nt", ctypes.c_int32), ("stride", ctypes.c_int32), ("mode", ctypes.c_int32),
        ("record", ctypes.c_int32), ("nrec", ctypes.c_int32), ("src_comp", ctypes.c_int32),
        ("src_bx", ctypes.c_int32), ("src_by", ctypes.c_int32), ("ckpt_k", ctypes.c_int32),
        ("path", ctypes.c_int32), ("flags", ctypes.c_int32),
        ("h", ctypes.c_double), ("dt", ctypes.c_double),
    ]


class ErnnInputs(ctypes.Structure):
    """Mirror of struct ErnnInputs (include/ernn.h); every field is a device pointer."""
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("C", "D", "rho", "src_signal", "src_map", "src_origin", "rec_idx")]


class ErnnInstances(ctypes.Structure):
    """Mirror of struct ErnnInstances (include/ernn.h); the arrays are host int32."""
    _fields_ = [("count", ctypes.c_int32)] + [(n, ctypes.POINTER(ctypes.c_int32)) for n in
                                               ("x0", "y0", "nx", "ny", "nt")]


class ErnnFemProblem(ctypes.Structure):
    """Mirror of struct ErnnFemProblem (include/ernn.h)."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nt", ctypes.c_int32),
                ("stride", ctypes.c_int32), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("dt", ctypes.c_double), ("rho", ctypes.c_double), ("C", ctypes.c_double * 6),
                ("out_scale", ctypes.c_double)]


class ErnnSeries(ctypes.Structure):
    """Mirror of struct ErnnSeries (include/ernn.h)."""
    _fields_ = [("series", ctypes.c_int64), ("frames", ctypes.c_int64), ("nx", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("frame_stride", ctypes.c_int32), ("space_stride", ctypes.c_int32),
                ("wx", ctypes.c_double), ("wy", ctypes.c_double)]


class ErnnAdamTensor(ctypes.Structure):
    """Mirror of struct ErnnAdamTensor (include/ernn.h)."""
    _fields_ = [("param", ctypes.c_void_p), ("grad", ctypes.c_void_p), ("exp_avg", ctypes.c_void_p),
                ("exp_avg_sq", ctypes.c_void_p), ("n", ctypes.c_int64)]


class ErnnAdamHyper(ctypes.Structure):
    """Mirror of struct ErnnAdamHyper (include/ernn.h)."""
    _fields_ = [(n, ctypes.c_double) for n in ("lr", "beta1", "beta2", "eps", "weight_decay")]


# name -> (restype, argtypes); the complete exported surface of include/ernn.h
_P = ctypes.c_void_p
SIGNATURES = {
    "ernn_abi_version": (ctypes.c_int, []),
    "ernn_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "ernn_validate": (ctypes.c_int, [ctypes.POINTER(ErnnProblem)]),
    "ernn_tape_bytes": (ctypes.c_size_t, [ctypes.POINTER(ErnnProblem), ctypes.c_int]),
    "ernn_adjoint_scratch_bytes": (ctypes.c_size_t, [ctypes.POINTER(ErnnProblem)]),
    "ernn_check_stability": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, _P]),
    "ernn_operator": (ctypes.c_int, [ctypes.c_int32] * 4 + [ctypes.c_double] + [_P] * 10),
    "ernn_forward": (ctypes.c_int, [ctypes.POINTER(ErnnProblem), ctypes.POINTER(ErnnInputs),
                                    _P, _P, _P, ctypes.c_size_t, ctypes.c_int, _P]),
    "ernn_forward_instances": (ctypes.c_int, [ctypes.POINTER(ErnnProblem), ctypes.POINTER(ErnnInputs),
                                              ctypes.POINTER(ErnnInstances), _P, _P, _P, ctypes.c_size_t,
                                              ctypes.c_int, _P]),
    "ernn_adjoint_instances": (ctypes.c_int, [ctypes.POINTER(ErnnProblem), ctypes.POINTER(ErnnInputs),
                                              ctypes.POINTER(ErnnInstances), _P, _P, _P, ctypes.c_size_t,
                                              _P, ctypes.c_size_t, _P, _P]),
    "ernn_adjoint": (ctypes.c_int, [ctypes.POINTER(ErnnProblem), ctypes.POINTER(ErnnInputs),
                                    _P, _P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P, _P,
                                    _P]),
    "ernn_forward_static": (ctypes.c_int, [ctypes.POINTER(ErnnProblem), ctypes.POINTER(ErnnInputs),
                                           _P, _P, _P]),
    "ernn_fem_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(ErnnFemProblem)]),
    "ernn_fem_forward": (ctypes.c_int, [ctypes.POINTER(ErnnFemProblem), _P, _P, _P, _P, _P, _P,
                                        ctypes.c_size_t, _P]),
    "ernn_misfit_workspace_bytes": (ctypes.c_size_t, []),
    "ernn_misfit": (ctypes.c_int, [ctypes.POINTER(ErnnSeries), _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "ernn_misfit_grad": (ctypes.c_int, [ctypes.POINTER(ErnnSeries), _P, _P, _P, _P, _P, _P, _P, _P]),
    "ernn_adam_step": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(ErnnAdamHyper), _P, _P]),
    "ernn_launch_count": (ctypes.c_uint64, []),
    "ernn_last_path": (ctypes.c_int32, []),
    "ernn_set_launch_overlap": (ctypes.c_int, [ctypes.c_int]),
    "ernn_device_status": (ctypes.c_int, [ctypes.POINTER(ErnnProblem), ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]),
    "ernn_wait_selftest": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]),
    "ernn_profile_enable": (ctypes.c_int, [ctypes.c_int]),
    "ernn_profile_read": (ctypes.c_int, [_P, _P, _P]),
}


def profile(enable: bool) -> None:
    """Start (True) or stop (False) the library's event timing of its own launches."""
    call("ernn_profile_enable", int(enable))


def launch_overlap(on: bool) -> bool:
    """Turn the launch overlap of consecutive step kernels (programmatic
    dependent launch) on or off; returns the previous setting."""
    return bool(load().ernn_set_launch_overlap(int(bool(on))))


def profile_read():
    """{class: (total_ms, launches, algorithmic_bytes)} for classes 'forward',
    'adjoint', 'other'."""
    ms = (ctypes.c_double * 3)()
    n = (ctypes.c_uint64 * 3)()
    b = (ctypes.c_double * 3)()
    call("ernn_profile_read", ctypes.cast(ms, ctypes.c_void_p), ctypes.cast(n, ctypes.c_void_p),
         ctypes.cast(b, ctypes.c_void_p))
    return {name: (ms[i], int(n[i]), b[i]) for i, name in enumerate(("forward", "adjoint", "other"))}

_LIB = None


class ErnnError(RuntimeError):
    """A library call returned a non-zero status."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with code {code}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the CUDA library, building it in-tree when it is missing or stale."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and _build.is_stale():
        _build.build()
    if not os.path.exists(path):
        raise ImportError(f"libernn_gb300.so not found at {path}; build it with "
                          "__graft_entry__.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.ernn_abi_version() != 1:
        raise ImportError("libernn_gb300.so ABI version mismatch")
    _LIB = lib
    return lib


def check(fn: str, code: int) -> None:
    if code != 0:
        lib = load()
        raise ErnnError(fn, code, lib.ernn_error_string(code).decode())


def call(name: str, *args) -> int:
    lib = load()
    rc = getattr(lib, name)(*args)
    check(name, rc)
    return rc
