"""Elastic constants in the 2D plane: in-plane rotation and the stability check.

Constants are ordered (C11, C22, C12, C16, C26, C66) in the reference's x-y
naming.  The x-z names of the benchmark configurations map one to one:
C11 -> C11, C33 -> C22, C13 -> C12, C15 -> C16, C35 -> C26, C55 -> C66.
"""
from __future__ import annotations

import ctypes

from . import _lib
from .configs import from_voigt, orthotropic_xz, rotate, stability_number, voigt_matrix  # noqa: F401

ORDER = ("C11", "C22", "C12", "C16", "C26", "C66")
XZ_NAMES = ("C11", "C33", "C13", "C15", "C35", "C55")


def check_stability(c6, rho, h, dt):
    """Return the stability number of the leapfrog scheme (stable when <= 1);
    raises ValueError above 1 or for an indefinite material."""
    lib = _lib.load()
    arr = (ctypes.c_double * 6)(*[float(v) for v in c6])
    out = ctypes.c_double(0.0)
    rc = lib.ernn_check_stability(ctypes.cast(arr, ctypes.c_void_p), float(rho), float(h),
                                  float(dt), ctypes.cast(ctypes.pointer(out), ctypes.c_void_p))
    if rc == 4:
        raise ValueError(f"time step unstable for these constants (stability number {out.value:.3f})")
    _lib.check("ernn_check_stability", rc)
    return out.value
