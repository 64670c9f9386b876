"""Elastic constants in the 2D plane: in-plane rotation and the stability check.

Constants are ordered (C11, C22, C12, C16, C26, C66) in the reference's x-y
naming.  The x-z names of the benchmark configurations map one to one:
C11 -> C11, C33 -> C22, C13 -> C12, C15 -> C16, C35 -> C26, C55 -> C66.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

ORDER = ("C11", "C22", "C12", "C16", "C26", "C66")
XZ_NAMES = ("C11", "C33", "C13", "C15", "C35", "C55")

# Voigt index of the symmetric pair (a, b) in 2D: xx -> 0 (1), yy -> 1 (2), xy -> 2 (6)
_V = {(0, 0): 0, (1, 1): 1, (0, 1): 2, (1, 0): 2}


def voigt_matrix(c6):
    """3x3 Voigt matrix [[C11, C12, C16], [C12, C22, C26], [C16, C26, C66]]."""
    C11, C22, C12, C16, C26, C66 = (float(v) for v in c6)
    return np.array([[C11, C12, C16], [C12, C22, C26], [C16, C26, C66]])


def from_voigt(M):
    return np.array([M[0, 0], M[1, 1], M[0, 1], M[0, 2], M[1, 2], M[2, 2]])


def rotate(c6, theta_deg):
    """Constants of the material rotated by theta in the plane (tensor rotation
    C'_ijkl = R_ia R_jb R_kc R_ld C_abcd)."""
    M = voigt_matrix(c6)
    C = np.zeros((2, 2, 2, 2))
    for i in range(2):
        for j in range(2):
            for k in range(2):
                for l in range(2):
                    C[i, j, k, l] = M[_V[(i, j)], _V[(k, l)]]
    t = np.deg2rad(theta_deg)
    R = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
    Cr = np.einsum("ia,jb,kc,ld,abcd->ijkl", R, R, R, R, C)
    Mr = np.zeros((3, 3))
    for (i, j), p in _V.items():
        for (k, l), q in _V.items():
            Mr[p, q] = Cr[i, j, k, l]
    return from_voigt(Mr)


def orthotropic_xz(C11, C33, C13, C55, C15=0.0, C35=0.0):
    """x-z constants of the benchmark configurations, returned in (C11, C22, C12, C16, C26, C66) order."""
    return np.array([C11, C33, C13, C15, C35, C55], dtype=np.float64)


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
