"""Seeded problem builders shared by the oracle and the CUDA-path tests."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O

H, DT, RHO = 1e-4, 5e-9, 1560.0
# orthotropic x-z constants of the benchmark configurations rotated 30 degrees
# in-plane (all six non-zero), (C11, C22, C12, C16, C26, C66) order
C_ROT30 = np.array([80.25e9, 21.25e9, 26.25e9, 37.23909236e9, 13.85640646e9, 25.75e9])


def gauss_map(nx, ny, h, x0, y0, a=5e6):
    x = np.linspace(-h * (nx - 1) / 2, h * (nx - 1) / 2, nx, dtype=np.float32)
    y = np.linspace(-h * (ny - 1) / 2, h * (ny - 1) / 2, ny, dtype=np.float32)
    X, Y = np.meshgrid(x, y, indexing="ij")
    return (a / np.pi * np.exp(-a * ((X - x0) ** 2 + (Y - y0) ** 2))).astype(np.float32)


def random_case(nx=33, ny=29, nt=120, stride=3, mode=O.MODE_SCALAR, record=O.RECORD_FIELDS,
                S=1, nrec=7, box=9, seed=0, src_comp=1, dup_receiver=False):
    """A propagation problem with S shots, each with a box load at a random
    position (possibly partly outside the grid) and a random signal."""
    rng = np.random.default_rng(seed)
    f0 = 2e6
    t = np.arange(nt) * DT
    sig = np.stack([np.sin(2 * np.pi * f0 * t + rng.uniform(0, 6)) * np.exp(-((t - 2e-7) / 1.5e-7) ** 2)
                    for _ in range(S)]).astype(np.float32) * 1e10
    g = gauss_map(box, box, H, 0.0, 0.0)
    smap = np.stack([g * rng.uniform(0.5, 1.5) for _ in range(S)]).astype(np.float32)
    org = np.stack([[rng.integers(-box // 2, nx - box // 2), rng.integers(-box // 2, ny - box // 2)]
                    for _ in range(S)]).astype(np.int32)
    rec = None
    if record == O.RECORD_RECEIVERS:
        rec = np.stack([rng.choice(nx * ny, size=nrec, replace=False) for _ in range(S)]).astype(np.int32)
        if dup_receiver:
            rec[:, -1] = rec[:, 0]
    C = C_ROT30.astype(np.float32).astype(np.float64)
    D = None
    if mode == O.MODE_FIELDS:
        C = (C_ROT30[:, None, None] * (1 + 0.15 * rng.random((6, nx, ny)))).astype(np.float32).astype(np.float64)
    if mode == O.MODE_DFIELD:
        D = (0.6 * rng.random((nx, ny))).astype(np.float32).astype(np.float64)
    return O.Case(nx, ny, nt, H, DT, RHO, C, sig.astype(np.float64), smap.astype(np.float64), org,
                  stride=stride, mode=mode, record=record, rec_idx=rec, D=D, src_comp=src_comp)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
