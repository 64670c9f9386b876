"""Misfit oracle (test infrastructure only).

ORACLE: the oracle the fused CUDA misfit (ernn_misfit / ernn_misfit_grad)
is compared against; only tests/ import it.  A numpy restatement in FP64 of
  - compute_loss of the parameter inverter
    (Parameter_inversion/Inversion_adam.py:358-391): [:, ::ts, ::ss, ::ss] of
    predictions and of targets (:339-342), mean((p - t)^2) per component,
    summed (weights 1, 1);
  - the data term of the damage inverter's compute_loss
    (Damage_inversion/Inversion_adam.py:441-463): [:, ::ts] of both
    (:420-422), 5 * mean_x + mean_y;
and their gradients to the predictions, 2 w (p - t) / count on the counted
elements and zero elsewhere.  Pinned by tests/golden/misfit.npz (the two
reference methods run on random histories, with autograd gradients).
"""
from __future__ import annotations

import numpy as np


def _select(a: np.ndarray, ts: int, ss: int):
    if a.ndim == 4:
        return (slice(None), slice(None, None, ts), slice(None, None, ss), slice(None, None, ss))
    if ss != 1:
        raise ValueError("a space stride needs (series, frames, nx, ny) arrays")
    return (slice(None), slice(None, None, ts)) + (slice(None),) * (a.ndim - 2)


def misfit(px, py, ox, oy, wx=1.0, wy=1.0, ts=1, ss=1):
    """(loss, mean square x, mean square y, grad_x, grad_y) in FP64."""
    px, py, ox, oy = (np.asarray(a, dtype=np.float64) for a in (px, py, ox, oy))
    sel = _select(px, ts, ss)
    dx = px[sel] - ox[sel]
    dy = py[sel] - oy[sel]
    count = dx.size
    mx = float(np.sum(dx * dx) / count)
    my = float(np.sum(dy * dy) / count)
    gx = np.zeros_like(px)
    gy = np.zeros_like(py)
    gx[sel] = 2.0 * wx * dx / count
    gy[sel] = 2.0 * wy * dy / count
    return wx * mx + wy * my, mx, my, gx, gy
