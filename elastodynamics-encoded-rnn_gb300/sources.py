"""Source signals and spatial loads.

ricker_wavelet and gaussian_point_load restate the reference's source model
(Parameter_inversion/Inversion_adam.py:28-41); tone_burst is the 5-cycle
Hann-windowed burst of the benchmark configurations.  Spatial loads are handed
to the kernels as a small box (origin + dense map) per shot, cropped to the
cells where the load is non-zero.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def ricker_wavelet(t, f0, t0, amplitude=1.0):
    """R(t) = A (1 - 2 pi^2 f0^2 (t - t0)^2) exp(-pi^2 f0^2 (t - t0)^2)
    (Parameter_inversion/Inversion_adam.py:28-35); numpy or torch input."""
    tau = t - t0
    a = (np.pi * f0 * tau) ** 2
    if isinstance(t, torch.Tensor):
        return amplitude * (1 - 2 * a) * torch.exp(-a)
    return amplitude * (1 - 2 * a) * np.exp(-a)


def gaussian_point_load(X, Y, x0, y0, a=150):
    """(a / pi) exp(-a r^2) around (x0, y0) (Parameter_inversion/Inversion_adam.py:38-41)."""
    r2 = (X - x0) ** 2 + (Y - y0) ** 2
    return (a / np.pi) * torch.exp(-a * r2)


def tone_burst(t, f0, cycles=5, amplitude=1.0):
    """Hann-windowed sine burst of `cycles` periods at f0, zero outside [0, cycles/f0]."""
    t = np.asarray(t, dtype=np.float64)
    T = cycles / f0
    w = np.where((t >= 0) & (t <= T), 0.5 * (1 - np.cos(2 * np.pi * t / T)), 0.0)
    return amplitude * w * np.sin(2 * np.pi * f0 * t)


def centered_grid(nx, ny, h, device=None, dtype=None):
    """Cell-centre coordinates on linspace(-L/2, L/2), indexing 'ij'
    (Parameter_inversion/Inversion_adam.py:186-191)."""
    Lx, Ly = h * (nx - 1), h * (ny - 1)
    x = torch.linspace(-Lx / 2, Lx / 2, nx, device=device, dtype=dtype)
    y = torch.linspace(-Ly / 2, Ly / 2, ny, device=device, dtype=dtype)
    return torch.meshgrid(x, y, indexing="ij")


def crop_box(dense: torch.Tensor):
    """Bounding box of the non-zero cells of a (S, nx, ny) load.

    Returns (map (S, bx, by) float32, origin (S, 2) int32) on the input's
    device, one common box size, per-shot origins.  An all-zero load gives a
    1x1 zero box."""
    S, nx, ny = dense.shape
    maps, origins, boxes = [], [], []
    nz = (dense != 0).cpu()
    for s in range(S):
        rows = torch.nonzero(nz[s].any(dim=1)).flatten()
        cols = torch.nonzero(nz[s].any(dim=0)).flatten()
        if rows.numel() == 0:
            boxes.append((0, 0, 1, 1))
        else:
            r0, r1 = int(rows[0]), int(rows[-1]) + 1
            c0, c1 = int(cols[0]), int(cols[-1]) + 1
            boxes.append((r0, c0, r1 - r0, c1 - c0))
    bx = max(b[2] for b in boxes)
    by = max(b[3] for b in boxes)
    for s, (r0, c0, _, _) in enumerate(boxes):
        # keep the common box inside the grid when possible
        r0 = max(0, min(r0, nx - bx))
        c0 = max(0, min(c0, ny - by))
        m = torch.zeros((bx, by), dtype=torch.float32, device=dense.device)
        sub = dense[s, r0:r0 + bx, c0:c0 + by].to(torch.float32)
        m[:sub.shape[0], :sub.shape[1]] = sub
        maps.append(m)
        origins.append((r0, c0))
    return (torch.stack(maps).contiguous(),
            torch.tensor(origins, dtype=torch.int32, device=dense.device))


def point_load_maps(nx, ny, h, positions, gaussian_param, device=None):
    """Gaussian point loads of the reference (float32, as Inversion_adam.py:186-196
    computes them) at physical positions [(x0, y0), ...] on the centred grid."""
    X, Y = centered_grid(nx, ny, h, device=device, dtype=torch.float32)
    return torch.stack([gaussian_point_load(X, Y, x0, y0, gaussian_param)
                        for (x0, y0) in positions])


def cell_position(i, j, nx, ny, h):
    """Physical coordinate of cell (i, j) on the centred grid."""
    return (-h * (nx - 1) / 2 + i * h, -h * (ny - 1) / 2 + j * h)


def signal_times(nt, dt):
    """t_i = i dt (Parameter_inversion/Inversion_adam.py:212)."""
    return np.arange(nt) * dt


def hann_burst_signal(nt, dt, f0=1e6, cycles=5, amplitude=1.0):
    return tone_burst(signal_times(nt, dt), f0, cycles, amplitude)


def courant_number(c_max, rho, h, dt):
    """v_p dt / h with v_p = sqrt(c_max / rho)."""
    return math.sqrt(c_max / rho) * dt / h
