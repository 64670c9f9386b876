"""PyTorch restatement of the reference's propagation path (test/benchmark
infrastructure only, never used by the product).

It performs the same tensor operations, in the same order, as the reference:
per step a float32 force map, the transposed view, zero padding and six 3x3
F.conv2d second differences, the constant-weighted combination, (L + f)/rho
and the leapfrog update, with autograd recording every step
(Parameter_inversion/Inversion_adam.py:44-106 and 240-307).  bench.py times
it on the host cores as the reference's CPU path, and on the GPU as the
reference's autograd path on the same device; tests pin it against the golden
vectors of the reference module.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F


def _stencil_kernels(h, device, dtype):
    inv = h ** (-2)
    base = {
        "xx": [[0.0, 0.0, 0.0], [1.0, -2.0, 1.0], [0.0, 0.0, 0.0]],
        "yy": [[0.0, 1.0, 0.0], [0.0, -2.0, 0.0], [0.0, 1.0, 0.0]],
        "xy": [[0.25, 0.0, -0.25], [0.0, 0.0, 0.0], [-0.25, 0.0, 0.25]],
    }
    return {k: inv * torch.tensor([[v]], device=device, dtype=dtype) for k, v in base.items()}


def _second_differences(u, kern):
    """u: (B, nx, ny) -> dict of (B, ny, nx) second differences on the transposed view."""
    ut = u.transpose(1, 2).unsqueeze(1)
    padded = F.pad(ut, (1, 1, 1, 1), mode="constant", value=0.0)
    return {k: F.conv2d(padded, w, padding=0).squeeze(1) for k, w in kern.items()}


def operator(ux, uy, C, h, fx, fy, rho):
    """((A u + f) / rho) with C = (C11, C22, C12, C16, C26, C66) 0-dim tensors or
    (B, nx, ny) fields."""
    kern = _stencil_kernels(h, ux.device, ux.dtype)
    dx = _second_differences(ux, kern)
    dy = _second_differences(uy, kern)
    C11, C22, C12, C16, C26, C66 = [c.transpose(1, 2) if c.dim() == 3 else c for c in C]
    lx = (C11 * dx["xx"] + C66 * dx["yy"] + (C12 + C66) * dy["xy"] + 2 * C16 * dx["xy"] +
          C16 * dy["xx"] + C26 * dy["yy"])
    ly = (C66 * dy["xx"] + C22 * dy["yy"] + (C12 + C66) * dx["xy"] + C16 * dx["xx"] +
          C26 * dx["yy"] + 2 * C26 * dy["xy"])
    return (lx.transpose(1, 2) + fx) / rho, (ly.transpose(1, 2) + fy) / rho


def propagate(C, rho, nx, ny, nt, h, dt, signal, load, stride=1, rec_idx=None, src_comp=1):
    """Forward loop of one or more shots.

    C: six 0-dim tensors or (1, nx, ny) fields; signal: (S, nt); load: (S, nx, ny)
    dense spatial load; rec_idx: (S, R) flat cells or None for dense history.
    Returns (ux, uy): (S, nt_out, nx, ny) or (S, nt_out, R)."""
    outs_x, outs_y = [], []
    for s in range(signal.shape[0]):
        z = torch.zeros((1, nx, ny), device=load.device, dtype=load.dtype)
        ux1, uy1, ux2, uy2 = z, z, z, z
        hx, hy = [], []
        for i in range(nt):
            f = signal[s, i] * load[s].unsqueeze(0)
            fx, fy = (f, torch.zeros_like(ux1)) if src_comp == 0 else (torch.zeros_like(ux1), f)
            Lx, Ly = operator(ux1, uy1, C, h, fx, fy, rho)
            ux_new = 2 * ux1 - ux2 + dt ** 2 * Lx
            uy_new = 2 * uy1 - uy2 + dt ** 2 * Ly
            ux2, uy2 = ux1, uy1
            ux1, uy1 = ux_new, uy_new
            if i % stride == 0:
                if rec_idx is None:
                    hx.append(ux1)
                    hy.append(uy1)
                else:
                    hx.append(ux1.reshape(-1)[rec_idx[s].long()].unsqueeze(0))
                    hy.append(uy1.reshape(-1)[rec_idx[s].long()].unsqueeze(0))
        outs_x.append(torch.stack(hx, dim=1))
        outs_y.append(torch.stack(hy, dim=1))
    return torch.cat(outs_x, 0), torch.cat(outs_y, 0)
