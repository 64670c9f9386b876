"""Forward-trace and gradient error of a benchmark workload against the FP64
run of the same scheme (test infrastructure: the oracle, never the product).

ORACLE: only tests/, __graft_entry__.smoke() and bench.py's CPU leg use it.

For one workload of the benchmark (its grid, steps, sources, receivers and
constants; optionally fewer steps), the CUDA path computes the receiver
traces at the initial guess and the gradient of the inversion objective
(MSE(ux) + MSE(uy) against the observed traces,
Parameter_inversion/Inversion_adam.py:358-391, differentiated as
loss.backward() at :447).  The C oracle (oracle/ernn_oracle_impl.h) runs the
same scheme in FP64 with checkpoint recomputation, forms its own residual
against the same observations and runs the exact discrete adjoint.
Reported: relative L2 error of the traces, of the gradient of the
normalised constants (or of the degradation map), and per constant; the
relative difference of the residual itself (CUDA against FP64 traces, both
minus the observations); and the gradient error with the FP64 adjoint driven
by the CUDA path's own residual, which separates the adjoint arithmetic from
the residual's sensitivity to FP32 rounding of the forward.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import oracle as O


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_case(geom, C, rho, D=None):
    """The oracle problem of a library Geometry (float32 inputs, in FP64)."""
    f64 = lambda t: t.detach().double().cpu().numpy()
    mode = O.MODE_DFIELD if D is not None else O.MODE_SCALAR
    rec = geom.rec_idx.detach().cpu().numpy().astype(np.int32)
    return O.Case(geom.nx, geom.ny, geom.nt, geom.h, geom.dt, float(rho),
                  np.asarray(C, np.float32).astype(np.float64), f64(geom.src_signal), f64(geom.src_map),
                  geom.src_origin.detach().cpu().numpy().astype(np.int32), stride=geom.stride,
                  mode=mode, record=O.RECORD_RECEIVERS, rec_idx=rec, src_comp=geom.src_comp,
                  D=None if D is None else np.asarray(D, np.float32).astype(np.float64))


def source_distance_mask(w, radius):
    """Cells at least `radius` cells away from every source cell of `w`."""
    i = np.arange(w.nx)[:, None]
    j = np.arange(w.ny)[None, :]
    far = np.ones((w.nx, w.ny), bool)
    for (si, sj) in w.src_cells:
        far &= (i - si) ** 2 + (j - sj) ** 2 >= radius ** 2
    return far


def workload_errors(w, device, nt=None, ckpt_k=None, path=0, oracle_k=None, fp32_floor=False,
                    source_radius=16, C=None):
    """Errors of the CUDA path on workload `w` (scalar constants at the
    seeded initial guess, or the degradation map at D = 0) against FP64.

    nt: steps (default: the workload's own); ckpt_k: the library's checkpoint
    interval (default: the workload's); path: the library's kernel path.
    C: scalar constants to evaluate at (default: the seeded initial guess).
    fp32_floor: also run the oracle in FP32 (FP32 fields and arithmetic, FP64
    sums) and report its gradient error against FP64, the error any FP32
    evaluation of this scheme can be expected to carry.  For the degradation
    map the gradient error is also reported over the cells at least
    `source_radius` cells from every source (near a source the per-cell
    gradient is a sum of large imaging products that cancel, where FP32
    rounding shows most).
    Returns a dict of errors, the kernel path that ran and the oracle's
    wall time."""
    import ernn_gb300 as E
    from ernn_gb300 import harness as Hn

    w.path = path
    if ckpt_k is not None:
        w.ckpt_k = ckpt_k
    geom = Hn.geometry(w, device, nt)
    obs = Hn.observed(w, geom, device)
    rho = torch.tensor(Hn.RHO, device=device)
    damage = w.D_true is not None
    if damage:
        C = torch.tensor(w.C_true, dtype=torch.float32, device=device)
        D = torch.zeros((w.nx, w.ny), device=device, requires_grad=True)
        ux, uy = E.propagate(C, rho, geom, D=D)
    else:
        C0 = Hn.initial_guess(w) if C is None else np.asarray(C, np.float64)
        C = torch.tensor(C0, dtype=torch.float32, device=device, requires_grad=True)
        D = None
        ux, uy = E.propagate(C, rho, geom)
    loss = Hn.trace_misfit(ux, uy, obs[0], obs[1])
    loss.backward()
    torch.cuda.synchronize()
    used = int(E.load_library().ernn_last_path())
    gpu_x, gpu_y = ux.detach().cpu().numpy(), uy.detach().cpu().numpy()
    g_gpu = (D.grad if damage else C.grad).detach().double().cpu().numpy()

    t0 = time.perf_counter()
    case = oracle_case(geom, C.detach().cpu().numpy(), Hn.RHO,
                       None if not damage else np.zeros((w.nx, w.ny)))
    k = oracle_k or max(1, int(round(np.sqrt(2 * geom.nt))))
    px, py, ck = O.forward_ckpt(case, k, "f64")
    ox, oy = (o.detach().double().cpu().numpy() for o in obs)
    count = px.size
    gx, gy = 2.0 * (px - ox) / count, 2.0 * (py - oy) / count
    gC, gD = O.adjoint_ckpt(case, k, ck, gx, gy, "f64")
    # the FP64 adjoint driven by the CUDA path's own adjoint source (its FP32
    # traces against the same observations): compares the adjoint arithmetic
    # alone, without the sensitivity of the residual to the FP32 forward
    sx, sy = 2.0 * (gpu_x.astype(np.float64) - ox) / count, 2.0 * (gpu_y.astype(np.float64) - oy) / count
    sC, sD = O.adjoint_ckpt(case, k, ck, sx, sy, "f64")
    floor = None
    if fp32_floor:
        qx, qy, ck32 = O.forward_ckpt(case, k, "f32")
        del ck
        hx, hy = (2.0 * (q.astype(np.float64) - o) / count for q, o in ((qx, ox), (qy, oy)))
        fC, fD = O.adjoint_ckpt(case, k, ck32, hx, hy, "f32")
        floor = _rel(fD, gD) if damage else _rel(fC * Hn.scales(w.C_true), gC * Hn.scales(w.C_true))
    secs = time.perf_counter() - t0
    out = {"fwd_rel_err": max(_rel(gpu_x, px), _rel(gpu_y, py)),
           "nt": geom.nt, "kernel_path": {1: "step", 2: "resident", 3: "tiled"}.get(used, str(used)),
           "ckpt_k": geom.ckpt_k, "oracle_s": round(secs, 1)}
    if floor is not None:
        out["oracle_fp32_grad_rel_err"] = floor
    out["residual_rel_diff"] = max(_rel(gpu_x - ox, px - ox), _rel(gpu_y - oy, py - oy))
    if damage:
        out["grad_rel_err"] = _rel(g_gpu, gD)
        out["grad_rel_err_same_residual"] = _rel(g_gpu, sD)
        far = source_distance_mask(w, source_radius)
        out["grad_rel_err_away_from_sources"] = _rel(g_gpu[far], gD[far])
        out["source_radius_cells"] = source_radius
    else:
        s = Hn.scales(w.C_true)  # gradient of the normalised constants Adam steps on
        out["grad_rel_err"] = _rel(g_gpu * s, gC * s)
        out["grad_rel_err_same_residual"] = _rel(g_gpu * s, sC * s)
        out["grad_rel_err_per_constant"] = [abs(float(a - b)) / max(abs(float(b)), 1e-300)
                                            for a, b in zip(g_gpu, gC)]
    return out
