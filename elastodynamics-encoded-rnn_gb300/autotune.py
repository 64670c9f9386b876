"""Measured choice of the kernel path, tile geometry and checkpoint interval.

`choose_ckpt_k` (propagate.py) sizes the checkpoint interval from memory;
ERNN_PATH_AUTO picks the kernel path from static rules (cluster-resident when
the state fits a cluster, tiled when a step has >= 4 tiles per SM, plain
otherwise).  The rules are right for one problem running alone; for problems
that share the GPU with others (the streams of a multi-instance iteration) or
sit near a threshold, `tune` times the candidates instead: every eligible
path — on the tiled path both tile geometries, 64 x 16 and 64 x 32 tiles
(ERNN_FLAG_TALL_TILES) — and, when the tape does not fit, the memory-sized
interval and half of it, on a short forward + adjoint of the same problem
(`probe_steps` steps, the problem's own shots, grid and receivers), and
keeps the fastest.  Results are cached per (device name, grid, shots, steps,
mode, record, per-shot constants) for the process, and optionally in a JSON
file.
"""
from __future__ import annotations

import dataclasses
import json
import os

import torch

from . import _lib
from .propagate import Geometry, choose_ckpt_k, propagate

_CACHE: dict = {}


def _key(geom: Geometry, C: torch.Tensor, D, device) -> str:
    mode = "dfield" if D is not None else ("fields" if C.dim() == 3 else
                                           ("shots" if C.dim() == 2 else "scalar"))
    return json.dumps([torch.cuda.get_device_name(device), geom.nx, geom.ny, geom.nshots, geom.nt,
                       geom.stride, mode, geom.record, geom.ckpt_k])


def _time(geom: Geometry, C, rho, D, steps: int, reps: int) -> float:
    g = dataclasses.replace(geom, nt=steps, src_signal=geom.src_signal[:, :steps].contiguous(),
                            _checked=False)
    Cv = C.detach().clone().requires_grad_(D is None)
    Dv = None if D is None else D.detach().clone().requires_grad_(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps + 1)]
    for r in range(reps + 1):
        ev[r][0].record()
        ux, uy = propagate(Cv, rho, g, D=Dv)
        (ux.double().square().sum() + uy.double().square().sum()).backward()
        ev[r][1].record()
    torch.cuda.synchronize()
    return min(a.elapsed_time(b) for a, b in ev[1:])


def tune(geom: Geometry, C: torch.Tensor, rho: torch.Tensor, D=None, probe_steps: int = 96,
         reps: int = 2, cache_file: str | None = None) -> tuple[int, int, int]:
    """(path, ckpt_k, tile_rows) for this problem, measured; sets none of them
    on `geom`.  A checkpoint interval already set on `geom` is kept.
    tile_rows: 32 for 64 x 32 tiles on the tiled path, else 16."""
    dev = C.device
    key = _key(geom, C, D, dev)
    if key not in _CACHE and cache_file and os.path.exists(cache_file):
        with open(cache_file) as f:
            _CACHE.update(json.load(f))
    if key in _CACHE:
        return tuple(_CACHE[key])
    mode = 1 if D is not None else (2 if C.dim() == 3 else 0)
    flags = _lib.FLAG_SHOT_CONSTANTS if (D is None and C.dim() == 2) else 0
    steps = max(2, min(probe_steps, geom.nt))
    if geom.ckpt_k is not None:  # an interval the caller fixed is kept
        ks = [geom.ckpt_k]
    else:
        # intervals within the same memory budget: the memory-sized one and
        # half of it (a larger one would not leave room for a captured
        # graph's own workspace pool)
        k_mem = choose_ckpt_k(geom, mode, dev, flags=flags)
        ks = [k_mem] if k_mem >= geom.nt else sorted({max(1, k_mem // 2), k_mem})
    best = None
    for path in (_lib.PATH_RESIDENT, _lib.PATH_TILED, _lib.PATH_STEP):
        rows = (16, 32) if path == _lib.PATH_TILED else (16,)
        eligible = True
        for tr in rows:
            for k in ks:
                # the probe keeps the interval's ratio to the step count
                k_probe = max(1, min(steps, round(k * steps / geom.nt)))
                g = dataclasses.replace(geom, path=path, ckpt_k=k_probe, tile_rows=tr, _checked=False)
                try:
                    ms = _time(g, C, rho, D, steps, reps)
                except _lib.ErnnError as e:
                    if e.code == 6:  # ERNN_ERR_UNSUPPORTED: path not eligible
                        eligible = False
                        break
                    raise
                if best is None or ms < best[0]:
                    best = (ms, path, k, tr)
            if not eligible:
                break
    _CACHE[key] = (best[1], best[2], best[3])
    if cache_file:
        with open(cache_file, "w") as f:
            json.dump(_CACHE, f)
    return tuple(_CACHE[key])
