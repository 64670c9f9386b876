"""FusedAdam: torch.optim.Adam's update for every parameter of a group in one
launch of libernn_gb300.so (ernn_adam_step), the optimiser of the inversion
loops (Parameter_inversion/Inversion_adam.py:421-447,
Damage_inversion/Inversion_adam.py:477-514).

Same constructor arguments and update as torch.optim.Adam without amsgrad
(lr, betas, eps, weight_decay).  The step count is kept on the device, so a
CUDA graph that captured `step()` advances it on every replay; the launch
table (parameter, gradient and moment pointers) is built on the first step
and rebuilt only when a gradient tensor is replaced (zero_grad with
set_to_none=False keeps them), so capture after one warm-up step.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


class FusedAdam(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=0.0):
        if lr < 0 or eps < 0 or weight_decay < 0 or not (0 <= betas[0] < 1 and 0 <= betas[1] < 1):
            raise ValueError("invalid Adam hyper-parameters")
        super().__init__(params, dict(lr=lr, betas=tuple(betas), eps=eps, weight_decay=weight_decay))
        self._launch = {}  # group index -> (pointer key, device table, device step state, numel max)

    def _table(self, k, params):
        key = tuple((p.data_ptr(), p.grad.data_ptr()) for p in params)
        cached = self._launch.get(k)
        if cached is not None and cached[0] == key:
            return cached
        dev = params[0].device
        descs = []
        for p in params:
            st = self.state[p]
            if "exp_avg" not in st:
                st["exp_avg"] = torch.zeros_like(p, memory_format=torch.contiguous_format)
                st["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.contiguous_format)
            descs.append(_lib.ErnnAdamTensor(p.data_ptr(), p.grad.data_ptr(), st["exp_avg"].data_ptr(),
                                              st["exp_avg_sq"].data_ptr(), p.numel()))
        arr = (_lib.ErnnAdamTensor * len(descs))(*descs)
        table = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
        steps = cached[2] if cached is not None else torch.zeros(2, dtype=torch.int32, device=dev)
        entry = (key, table, steps, max(p.numel() for p in params))
        self._launch[k] = entry
        return entry

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        lib = _lib.load()
        for k, group in enumerate(self.param_groups):
            params = [p for p in group["params"] if p.grad is not None]
            if not params:
                continue
            for p in params:
                if not p.is_cuda:
                    raise RuntimeError("FusedAdam runs only on CUDA parameters through libernn_gb300.so")
                if p.dtype != torch.float32 or p.grad.dtype != torch.float32 or not p.is_contiguous() \
                        or not p.grad.is_contiguous() or p.grad.is_sparse:
                    raise ValueError("FusedAdam needs contiguous float32 parameters and dense gradients")
                if p.device != params[0].device:
                    raise ValueError("one device per parameter group")
            _, table, steps, nmax = self._table(k, params)
            b1, b2 = group["betas"]
            h = _lib.ErnnAdamHyper(float(group["lr"]), float(b1), float(b2), float(group["eps"]),
                                   float(group["weight_decay"]))
            dev = params[0].device
            stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            with torch.cuda.device(dev):
                _lib.check("ernn_adam_step", lib.ernn_adam_step(
                    ctypes.c_void_p(table.data_ptr()), len(params), nmax, ctypes.byref(h),
                    ctypes.c_void_p(steps.data_ptr()), stream))
        return loss

    def step_count(self, group: int = 0) -> torch.Tensor:
        """The device step counter of a parameter group (0-dim int32 view)."""
        return self._launch[group][2][0]
