"""The misfit of an inversion iteration on the device: predicted against
observed traces or histories, loss in FP64 and its gradient (the adjoint
source of the hand adjoint), each one fused pass of libernn_gb300.so.

`series_misfit(px, py, ox, oy, wx, wy, frame_stride, space_stride)` is
    wx * mean((px - ox)^2) + wy * mean((py - oy)^2)
over [:, ::frame_stride, ::space_stride, ::space_stride] of both: compute_loss
of Parameter_inversion/Inversion_adam.py:358-391 with wx = wy = 1 (targets
subsampled the same way, :339-342), and the 5:1 data term of
Damage_inversion/Inversion_adam.py:441-463 on every secondary_time_stride-th
frame (:420-422) with wx = 5, wy = 1.
Differences in FP32 as the reference forms them, sums in FP64 in a fixed
order (bitwise reproducible, graph-capturable: no host synchronisation).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def _series(px: torch.Tensor, frame_stride: int, space_stride: int, wx: float, wy: float) -> _lib.ErnnSeries:
    if px.dim() < 2 or px.dim() > 4:
        raise ValueError("series tensors are (series, frames), (series, frames, n) or "
                         "(series, frames, nx, ny)")
    grid = [int(d) for d in px.shape[2:]]
    nx, ny = ([1, 1] + grid)[-2:]
    if space_stride != 1 and px.dim() != 4:
        raise ValueError("a space stride needs (series, frames, nx, ny) tensors")
    if frame_stride < 1 or space_stride < 1:
        raise ValueError("strides must be >= 1")
    return _lib.ErnnSeries(int(px.shape[0]), int(px.shape[1]), nx, ny, int(frame_stride),
                           int(space_stride), float(wx), float(wy))


def _check(*ts):
    ref = ts[0]
    for t in ts:
        if not t.is_cuda:
            raise RuntimeError("series_misfit runs only on CUDA tensors through libernn_gb300.so")
        if t.dtype != torch.float32 or tuple(t.shape) != tuple(ref.shape) or t.device != ref.device:
            raise ValueError("predicted and observed series must be float32 tensors of one shape "
                             "on one device")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class SeriesMisfit(torch.autograd.Function):
    """(loss, mean square x, mean square y) as a (3,) float64 tensor, of
    predicted (px, py) against observed (ox, oy); differentiable in px, py."""

    @staticmethod
    def forward(ctx, px, py, ox, oy, wx, wy, frame_stride, space_stride):
        s = _series(px, frame_stride, space_stride, wx, wy)  # layout first: host-side checks
        px, py, ox, oy = (t.contiguous() for t in (px, py, ox, oy))
        _check(px, py, ox, oy)
        lib = _lib.load()
        dev = px.device
        with torch.cuda.device(dev):
            out = torch.empty(3, dtype=torch.float64, device=dev)
            nbytes = lib.ernn_misfit_workspace_bytes()
            ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            _lib.check("ernn_misfit", lib.ernn_misfit(ctypes.byref(s), _ptr(px), _ptr(py), _ptr(ox), _ptr(oy),
                                                      _ptr(out), _ptr(ws), ctypes.c_size_t(nbytes), stream))
        ctx.save_for_backward(px, py, ox, oy)
        ctx.series = s
        return out

    @staticmethod
    def backward(ctx, g):
        px, py, ox, oy = ctx.saved_tensors
        dev = px.device
        with torch.cuda.device(dev):
            g = g.detach().to(torch.float64).contiguous()
            gx = torch.empty_like(px)
            gy = torch.empty_like(py)
            stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            lib = _lib.load()
            _lib.check("ernn_misfit_grad", lib.ernn_misfit_grad(ctypes.byref(ctx.series), _ptr(px), _ptr(py),
                                                                _ptr(ox), _ptr(oy), _ptr(g), _ptr(gx),
                                                                _ptr(gy), stream))
        return gx, gy, None, None, None, None, None, None


def series_misfit(px, py, ox, oy, wx: float = 1.0, wy: float = 1.0, frame_stride: int = 1,
                  space_stride: int = 1, parts: bool = False):
    """wx * mean((px - ox)^2) + wy * mean((py - oy)^2) over frames 0,
    frame_stride, ... (dim 1) and, for (series, frames, nx, ny) tensors, the
    cells of both grid axes at multiples of space_stride: float32 CUDA
    tensors in, a 0-dim float64 tensor out, differentiable in px and py.
    With parts=True also the two mean squares (a (2,) float64 tensor)."""
    out = SeriesMisfit.apply(px, py, ox.detach(), oy.detach(), wx, wy, frame_stride, space_stride)
    return (out[0], out[1:]) if parts else out[0]
