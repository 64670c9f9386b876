"""The inversion iteration built on the CUDA path, over the benchmark
configurations of `configs` (re-exported here).

One inversion iteration = forward (receiver traces) -> FP64 misfit ->
hand adjoint -> Adam step on normalised constants.  Observations: the same
forward at the true constants plus Gaussian noise of 0.5 % of the trace RMS.
"""
from __future__ import annotations

import numpy as np
import torch

from . import sources
from .configs import (C_ORTHO, DT, FIELDS301, H, RHO, WORKLOADS, Workload, _top,  # noqa: F401
                      damage512, damage_map, fields301, initial_guess, multi_instances, plate128,
                      rot256, scales, shots1024)
from .misfit import series_misfit
from .optim import FusedAdam
from .propagate import Geometry, check_device_status, propagate


def geometry(w: Workload, device, nt=None) -> Geometry:
    nt = w.nt if nt is None else nt
    sig = sources.hann_burst_signal(nt, DT, w.f0, 5, w.amplitude).astype(np.float32)
    S = w.nshots
    pos = [sources.cell_position(i, j, w.nx, w.ny, H) for (i, j) in w.src_cells]
    # the load of each shot only matters where it is non-zero: build it on a
    # window around the source cell and crop
    dense = sources.point_load_maps(w.nx, w.ny, H, pos, w.gaussian_param, device=device)
    smap, origin = sources.crop_box(dense)
    rec = torch.tensor([[i * w.ny + j for (i, j) in w.rec_cells]] * S, dtype=torch.int32, device=device)
    return Geometry(nx=w.nx, ny=w.ny, nt=nt, h=H, dt=DT,
                    src_signal=torch.tensor(np.repeat(sig[None], S, 0), device=device),
                    src_map=smap, src_origin=origin, stride=w.stride, src_comp=1, rec_idx=rec,
                    ckpt_k=w.ckpt_k, path=w.path)


def observed(w: Workload, geom: Geometry, device, noise=0.005, seed=0):
    """Traces at the true constants plus seeded Gaussian noise of `noise` x RMS
    (0.5 % ~ add_noise_snr at 46 dB, Parameter_inversion/Inversion_adam.py:109-129)."""
    rho = torch.tensor(RHO, device=device)
    C = torch.tensor(w.C_true, dtype=torch.float32, device=device)
    with torch.no_grad():
        if w.D_true is not None:
            ox, oy = propagate(C, rho, geom, D=torch.tensor(w.D_true, dtype=torch.float32, device=device))
        else:
            ox, oy = propagate(C, rho, geom)
    g = torch.Generator(device=device).manual_seed(seed)
    out = []
    for o in (ox, oy):
        rms = o.double().pow(2).mean().sqrt().float()
        out.append(o + noise * rms * torch.randn(o.shape, generator=g, device=device))
    return out


def trace_misfit(pred_x, pred_y, obs_x, obs_y):
    """MSE(ux) + MSE(uy) (the loss of Parameter_inversion/Inversion_adam.py:389-391)
    of (S, nt_out, nrec) traces, summed in FP64: one fused pass of the library,
    whose gradient (the adjoint source) is a second one."""
    return series_misfit(pred_x, pred_y, obs_x, obs_y)


class NormalisedConstants(torch.nn.Module):
    """C_t = s_t * theta_t with theta trained by Adam; s_t is a fixed per-constant
    scale (the constant's magnitude, or 5 % of C11 for constants that are zero)."""

    def __init__(self, C_init, C_scale):
        super().__init__()
        self.register_buffer("scale", torch.tensor(np.asarray(C_scale, np.float32)))
        self.theta = torch.nn.Parameter(torch.tensor(np.asarray(C_init) / np.asarray(C_scale),
                                                     dtype=torch.float32))

    def forward(self):
        return self.theta * self.scale


class _GraphedIteration:
    """CUDA-graph replay of an inversion iteration: `capture()` warms the
    iteration up on a side stream (allocator pools, library caches, the
    checkpoint choice), then records one iteration — the library's time
    loops, the misfit, the adjoint and the optimiser step — as one graph;
    `step(obs)` copies new observations (host tensors, pinned for an
    asynchronous copy, or device tensors) into the captured input tensors and
    replays it.  `step_eager()` runs the same iteration without the graph."""

    graph = None
    _loss = None

    def capture(self):
        dev = self.device
        if isinstance(self.opt, torch.optim.Adam):  # optimiser state kept on the device
            for group in self.opt.param_groups:
                group["capturable"] = True
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(2):
                self.step_eager()
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        check_device_status()
        # the graph allocates from its own pool: hand the warm-up iterations'
        # cached blocks back first, so no allocation during capture has to
        # free memory (not allowed while capturing)
        torch.cuda.empty_cache()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._loss = self.step_eager()
        return self

    def step(self, obs=None):
        if obs is not None:
            for dst, src in zip(self.obs, obs):
                if dst.data_ptr() != src.data_ptr():
                    dst.copy_(src, non_blocking=True)
        if self.graph is None:
            return self.step_eager()
        self.graph.replay()
        return self._loss


class Inversion(_GraphedIteration):
    """One inversion iteration of the scalar-constant workloads."""

    def __init__(self, w: Workload, device, lr=1e-2, seed=0, nt=None, graph=False):
        self.w = w
        self.device = device
        self.geom = geometry(w, device, nt)
        self.obs = observed(w, self.geom, device, seed=seed)
        self.rho = torch.tensor(RHO, device=device)
        self.params = NormalisedConstants(initial_guess(w, seed), scales(w.C_true)).to(device)
        self.opt = FusedAdam(self.params.parameters(), lr=lr)
        if graph:
            self.capture()

    def step_eager(self):
        obs = self.obs
        self.opt.zero_grad(set_to_none=False)
        ux, uy = propagate(self.params(), self.rho, self.geom)
        loss = trace_misfit(ux, uy, obs[0], obs[1])
        loss.backward()
        self.opt.step()
        return loss

    def forward_only(self):
        with torch.no_grad():
            return propagate(self.params().detach(), self.rho, self.geom)

    def gradient(self):
        return self.params.theta.grad

    def constants(self):
        return self.params().detach().double().cpu().numpy()

    def relative_errors(self):
        C, T = self.constants(), self.w.C_true
        sc = scales(T)
        return np.abs(C - T) / sc


class DamageInversion(_GraphedIteration):
    """One inversion iteration of the degradation-map workload: D(x) trained by
    Adam with C(x) = (1 - D(x)) C0 (initial guess D = 0).

    The objective is the trace MSE divided by its value at the initial guess
    (a fixed factor, one pass of the same fused misfit).  The plain MSE of
    these displacements is about 1e-11 and its gradient per cell about
    1e-13, far below Adam's eps = 1e-8: Adam would then move D by a few
    millionths of lr per step.  Normalised, the objective starts at 1 and
    the steps are of order lr, as for the scalar constants."""

    def __init__(self, w: Workload, device, lr=1e-2, seed=0, nt=None, graph=False):
        if w.D_true is None:
            raise ValueError("workload has no degradation map")
        self.w = w
        self.device = device
        self.geom = geometry(w, device, nt)
        self.obs = observed(w, self.geom, device, seed=seed)
        self.rho = torch.tensor(RHO, device=device)
        self.C0 = torch.tensor(w.C_true, dtype=torch.float32, device=device)
        self.D = torch.nn.Parameter(torch.zeros((w.nx, w.ny), device=device))
        self.opt = FusedAdam([self.D], lr=lr)
        with torch.no_grad():
            ux, uy = propagate(self.C0, self.rho, self.geom, D=self.D.detach())
            self.loss_scale = float(1.0 / trace_misfit(ux, uy, self.obs[0], self.obs[1]))
        if graph:
            self.capture()

    def step_eager(self):
        obs = self.obs
        self.opt.zero_grad(set_to_none=False)
        ux, uy = propagate(self.C0, self.rho, self.geom, D=self.D)
        loss = series_misfit(ux, uy, obs[0], obs[1], self.loss_scale, self.loss_scale)
        loss.backward()
        self.opt.step()
        return loss

    def forward_only(self):
        with torch.no_grad():
            return propagate(self.C0, self.rho, self.geom, D=self.D.detach())

    def gradient(self):
        return self.D.grad


class FieldsInversion(_GraphedIteration):
    """One iteration of the reference's damage loop on the drop-in simulator:
    six per-cell log-constant fields, the 5:1 misfit on every 2nd frame of the
    dense history plus the TV term, Adam.  The observations are the forward
    of the same simulator with the constants halved inside a 2 cm circle
    (the damaged-plate generator's default region) plus 0.5 % noise."""

    def __init__(self, w: Workload, device, lr=None, seed=0, nt=None, graph=False):
        from .simulators import SpatiallyVaryingAnisotropicSimulator, damage_loss
        c = FIELDS301
        self.w = w
        self.device = device
        nt = w.nt if nt is None else nt
        h = c["L"] / (w.nx - 1)
        C0 = dict(zip(("C11_init", "C22_init", "C12_init", "C16_init", "C26_init", "C66_init"), c["C0"]))
        make = lambda: SpatiallyVaryingAnisotropicSimulator(
            (w.nx, w.ny), h, c["total_time"] / (c["nt"] - 1), nt, w.stride, source_f0=c["f0"],
            source_t0=c["t0"], source_amplitude=c["amplitude"], total_time=c["total_time"],
            rho_known=c["rho"], gaussian_param=c["gaussian_param"], **C0).to(device)
        self.loss_fn = damage_loss
        true = make()
        x = (torch.arange(w.nx, device=device) - (w.nx - 1) / 2) * h
        X, Y = torch.meshgrid(x, x, indexing="ij")
        damaged = (((X - 0.1) ** 2 + (Y - 0.1) ** 2).sqrt() <= 0.02)[None]
        with torch.no_grad():
            for n in ("log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66"):
                getattr(true, n).add_(damaged * float(np.log(0.5)))
            tx, ty = true()
            g = torch.Generator(device=device).manual_seed(seed)
            tx = tx + 0.005 * tx.std() * torch.randn(tx.shape, generator=g, device=device)
            ty = ty + 0.005 * ty.std() * torch.randn(ty.shape, generator=g, device=device)
        del true
        self.sim = make()
        from .propagate import MODE_FIELDS, choose_ckpt_k
        self.sim.ckpt_k = choose_ckpt_k(self.sim.geometry(), MODE_FIELDS, device)  # fixed before any capture
        self.obs = (tx.contiguous(), ty.contiguous())
        self.opt = torch.optim.Adam(self.sim.parameters(), lr=c["lr"] if lr is None else lr,
                                    capturable=graph)
        self._start = [p.detach().clone() for p in self.sim.parameters()]
        if graph:
            self.capture()

    def restart(self):
        """Back to the initial guess with a fresh optimiser state, in place (a
        captured graph keeps its tensors).  On this synthetic target the loop's
        12th Adam step leaves the first cells with a stiffness that is not
        positive-definite (the reference's loop does the same), and a few
        iterations later the wavefield overflows."""
        with torch.no_grad():
            for p, p0 in zip(self.sim.parameters(), self._start):
                p.copy_(p0)
            for st in self.opt.state.values():
                for k in ("exp_avg", "exp_avg_sq"):
                    if k in st:
                        st[k].zero_()
                if torch.is_tensor(st.get("step")):
                    st["step"].zero_()
                elif "step" in st:
                    st["step"] = 0

    @property
    def geom(self):
        return self.sim.geometry()

    def step_eager(self):
        obs = self.obs
        self.opt.zero_grad(set_to_none=False)
        ux, uy = self.sim()
        loss, _, _ = self.loss_fn(self.sim, ux, uy, obs[0], obs[1], FIELDS301["ts"], FIELDS301["lambda_tv"])
        loss.backward()
        self.opt.step()
        return loss

    def forward_only(self):
        with torch.no_grad():
            return self.sim()

    def gradient(self):
        return torch.cat([p.grad.reshape(-1) for p in self.sim.parameters()])


def make_inversion(w: Workload, device, **kw):
    """The inversion iteration matching the workload (constants, degradation
    map, or six constant fields)."""
    if w.extra.get("fields"):
        return FieldsInversion(w, device, **kw)
    return DamageInversion(w, device, **kw) if w.D_true is not None else Inversion(w, device, **kw)


def run_inversion(w: Workload, device, iters=200, lr=1e-2, seed=0):
    """Adam on normalised constants for `iters` iterations; returns the final
    constants, their errors relative to each constant's scale, and the loss history."""
    inv = Inversion(w, device, lr=lr, seed=seed)
    losses = []
    for _ in range(iters):
        losses.append(inv.step())
    losses = [float(v) for v in torch.stack(losses).cpu()]
    return inv.constants(), inv.relative_errors(), losses


class _InstanceGroup:
    """Instances of one grid size, step count and acquisition geometry, run as
    the shots of one propagation with per-shot constants: each keeps its own
    constants, density, observations and gradient."""

    def __init__(self, invs, device, budget_fraction, tuned=False):
        from .propagate import choose_ckpt_k
        from ._lib import FLAG_SHOT_CONSTANTS
        self.invs = invs
        g0 = invs[0].geom
        S = len(invs)
        rep = lambda t: t.repeat((S,) + (1,) * (t.dim() - 1)).contiguous()
        self.geom = Geometry(nx=g0.nx, ny=g0.ny, nt=g0.nt, h=g0.h, dt=g0.dt,
                             src_signal=rep(g0.src_signal), src_map=rep(g0.src_map),
                             src_origin=rep(g0.src_origin), stride=g0.stride, src_comp=g0.src_comp,
                             rec_idx=rep(g0.rec_idx), path=g0.path)
        self.geom.ckpt_k = choose_ckpt_k(self.geom, 0, device, budget_fraction=budget_fraction,
                                         flags=FLAG_SHOT_CONSTANTS if S > 1 else 0)
        self.obs = [torch.cat([inv.obs[c] for inv in invs]).contiguous() for c in (0, 1)]
        self.rho = torch.full((S,), RHO, dtype=torch.float32, device=device)
        if tuned:  # measured kernel path at the memory-sized interval (autotune keeps a fixed one)
            from . import autotune
            C = torch.stack([inv.params() for inv in invs]).detach() if S > 1 else invs[0].params().detach()
            self.geom.path, self.geom.ckpt_k, self.geom.tile_rows = autotune.tune(
                self.geom, C, self.rho if S > 1 else self.rho[0])

    def loss(self):
        if len(self.invs) == 1:
            ux, uy = propagate(self.invs[0].params(), self.rho[0], self.geom)
            return trace_misfit(ux, uy, self.obs[0], self.obs[1])
        C = torch.stack([inv.params() for inv in self.invs])
        ux, uy = propagate(C, self.rho, self.geom)
        # the sum of each instance's own misfit: the instances share frames and
        # receivers, so it is S times the mean over the group (one fused pass)
        S = len(self.invs)
        return series_misfit(ux, uy, self.obs[0], self.obs[1], float(S), float(S))


class MultiInversion:
    """Many independent scalar-constant inversions advanced as one iteration:
    instances with the same grid size and step count run together as the
    shots of one propagation with per-shot constants (their own constants,
    densities and gradients), the groups on `nstreams` CUDA streams, one Adam
    step updates every instance, and the whole iteration is captured once in
    a CUDA graph and replayed (`step`).  group=False runs every instance on
    its own."""

    def __init__(self, ws, device, lr=1e-2, seed=0, nstreams=8, graph=True, group=True, path=None,
                 serial_big=False, tuned=False):
        self.ws = ws
        self.device = device
        if path is not None:
            for w in ws:
                w.path = path
        self.invs = [Inversion(w, device, lr=lr, seed=seed + k) for k, w in enumerate(ws)]
        keyed = {}
        for k, (w, inv) in enumerate(zip(ws, self.invs)):
            key = (w.nx, w.ny, inv.geom.nt, w.stride, tuple(w.src_cells), tuple(w.rec_cells), w.f0,
                   w.amplitude, w.gaussian_param, w.path) if group else k
            keyed.setdefault(key, []).append(inv)
        # largest work first: the longest groups start earliest on the streams
        members = sorted(keyed.values(), key=lambda g: -sum(i.w.cell_steps for i in g))
        self.groups = [_InstanceGroup(g, device, 0.4 * len(g) / len(ws), tuned=tuned) for g in members]
        # streams: round robin over the groups, or (serial_big) groups large
        # enough for the tiled kernels one after another on the first stream
        # and the smaller ones on the others
        sms = torch.cuda.get_device_properties(device).multi_processor_count
        big = lambda g: g.geom.nshots * -(-g.geom.nx // 32) * -(-g.geom.ny // 64) >= 4 * sms
        nsmall = max(1, nstreams - 1)
        small = 0
        self.stream_of = []
        for k, g in enumerate(self.groups):
            if not serial_big:
                self.stream_of.append(k % nstreams)
            elif big(g) or nstreams == 1:
                self.stream_of.append(0)
            else:
                self.stream_of.append(1 + small % nsmall)
                small += 1
        params = [inv.params.theta for inv in self.invs]
        self.opt = FusedAdam(params, lr=lr)  # one launch for every instance's constants
        self.streams = [torch.cuda.Stream(device) for _ in range(nstreams)]
        self.obs = [o for g in self.groups for o in g.obs]
        self.cell_steps = sum(w.cell_steps for w in ws)
        self.graph = None
        self.loss = None
        if graph:
            self._capture()

    def _eager_step(self):
        self.opt.zero_grad(set_to_none=False)
        main = torch.cuda.current_stream(self.device)
        losses = []
        used = sorted(set(self.stream_of))
        for k in used:
            self.streams[k].wait_stream(main)
        for k, grp in enumerate(self.groups):
            s = self.streams[self.stream_of[k]]
            with torch.cuda.stream(s):
                lk = grp.loss()
                lk.backward()
            losses.append(lk)
        for k in used:  # the streams that got work (joined a capture)
            main.wait_stream(self.streams[k])
        self.opt.step()
        return torch.stack([l.detach() for l in losses]).sum()

    def _capture(self):
        # warm up on a side stream (allocator pools, autograd, library caches)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(2):
                self._eager_step()
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        check_device_status()
        torch.cuda.empty_cache()  # the graph's own pool allocates next
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.loss = self._eager_step()

    def step(self, obs=None):
        if obs is not None:
            for dst, src in zip(self.obs, obs):
                if dst.data_ptr() != src.data_ptr():
                    dst.copy_(src, non_blocking=True)
        if self.graph is None:
            return self._eager_step()
        self.graph.replay()
        return self.loss

    def forward_only(self):
        with torch.no_grad():
            return [propagate(inv.params().detach(), inv.rho, inv.geom) for inv in self.invs]

    def gradient(self):
        return torch.cat([inv.params.theta.grad for inv in self.invs])

    def relative_errors(self):
        return np.stack([inv.relative_errors() for inv in self.invs])


def canvas_layout(ws, gap_rows=1, gap_cols=4, col_align=32):
    """Shelf packing of the instances' grids on one canvas: largest first,
    shelves of the canvas width (about square overall), regions at least
    gap_rows rows and gap_cols columns apart (the cells between them stay
    zero: the instances' ghost rings), each region's first column a multiple
    of col_align (32 floats: its rows start on 128-byte lines, as a grid's
    do, so that a tile's own boxes touch no extra sector per row).  Returns
    (X, Y, x0, y0) with x0, y0 per instance in the order of `ws`."""
    up = lambda v: -(-v // col_align) * col_align
    area = sum((w.nx + gap_rows) * up(w.ny + gap_cols) for w in ws)
    width = max(up(max(w.ny for w in ws) + gap_cols), int(np.ceil(np.sqrt(area) / 64.0)) * 64)
    order = sorted(range(len(ws)), key=lambda k: (-ws[k].nx, -ws[k].ny, k))
    x0, y0 = [0] * len(ws), [0] * len(ws)
    shelf_x, shelf_h, col = 0, 0, 0
    for k in order:
        w = ws[k]
        if col + w.ny > width:
            shelf_x += shelf_h + gap_rows
            shelf_h, col = 0, 0
        x0[k], y0[k] = shelf_x, col
        col = up(col + w.ny + gap_cols)
        shelf_h = max(shelf_h, w.nx)
    X = shelf_x + shelf_h
    Y = width
    return X, Y, x0, y0


class CanvasInversion(_GraphedIteration):
    """Many independent scalar-constant inversions of uneven grid sizes and
    step counts advanced as ONE propagation: the instances are regions of a
    canvas (canvas_layout) and every time step is one launch of the tiled
    kernels over the table of all running instances' tiles (instances drop
    out of the table as their step counts end); each instance keeps its own
    constants, source, receivers, observations and gradient; one fused Adam
    launch updates every instance; the whole iteration is one CUDA graph.

    Traces are (S, max nt_out, R), zero past each instance's own frames (the
    observations likewise), and the objective is S times their mean square
    residual: the sum of the instances' misfits up to a factor per instance
    that Adam's per-parameter step normalisation ignores."""

    def __init__(self, ws, device, lr=1e-2, seed=0, graph=True, nt=None, budget_fraction=0.4):
        from .propagate import Instances, choose_ckpt_k
        self.ws = ws
        self.device = device
        S = len(ws)
        nts = [w.nt if nt is None else min(w.nt, nt) for w in ws]
        X, Y, x0, y0 = canvas_layout(ws)
        self.canvas = (X, Y)
        self.x0, self.y0, self.nts = x0, y0, nts
        nt_max = max(nts)
        sig = np.zeros((S, nt_max), np.float32)
        maps, origins = [], []
        for k, w in enumerate(ws):
            sig[k, :nts[k]] = sources.hann_burst_signal(nts[k], DT, w.f0, 5, w.amplitude).astype(np.float32)
            (si, sj), = w.src_cells
            dense = sources.point_load_maps(w.nx, w.ny, H, [sources.cell_position(si, sj, w.nx, w.ny, H)],
                                            w.gaussian_param, device=device)
            m, o = sources.crop_box(dense)
            maps.append(m[0])
            origins.append((int(o[0, 0]) + x0[k], int(o[0, 1]) + y0[k]))
        bx = max(m.shape[0] for m in maps)
        by = max(m.shape[1] for m in maps)
        smap = torch.zeros((S, bx, by), dtype=torch.float32, device=device)
        for k, m in enumerate(maps):
            smap[k, :m.shape[0], :m.shape[1]] = m
        nrec = len(ws[0].rec_cells)
        if any(len(w.rec_cells) != nrec for w in ws):
            raise ValueError("every instance needs the same number of receivers")
        rec = torch.tensor([[(x0[k] + i) * Y + (y0[k] + j) for (i, j) in w.rec_cells]
                            for k, w in enumerate(ws)], dtype=torch.int32, device=device)
        inst = Instances(x0, y0, [w.nx for w in ws], [w.ny for w in ws], nts)
        self.geom = Geometry(nx=X, ny=Y, nt=nt_max, h=H, dt=DT, src_signal=torch.tensor(sig, device=device),
                             src_map=smap, src_origin=torch.tensor(origins, dtype=torch.int32, device=device),
                             stride=1, src_comp=1, rec_idx=rec, instances=inst)
        from ._lib import FLAG_INSTANCES
        self.geom.ckpt_k = choose_ckpt_k(self.geom, 0, device, budget_fraction=budget_fraction,
                                         flags=FLAG_INSTANCES)
        self.rho = torch.full((S,), RHO, dtype=torch.float32, device=device)
        # observations: the same propagation at the true constants plus
        # Gaussian noise of 0.5 % of each instance's trace RMS (seeded)
        Ct = torch.tensor(np.stack([w.C_true for w in ws]), dtype=torch.float32, device=device)
        with torch.no_grad():
            ox, oy = propagate(Ct, self.rho, self.geom)
        g = torch.Generator(device=device).manual_seed(seed)
        self.obs = []
        for o in (ox, oy):
            rms = o.double().pow(2).mean(dim=(1, 2), keepdim=True).sqrt().float()
            noisy = o + 0.005 * rms * torch.randn(o.shape, generator=g, device=device)
            valid = torch.zeros_like(o)
            for k in range(S):
                valid[k, :nts[k]] = 1.0
            self.obs.append((noisy * valid).contiguous())
        C0 = np.stack([initial_guess(w, seed + k) for k, w in enumerate(ws)])
        sc = np.stack([scales(w.C_true) for w in ws])
        self.scale = torch.tensor(sc, dtype=torch.float32, device=device)
        self.theta = torch.nn.Parameter(torch.tensor(C0 / sc, dtype=torch.float32, device=device))
        self.opt = FusedAdam([self.theta], lr=lr)
        self.cell_steps = sum(w.nx * w.ny * n for w, n in zip(ws, nts))
        if graph:
            self.capture()

    def params(self):
        return self.theta * self.scale

    def step_eager(self):
        obs = self.obs
        self.opt.zero_grad(set_to_none=False)
        ux, uy = propagate(self.params(), self.rho, self.geom)
        S = float(len(self.ws))
        loss = series_misfit(ux, uy, obs[0], obs[1], S, S)
        loss.backward()
        self.opt.step()
        return loss

    def forward_only(self):
        with torch.no_grad():
            return propagate(self.params().detach(), self.rho, self.geom)

    def gradient(self):
        return self.theta.grad.reshape(-1)

    def constants(self):
        return self.params().detach().double().cpu().numpy()


def split_by_work(ws, parts, nt=None):
    """Instances split into `parts` lists of about equal work (cell-steps):
    largest first, each to the currently lightest part.  Returns the lists of
    instance numbers (ascending), empty parts dropped."""
    work = [w.nx * w.ny * (w.nt if nt is None else min(w.nt, nt)) for w in ws]
    load = [0] * parts
    members = [[] for _ in range(parts)]
    for k in sorted(range(len(ws)), key=lambda k: (-work[k], k)):
        p = min(range(parts), key=lambda q: (load[q], q))
        members[p].append(k)
        load[p] += work[k]
    return [sorted(m) for m in members if m]


class CanvasSet(_GraphedIteration):
    """The instances split into `parts` canvases of about equal work
    (cell-steps, largest first to the lightest part), each a CanvasInversion
    advanced on its own CUDA stream, the whole iteration one graph.  Each
    canvas is one launch per step; the canvases' launches overlap, so one
    canvas's last partial wave of tiles runs beside the other's work."""

    def __init__(self, ws, device, parts=2, lr=1e-2, seed=0, graph=True, nt=None):
        self.device = device
        self.ws = ws
        self.members = split_by_work(ws, parts, nt)
        # each canvas's tape and scratch from its share of the memory budget
        self.parts = [CanvasInversion([ws[k] for k in m], device, lr=lr, seed=seed, graph=False, nt=nt,
                                      budget_fraction=0.4 / len(self.members))
                      for m in self.members]
        self.streams = [torch.cuda.Stream(device) for _ in self.parts]
        self.obs = [o for c in self.parts for o in c.obs]
        self.cell_steps = sum(c.cell_steps for c in self.parts)
        self.opt = None
        if graph:
            self.capture()

    def step_eager(self):
        main = torch.cuda.current_stream(self.device)
        losses = []
        for c, st in zip(self.parts, self.streams):
            st.wait_stream(main)
            with torch.cuda.stream(st):
                losses.append(c.step_eager())
        for st in self.streams:
            main.wait_stream(st)
        return torch.stack([l.detach() for l in losses]).sum()

    def step(self, obs=None):
        if obs is not None:
            for dst, src in zip(self.obs, obs):
                if dst.data_ptr() != src.data_ptr():
                    dst.copy_(src, non_blocking=True)
        if self.graph is None:
            return self.step_eager()
        self.graph.replay()
        return self._loss

    def gradient(self):
        """Gradients in the order of `ws`."""
        g = torch.empty((len(self.ws), 6), dtype=torch.float32, device=self.device)
        for c, m in zip(self.parts, self.members):
            g[m] = c.theta.grad
        return g.reshape(-1)
