#!/usr/bin/env python
"""Benchmark of the ERNN hot path: one inversion iteration of the rot256 workload.

A step = forward time loop (256x256, 2000 steps, 30-degree rotated orthotropic
constants, one top-centre 1 MHz tone-burst source, 64 top-edge receivers,
checkpoint every 100 steps) -> FP64 trace misfit -> hand-written adjoint
(gradient of the six constants) -> Adam step on normalised constants.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ernn|reference]

The ernn arm prints one JSON line: value = Gcell-steps/s of forward+adjoint
(cell-steps = shots x nx x ny x nt per iteration, summed over ranks), with
e2e (host traces in, loss and gradient out), roofline of the dominant
kernel, clocks sampled during the timed region and the CPU baseline (the
PyTorch restatement of the reference path on the host cores, bounded sample).
The reference arm (--impl reference) times that restatement on the host
cores (all threads) and, as an extra key, on the GPU with autograd.
Under torchrun every rank runs an independent replica (the path shards over
independent inversions; there is no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

L2_BYTES = 129 * 1024 * 1024
H_STEP, DT_STEP = 1e-4, 5e-9  # grid spacing and time step of every benchmark workload
# the CPU baseline times the whole iteration up to this many cell-steps
CPU_FULL_CELL_STEPS = 2.0e8
FLUSH_BYTES = 256 * 1024 * 1024


PATHS = {"auto": 0, "step": 1, "resident": 2, "tiled": 3, "tuned": -1}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ernn", "reference"], default="ernn")
    ap.add_argument("--workload", default="rot256")
    ap.add_argument("--cpu-sample-steps", type=int, default=200,
                    help="time steps of the bounded CPU sample (reference arm steps; larger workloads)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--err-instances", type=int, default=16,
                    help="multi64: instances whose gradient is checked against the FP64 oracle")
    ap.add_argument("--nt", type=int, default=None, help="override the workload's step count")
    ap.add_argument("--ckpt", type=int, default=None, help="override the checkpoint interval")
    ap.add_argument("--path", choices=list(PATHS), default="auto",
                    help="kernel path of the library (auto picks per problem)")
    ap.add_argument("--eager", action="store_true",
                    help="launch every iteration from the host instead of replaying a CUDA graph")
    ap.add_argument("--no-overlap", action="store_true",
                    help="launch consecutive step kernels without programmatic dependent launch")
    ap.add_argument("--canvas-parts", type=int, default=2,
                    help="multi64: split the instances over this many canvases of about equal work, "
                         "each on its own stream (1: one canvas)")
    ap.add_argument("--grouped", action="store_true",
                    help="multi64: the instances grouped by size, one call per group on 8 streams, "
                         "instead of one canvas with a tile table")
    ap.add_argument("--plain", action="store_true",
                    help="only run warmup + steps iterations (no timing, no JSON): a profiling target")
    return ap.parse_args(argv)


def make_workload(args):
    from ernn_gb300 import harness as Hn
    w = Hn.WORKLOADS[args.workload]()
    if args.nt is not None:
        w.nt = args.nt
    if args.ckpt is not None:
        w.ckpt_k = args.ckpt
    w.path = max(PATHS[args.path], 0)
    return w


# --------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg is not None:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if self.pg is None:
            return v
        dev = torch.device("cuda", self.local) if torch.cuda.is_available() else torch.device("cpu")
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg is not None:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_launch:"):
            return float(line.split(":", 1)[1])
    return None


# --------------------------------------------------------------------------
_CPU_EXTRA = {}


def _cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), or "unknown"."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


_STANDALONE = {}


def standalone(name):
    """Load <package>/<name>.py (configs, sources: numpy / torch only) by file
    path, without importing the package, so the reference arm's process never
    maps libernn_gb300.so."""
    if name not in _STANDALONE:
        import importlib.util
        path = os.path.join(ROOT, "elastodynamics-encoded-rnn_gb300", name + ".py")
        spec = importlib.util.spec_from_file_location("ernn_standalone_" + name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = mod  # dataclasses resolve annotations through sys.modules
        spec.loader.exec_module(mod)
        _STANDALONE[name] = mod
    return _STANDALONE[name]


def library_mapped():
    """Whether this process has mapped libernn_gb300.so (Linux /proc maps)."""
    try:
        with open("/proc/self/maps") as f:
            return any("libernn_gb300" in line for line in f)
    except OSError:
        return None


def cpu_sample(workload, nt_sample, iters=2):
    """The reference path (PyTorch restatement, autograd) on the host cores:
    forward (receiver traces) -> misfit -> backward -> Adam, truncated to
    nt_sample steps of the same grid.  Returns (Gcell-steps/s, threads, sample)."""
    Wk, Src = standalone("configs"), standalone("sources")
    from oracle import torch_ref

    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    w = Wk.WORKLOADS[workload]()
    dev = torch.device("cpu")
    if w.extra.get("fields"):
        t = fields_reference_iteration(w, nt_sample, dev, iters)
        return (w.nx * w.ny * nt_sample / t / 1e9, threads,
                f"{workload} grid, {nt_sample} of {w.nt} steps, six constant fields, best of {iters}")
    sig = torch.tensor(Src.hann_burst_signal(nt_sample, Wk.DT, w.f0, 5, w.amplitude),
                       dtype=torch.float32)[None].repeat(w.nshots, 1)
    pos = [Src.cell_position(i, j, w.nx, w.ny, Wk.H) for (i, j) in w.src_cells]
    load = Src.point_load_maps(w.nx, w.ny, Wk.H, pos, w.gaussian_param, device=dev)
    rec = torch.tensor([[i * w.ny + j for (i, j) in w.rec_cells]] * w.nshots, dtype=torch.int32)
    rho = torch.tensor(Wk.RHO)
    theta = torch.nn.Parameter(torch.tensor(Wk.initial_guess(w) / Wk.scales(w.C_true), dtype=torch.float32))
    sc = torch.tensor(Wk.scales(w.C_true), dtype=torch.float32)
    opt = torch.optim.Adam([theta], lr=1e-2)
    with torch.no_grad():  # the observations: also the forward-only timing
        Ct = [torch.tensor(float(c)) for c in w.C_true]
        t0 = time.perf_counter()
        ox, oy = torch_ref.propagate(Ct, rho, w.nx, w.ny, nt_sample, Wk.H, Wk.DT, sig, load, 1, rec)
        t_fwd = time.perf_counter() - t0
    _CPU_EXTRA["forward_only"] = round(w.nshots * w.nx * w.ny * nt_sample / t_fwd / 1e9, 6)
    _CPU_EXTRA["cpu_model"] = _cpu_model()
    times = []
    for _ in range(iters):
        t0 = time.perf_counter()
        opt.zero_grad()
        C = theta * sc
        px, py = torch_ref.propagate([C[i] for i in range(6)], rho, w.nx, w.ny, nt_sample, Wk.H,
                                     Wk.DT, sig, load, 1, rec)
        loss = ((px.double() - ox.double()) ** 2).mean() + ((py.double() - oy.double()) ** 2).mean()
        loss.backward()
        opt.step()
        times.append(time.perf_counter() - t0)
    t = min(times)
    cells = w.nshots * w.nx * w.ny * nt_sample
    return cells / t / 1e9, threads, f"{workload} grid, {nt_sample} of {w.nt} steps, {w.nshots} shot(s), best of {iters}"


def fields_reference_iteration(w, nt, dev, iters):
    """The reference damage loop restated op for op (oracle/torch_ref.py on six
    per-cell constant fields, autograd): forward with dense history every
    `stride` steps, 5:1 misfit on every 2nd frame + TV, backward, Adam.
    Returns the best time of `iters` iterations in seconds."""
    Src = standalone("sources")
    from oracle import torch_ref
    c = standalone("configs").FIELDS301
    h = c["L"] / (w.nx - 1)
    dt = c["total_time"] / (c["nt"] - 1)
    X, Y = Src.centered_grid(w.nx, w.ny, h, device=dev)
    load = Src.gaussian_point_load(X, Y, 0.0, 0.0, c["gaussian_param"]).t()[None].contiguous()
    tt = np.arange(nt) * dt
    sig = torch.tensor(Src.ricker_wavelet(tt, c["f0"], c["t0"], c["amplitude"]), dtype=torch.float32,
                       device=dev)[None]
    logs = [torch.nn.Parameter(torch.full((1, w.nx, w.ny), float(np.log(v)), device=dev)) for v in c["C0"]]
    rho = torch.tensor(c["rho"], device=dev)
    opt = torch.optim.Adam(logs, lr=c["lr"])
    with torch.no_grad():
        tx, ty = torch_ref.propagate([torch.exp(p) for p in logs], rho, w.nx, w.ny, nt, h, dt, sig, load,
                                     w.stride)
    times = []
    for _ in range(iters):
        if dev.type == "cuda":
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        opt.zero_grad()
        C = [torch.exp(p) for p in logs]
        px, py = torch_ref.propagate(C, rho, w.nx, w.ny, nt, h, dt, sig, load, w.stride)
        loss = 5 * torch.mean((px[:, ::2] - tx[:, ::2]) ** 2) + torch.mean((py[:, ::2] - ty[:, ::2]) ** 2)
        tv = sum(torch.sum(torch.abs(f[:, 1:] - f[:, :-1])) + torch.sum(torch.abs(f[:, :, 1:] - f[:, :, :-1]))
                 for f in C)
        (loss + c["lambda_tv"] * tv).backward()
        opt.step()
        if dev.type == "cuda":
            torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    return min(times)


# --------------------------------------------------------------------------
def run_ernn(args, dist):
    import ernn_gb300 as E
    from ernn_gb300 import harness as Hn

    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    lib = E.load_library()
    w = make_workload(args)
    inv = Hn.make_inversion(w, dev)
    tuned = None
    if args.path == "tuned":  # measured path and checkpoint interval (ernn_gb300.autotune)
        from ernn_gb300 import autotune
        damage = isinstance(inv, Hn.DamageInversion)
        with torch.no_grad():  # no autograd graph outlives the probes
            C = (inv.C0 if damage else inv.params()).detach()
            D = inv.D.detach() if damage else None
        tuned = autotune.tune(inv.geom, C, inv.rho, D=D)
        del C, D
        inv.geom.path, inv.geom.ckpt_k, inv.geom.tile_rows = tuned
        torch.cuda.synchronize()
        E.check_device_status()
    if not args.eager:  # the whole iteration as one CUDA graph, replayed per step
        inv.capture()
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    # workloads whose inversion leaves its stable range after a few iterations
    # restart from the initial guess before each one (outside the timed region)
    pre = inv.restart if w.extra.get("restart") else (lambda: None)
    for _ in range(max(args.warmup, 0)):
        pre()
        inv.step()
    torch.cuda.synchronize()
    if args.plain:
        for _ in range(args.steps):
            pre()
            inv.step()
        torch.cuda.synchronize()
        return None

    # ---- main timed region: device-resident inputs
    clocks = Clocks(dev.index)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    n0 = lib.ernn_launch_count()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()                       # L2 flush between timed iterations
        pre()
        ev[k][0].record()
        inv.step()
        ev[k][1].record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = (lib.ernn_launch_count() - n0) // max(args.steps, 1)
    clk = clocks.stop()
    dist.barrier()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    ms = dist.max(ms)
    value = dist.world * w.cell_steps / (ms * 1e-3) / 1e9

    # ---- e2e through the public API: pinned host traces in, loss + gradient out
    obs_h = [o.detach().cpu().pin_memory() for o in inv.obs]
    obs_d = [torch.empty_like(o) for o in inv.obs]
    out_h = torch.empty(1 + inv.gradient().numel(), dtype=torch.float64).pin_memory()
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        pre()
        e2e_ev[k][0].record()
        for hsrc, ddst in zip(obs_h, obs_d):
            ddst.copy_(hsrc, non_blocking=True)
        loss = inv.step(obs_d)
        res = torch.cat([loss.detach().reshape(1), inv.gradient().double().reshape(-1)])
        out_h.copy_(res, non_blocking=True)
        e2e_ev[k][1].record()
    torch.cuda.synchronize()
    e2e_ms = dist.max(sum(a.elapsed_time(b) for a, b in e2e_ev) / args.steps)
    h2d = sum(o.numel() * o.element_size() for o in obs_h)
    d2h = out_h.numel() * out_h.element_size()

    # ---- forward-only throughput (no tape)
    fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with torch.no_grad():
        for k in range(args.steps):
            flush.zero_()
            fev[k][0].record()
            inv.forward_only()
            fev[k][1].record()
    torch.cuda.synchronize()
    fwd_ms = dist.max(sum(a.elapsed_time(b) for a, b in fev) / args.steps)

    # ---- dominant kernel: per-launch device time from library events (an
    # eager iteration: a graph replay makes no library host calls)
    E._lib.profile(True)
    pre()
    n_eager = lib.ernn_launch_count()
    inv.step_eager()
    per_iter = lib.ernn_launch_count() - n_eager   # library kernels of one iteration
    if inv.graph is not None:  # replays launch the captured kernels without host calls
        launches = per_iter
    torch.cuda.synchronize()
    prof = E._lib.profile_read()
    E._lib.profile(False)
    per_class = {}
    for c in ("forward", "adjoint"):
        t_ms, n_l, b_tot = prof[c]
        if n_l:
            us = t_ms * 1e3 / n_l
            gbs = b_tot / n_l / (us * 1e-6) / 1e9
            per_class[c] = {"launches": n_l, "us_per_launch": round(us, 3), "ms_total": round(t_ms, 3),
                            "achieved_gbs": round(gbs, 1), "frac": round(gbs / peaks()[0], 4)}
    cls = max(("forward", "adjoint"), key=lambda c: prof[c][0])
    tot_ms, nlaunch, tot_bytes = prof[cls]
    per_launch_ms = tot_ms / max(nlaunch, 1)
    alg_bytes = tot_bytes / max(nlaunch, 1)        # algorithmic bytes per launch (library-counted)
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    used = int(lib.ernn_last_path())
    kernel_name = {E.PATH_RESIDENT: {"forward": "resident_kernel", "adjoint": "resident_kernel"},
                   E.PATH_TILED: {"forward": "tma_fwd_kernel", "adjoint": "tma_adj_kernel"}}.get(
        used, {"forward": "fwd_step_kernel", "adjoint": "adj_step_kernel"})[cls]
    traffic = profiled_traffic(kernel_name, args.workload)
    state_mb = w.nshots * 2 * w.nx * w.ny * 4 / 2**20
    l2_note = ("working set (three state levels) is L2-resident at this size; bytes are algorithmic"
               if 3 * state_mb < 100 else "state levels exceed L2; bytes are algorithmic")

    rec = {
        "metric": "Gcell-steps/s fwd+adj (hand adjoint, one Adam iteration)",
        "value": round(value, 4),
        "unit": "Gcell-steps/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded tone-burst shots; observations = same forward at true constants + 0.5% noise)",
        "config": {"workload": f"{w.name}: {w.nx}x{w.ny} grid, {w.nt} steps, {w.nshots} shot(s), "
                               f"{len(w.rec_cells)} receivers, "
                               f"{'six constant fields' if w.extra.get('fields') else 'D-field' if w.D_true is not None else 'scalar constants'}, "
                               f"ckpt every {inv.geom.ckpt_k} steps",
                   "cell_steps_per_iter": w.cell_steps,
                   "kernel_path": {0: "auto", 1: "step", 2: "resident", 3: "tiled"}[int(lib.ernn_last_path())],
                   "launch": ("one CUDA graph per iteration" if inv.graph is not None else "eager") +
                             ("" if args.no_overlap else ", step kernels overlapped (programmatic dependent launch)"),
                   "path_choice": (f"measured (autotune): tiles 64x{inv.geom.tile_rows}" if tuned
                                   else args.path),
                   "l2": "flushed between timed iterations (256 MiB write)",
                   **({"iterations": "each restarts from the initial guess (outside the timed region)"}
                      if w.extra.get("restart") else {}),
                   "parallelism": f"replicas x{dist.world}"},
        "e2e": {"value": round(dist.world * w.cell_steps / (e2e_ms * 1e-3) / 1e9, 4),
                "unit": "Gcell-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_ms, 4)},
        "forward_only": {"value": round(dist.world * w.cell_steps / (fwd_ms * 1e-3) / 1e9, 4),
                         "unit": "Gcell-steps/s", "ms": round(fwd_ms, 4)},
        "ms_per_iter": round(ms, 4),
        "wall_ms_per_step": round(wall * 1e3 / args.steps, 4),
        "gpu_launches": int(launches * args.steps),
        "roofline": {"bound": "hbm", "kernel": kernel_name, "class": cls, "achieved": round(achieved, 2),
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
                     "launch_us": round(per_launch_ms * 1e3, 3), "launches_per_iter": nlaunch,
                     "note": l2_note, "classes": per_class},
        "clocks": clk,
        "loss": float((pre(), inv.step())[1].item()),
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        # the whole iteration when it is about 20 s of host work or less
        # (rot256, plate128), else a bounded sample of its steps
        full = w.cell_steps <= CPU_FULL_CELL_STEPS and not w.extra.get("fields")
        v, thr, sample = cpu_sample(args.workload, w.nt if full else args.cpu_sample_steps,
                                    iters=1 if full else 2)
        rec["cpu_baseline"] = {"value": round(v, 6), "unit": "Gcell-steps/s", "cores": thr,
                               "kind": "port", "same_config": full,
                               "sample": sample + " (PyTorch restatement of the reference path, autograd)",
                               **_CPU_EXTRA}
        rec["errors"] = config_errors(args, dev)
    return rec


# the FP64 check of the benchmark line runs the whole workload up to this
# many cell-steps (about 10 s of host work); larger ones keep their grids and
# shots with fewer steps
ERR_FULL_CELL_STEPS = 2.0e8
ERR_SAMPLE_STEPS = 160


def config_errors(args, dev):
    """Forward-trace and gradient error of the benchmarked workload against
    the FP64 run of the same scheme (oracle/accuracy.py): same
    grid, shots, receivers, constants, checkpoint interval and kernel path."""
    from oracle.accuracy import workload_errors
    w = make_workload(args)
    if w.extra.get("fields"):
        return {"note": "not computed for the six-field workload (dense history, TV objective)"}
    full = w.cell_steps <= ERR_FULL_CELL_STEPS
    nt = None if full else min(w.nt, ERR_SAMPLE_STEPS)
    ckpt = None if full else max(1, (nt or w.nt) // 8)
    r = workload_errors(w, dev, nt=nt, ckpt_k=ckpt, path=w.path, fp32_floor=w.D_true is not None)
    r["bound"] = 1e-4
    r["scope"] = ("whole workload" if full else
                  f"full grid and shots, {r['nt']} of {w.nt} steps, checkpoint every {r['ckpt_k']}")
    r["against"] = "FP64 C oracle of the same scheme (checkpoint recompute), same observations"
    return r


def _dense_load(geom, dtype, device):
    """(S, nx, ny) load of a geometry's cropped source boxes."""
    S = geom.nshots
    load = torch.zeros((S, geom.nx, geom.ny), dtype=dtype)
    smap = geom.src_map.detach().cpu().to(dtype)
    org = geom.src_origin.detach().cpu().tolist()
    bx, by = smap.shape[1], smap.shape[2]
    for s in range(S):
        ox, oy = org[s]
        a0, a1 = max(0, -ox), min(bx, geom.nx - ox)
        b0, b1 = max(0, -oy), min(by, geom.ny - oy)
        if a0 < a1 and b0 < b1:
            load[s, ox + a0:ox + a1, oy + b0:oy + b1] = smap[s, a0:a1, b0:b1]
    return load.to(device)


def multi_grad_errors(inv, max_side=128, count=3):
    """Hand-adjoint gradients (FP32 fields, FP64 sums) of the first `count`
    instances with side <= max_side against the restated reference path in
    FP64 with autograd on the host cores, at the instances' current
    constants: relative L2 error of the gradient of the normalised constants."""
    import ernn_gb300.harness as Hn
    from oracle import torch_ref
    out = []
    for one in inv.invs:
        if len(out) >= count or one.w.nx > max_side:
            continue
        g = one.geom
        theta = one.params.theta
        theta.grad = None
        ux, uy = Hn.propagate(one.params(), one.rho, g)
        Hn.trace_misfit(ux, uy, one.obs[0], one.obs[1]).backward()
        g32 = theta.grad.detach().double().cpu()
        t64 = theta.detach().double().cpu().requires_grad_(True)
        C = t64 * one.params.scale.detach().double().cpu()
        rho = torch.tensor(float(one.rho), dtype=torch.float64)
        px, py = torch_ref.propagate([C[i] for i in range(6)], rho, g.nx, g.ny, g.nt, g.h, g.dt,
                                     g.src_signal.detach().double().cpu(), _dense_load(g, torch.float64, "cpu"),
                                     g.stride, g.rec_idx.detach().cpu(), g.src_comp)
        ox, oy = (o.detach().double().cpu() for o in one.obs)
        (((px - ox) ** 2).mean() + ((py - oy) ** 2).mean()).backward()
        e = float((g32 - t64.grad).norm() / t64.grad.norm())
        out.append({"side": g.nx, "nt": g.nt, "grad_rel_err": round(e, 9)})
    return out


def canvas_set_grad_errors(inv, dev, count=64):
    """canvas_grad_errors over the canvases of a CanvasSet: the `count`
    smallest instances of the whole set, instance numbers of the set."""
    order = sorted(range(len(inv.ws)), key=lambda k: inv.ws[k].nx)[:count]
    out, secs = [], 0.0
    for part, members in zip(inv.parts, inv.members):
        local = [members.index(k) for k in order if k in members]
        if not local:
            continue
        r = canvas_grad_errors(part, dev, select=local)
        secs += r["oracle_s"]
        for e in r["per_instance"]:
            out.append({**e, "instance": members[e["instance"]]})
    worst = max(out, key=lambda r: r["grad_rel_err"])
    return {"instances": len(out), "max_fwd_rel_err": max(r["fwd_rel_err"] for r in out),
            "max_grad_rel_err": worst["grad_rel_err"],
            "max_grad_rel_err_same_residual": max(r["grad_rel_err_same_residual"] for r in out),
            "worst": worst, "oracle_s": round(secs, 1), "per_instance": out}


def canvas_grad_errors(inv, dev, count=64, select=None):
    """Per-instance trace and gradient error of the canvas iteration against
    the FP64 C oracle (oracle/accuracy.py), every instance on
    its own grid with its own steps, at the instances' current constants, for
    the misfit of the canvas objective (S x mean over the padded traces) and
    the same observations.  Instances are checked smallest first (or the
    instances `select`)."""
    from oracle import oracle as O
    from oracle.accuracy import _rel
    ws, S = inv.ws, len(inv.ws)
    theta = inv.theta
    theta.grad = None
    with torch.enable_grad():
        from ernn_gb300.propagate import propagate as _prop
        from ernn_gb300.misfit import series_misfit
        ux, uy = _prop(inv.params(), inv.rho, inv.geom)
        series_misfit(ux, uy, inv.obs[0], inv.obs[1], float(S), float(S)).backward()
    g32 = (theta.grad.detach().double() / inv.scale.double()).cpu().numpy()  # dL/dC (C = theta x scale)
    px32, py32 = ux.detach().double().cpu().numpy(), uy.detach().double().cpu().numpy()
    C = inv.params().detach().cpu().numpy().astype(np.float64)
    ox, oy = (o.detach().double().cpu().numpy() for o in inv.obs)
    count_all = ox.size  # the canvas objective's mean counts the padded traces of all instances
    sig = inv.geom.src_signal.detach().double().cpu().numpy()
    smap = inv.geom.src_map.detach().double().cpu().numpy()
    org = inv.geom.src_origin.detach().cpu().numpy()
    rec = inv.geom.rec_idx.detach().cpu().numpy()
    X, Y = inv.canvas
    out, t0 = [], time.perf_counter()
    for k in (select if select is not None else sorted(range(S), key=lambda k: ws[k].nx)[:count]):
        w, nt = ws[k], inv.nts[k]
        x0, y0 = inv.x0[k], inv.y0[k]
        rk = ((rec[k] // Y - x0) * w.ny + (rec[k] % Y - y0)).astype(np.int32)
        case = O.Case(w.nx, w.ny, nt, H_STEP, DT_STEP, float(inv.rho[k]), C[k].astype(np.float32).astype(np.float64),
                      sig[k:k + 1, :nt], smap[k:k + 1], np.array([[org[k, 0] - x0, org[k, 1] - y0]], np.int32),
                      record=O.RECORD_RECEIVERS, rec_idx=rk[None])
        kk = max(1, int(round((2 * nt) ** 0.5)))
        qx, qy, ck = O.forward_ckpt(case, kk, "f64")
        gx = 2.0 * S * (qx - ox[k:k + 1, :nt]) / count_all
        gy = 2.0 * S * (qy - oy[k:k + 1, :nt]) / count_all
        gC, _ = O.adjoint_ckpt(case, kk, ck, gx, gy, "f64")
        # the FP64 adjoint driven by the canvas's own FP32 traces: the adjoint
        # arithmetic alone, without the residual's sensitivity to the forward
        rx = 2.0 * S * (px32[k:k + 1, :nt] - ox[k:k + 1, :nt]) / count_all
        ry = 2.0 * S * (py32[k:k + 1, :nt] - oy[k:k + 1, :nt]) / count_all
        sC, _ = O.adjoint_ckpt(case, kk, ck, rx, ry, "f64")
        s = inv.scale[k].detach().double().cpu().numpy()
        row = {"instance": k, "side": w.nx, "nt": nt,
               "fwd_rel_err": round(max(_rel(px32[k:k + 1, :nt], qx), _rel(py32[k:k + 1, :nt], qy)), 9),
               "residual_rel_diff": round(max(_rel(rx, gx), _rel(ry, gy)), 9),
               "grad_rel_err": round(_rel(g32[k] * s, gC * s), 9),
               "grad_rel_err_same_residual": round(_rel(g32[k] * s, sC * s), 9)}
        if row["grad_rel_err"] > 1e-4:
            # the same scheme in FP32 (the C oracle: FP32 fields and arithmetic,
            # FP64 sums): the gradient difference any FP32 evaluation carries
            # where the residual is this sensitive to the forward
            fx, fy, ck32 = O.forward_ckpt(case, kk, "f32")
            hx = 2.0 * S * (fx.astype(np.float64) - ox[k:k + 1, :nt]) / count_all
            hy = 2.0 * S * (fy.astype(np.float64) - oy[k:k + 1, :nt]) / count_all
            fC, _ = O.adjoint_ckpt(case, kk, ck32, hx, hy, "f32")
            row["oracle_fp32_grad_rel_err"] = round(_rel(fC * s, gC * s), 9)
            row["oracle_fp32_fwd_rel_err"] = round(max(_rel(fx.astype(np.float64), qx),
                                                       _rel(fy.astype(np.float64), qy)), 9)
            row["oracle_fp32_residual_rel_diff"] = round(max(_rel(hx, gx), _rel(hy, gy)), 9)
        out.append(row)
    worst = max(out, key=lambda r: r["grad_rel_err"]) if out else None
    return {"instances": len(out), "max_fwd_rel_err": max(r["fwd_rel_err"] for r in out),
            "max_grad_rel_err": worst["grad_rel_err"],
            "max_grad_rel_err_same_residual": max(r["grad_rel_err_same_residual"] for r in out),
            "worst": worst, "oracle_s": round(time.perf_counter() - t0, 1), "per_instance": out}


def multi_plain_autograd(ws, dev, nt=100, count=8):
    """The restated reference path with autograd on the GPU (FP32), looped over
    `count` of the instances `ws` spread over the sizes, `nt` steps each, at
    their seeded initial guesses: cell-steps per second of forward + backward
    (the plain form the multi-instance configuration compares with)."""
    import ernn_gb300.harness as Hn
    from oracle import torch_ref
    order = sorted(range(len(ws)), key=lambda k: ws[k].nx)
    pick = [order[round(i * (len(order) - 1) / max(1, count - 1))] for i in range(count)]
    cells, secs = 0, 0.0
    rho = torch.tensor(Hn.RHO, device=dev)
    for k in pick:
        g = Hn.geometry(ws[k], dev)
        C = torch.tensor(Hn.initial_guess(ws[k], k), dtype=torch.float32, device=dev, requires_grad=True)
        load = _dense_load(g, torch.float32, dev)
        sig = g.src_signal[:, :nt].contiguous()
        rec = g.rec_idx
        for rep in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            px, py = torch_ref.propagate([C[i] for i in range(6)], rho, g.nx, g.ny, nt, g.h, g.dt,
                                         sig, load, g.stride, rec, g.src_comp)
            ((px.double() ** 2).mean() + (py.double() ** 2).mean()).backward()
            torch.cuda.synchronize()
            if rep == 1:
                secs += time.perf_counter() - t0
                cells += g.nx * g.ny * nt
    return {"value": round(cells / secs / 1e9, 5), "unit": "Gcell-steps/s",
            "sample": f"{count} of {len(ws)} instances (sides "
                      f"{sorted(ws[k].nx for k in pick)}), {nt} steps each, "
                      f"PyTorch restatement of the reference path with autograd on the same GPU"}


def run_multi(args, dist):
    """multi64: 64 uneven inversions, one CUDA-graph-captured Adam iteration."""
    import ernn_gb300 as E
    from ernn_gb300 import harness as Hn

    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    lib = E.load_library()
    ws = Hn.multi_instances(64)
    t0 = time.perf_counter()
    tuned = False
    if args.grouped:
        # instances grouped by size, each group one call with per-shot
        # constants; kernel path per group from the autotuner unless forced
        tuned = args.path in ("auto", "tuned")
        inv = Hn.MultiInversion(ws, dev, tuned=tuned, path=None if tuned else PATHS[args.path])
    else:
        # configuration 5 as one propagation: every instance a region of one
        # canvas, one launch per time step over the running instances' tiles
        inv = (Hn.CanvasInversion(ws, dev, nt=args.nt) if args.canvas_parts <= 1 else
               Hn.CanvasSet(ws, dev, parts=args.canvas_parts, nt=args.nt))
    setup_s = time.perf_counter() - t0
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    for _ in range(max(args.warmup, 0)):
        inv.step()
    torch.cuda.synchronize()
    if args.plain:
        for _ in range(args.steps):
            inv.step()
        torch.cuda.synchronize()
        return None
    clocks = Clocks(dev.index)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    n0 = lib.ernn_launch_count()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record()
        loss = inv.step()
        ev[k][1].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = lib.ernn_launch_count() - n0   # graph replays launch kernels without host calls
    ms = dist.max(sum(a.elapsed_time(b) for a, b in ev) / args.steps)
    value = dist.world * inv.cell_steps / (ms * 1e-3) / 1e9
    # e2e: observations in from pinned host memory, losses and gradients out
    obs_h = [o.detach().cpu().pin_memory() for o in inv.obs]
    out_h = torch.empty(1 + inv.gradient().numel(), dtype=torch.float64).pin_memory()
    e2e = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        e2e[k][0].record()
        loss = inv.step([o.to(dev, non_blocking=True) for o in obs_h])
        out_h.copy_(torch.cat([loss.reshape(1), inv.gradient().double()]), non_blocking=True)
        e2e[k][1].record()
    torch.cuda.synchronize()
    e2e_ms = dist.max(sum(a.elapsed_time(b) for a, b in e2e) / args.steps)
    sides = [w.nx for w in ws]
    # library kernels of one iteration (an eager iteration: replays make no
    # host calls), timed per kernel class by the library's own events
    E._lib.profile(True)
    n_eager = lib.ernn_launch_count()
    (inv._eager_step if args.grouped else inv.step_eager)()
    torch.cuda.synchronize()
    per_iter = lib.ernn_launch_count() - n_eager
    prof = E._lib.profile_read()
    E._lib.profile(False)
    classes = {}
    for c in ("forward", "adjoint", "other"):
        t_ms, n_l, b_tot = prof[c]
        if n_l:
            classes[c] = {"launches": n_l, "ms_total": round(t_ms, 3), "us_per_launch": round(t_ms * 1e3 / n_l, 3),
                          "achieved_gbs": round(b_tot / (t_ms * 1e-3) / 1e9, 1) if b_tot else None,
                          "frac": round(b_tot / (t_ms * 1e-3) / 1e9 / peaks()[0], 4) if b_tot else None}
    extra = {}
    if dist.rank == 0 and not args.no_cpu_baseline:
        if args.grouped:
            extra["grad_error_vs_fp64"] = multi_grad_errors(inv)
            extra["plain_autograd_loop"] = multi_plain_autograd(ws, dev)
        elif args.canvas_parts <= 1:
            extra["grad_error_vs_fp64"] = canvas_grad_errors(inv, dev, count=args.err_instances)
        else:
            extra["grad_error_vs_fp64"] = canvas_set_grad_errors(inv, dev, count=args.err_instances)
        if not args.grouped:
            extra["plain_autograd_loop"] = multi_plain_autograd(ws, dev)
    return {
        "metric": "Gcell-steps/s fwd+adj (hand adjoint, one Adam iteration)",
        "value": round(value, 4), "unit": "Gcell-steps/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded instances and observations)",
        "config": {"workload": f"multi64: 64 inversions, side {min(sides)}..{max(sides)}, nt = 5.2 side, "
                               f"one CUDA-graph-captured Adam iteration over all instances; " +
                               (f"{len(inv.groups)} groups of equal instances, each one call with "
                                f"per-shot constants, on 8 streams" if args.grouped else
                                f"one {inv.canvas[0]}x{inv.canvas[1]} canvas, one launch per step over "
                                f"a tile table of the running instances (checkpoint every "
                                f"{inv.geom.ckpt_k})" if args.canvas_parts <= 1 else
                                f"{len(inv.parts)} canvases (" + ", ".join(f"{c.canvas[0]}x{c.canvas[1]}"
                                                                         for c in inv.parts) +
                                "), each one launch per step over its running instances' tiles, "
                                "on their own streams"),
                   "cell_steps_per_iter": inv.cell_steps,
                   "path_choice": "measured per group (autotune)" if tuned else args.path,
                   "l2": "flushed between timed iterations (256 MiB write)"},
        "e2e": {"value": round(dist.world * inv.cell_steps / (e2e_ms * 1e-3) / 1e9, 4),
                "unit": "Gcell-steps/s", "h2d_bytes_per_step": sum(o.numel() * 4 for o in obs_h),
                "d2h_bytes_per_step": out_h.numel() * 8},
        "ms_per_iter": round(ms, 3), "graph_capture_setup_s": round(setup_s, 2),
        "kernel_classes_eager": classes,
        "host_launch_calls_in_timed_region": int(launches),
        "gpu_launches": int(per_iter * args.steps),
        "clocks": clk, "loss": float(loss), **extra,
    }


FEM301 = dict(nx=301, ny=301, Lx=0.4, Ly=0.4, nt=2001, t_total=60e-6, source_amplitude=1e10,
              source_f0=100e3, source_t0=10e-6, gaussian_param=5e6, C11=130.74e9, C22=11.50e9,
              C12=10.49e9, C16=30.67e9, C26=3.75e9, C66=14.77e9, rho=1610.0,
              source_position=(0.0, 0.0))


def run_fem(args, dist):
    """fem301: the FEM data generator's own configuration (301^2 nodes, 2001
    levels, frames every 5 levels); a step is one generator run."""
    import ernn_gb300 as E
    from ernn_gb300 import fem as EF

    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    lib = E.load_library()
    c = dict(FEM301)
    x, y, el, bnd, dx, dy = EF.create_structured_triangular_mesh(c["nx"], c["ny"], c["Lx"], c["Ly"])
    t, dt, nt = EF._time_axis(c["nt"] if args.nt is None else args.nt, c["t_total"], dx, dy,
                              c["C11"], c["C22"], c["C66"], c["rho"])
    X, Y = np.meshgrid(x, y, indexing="ij")
    load = EF.gaussian_point_load(X, Y, 0.0, 0.0, c["gaussian_param"]).astype(np.float32)
    sig = EF.ricker_wavelet(t, c["source_f0"], c["source_t0"], c["source_amplitude"]).astype(np.float32)
    C = tuple(c[k] for k in ("C11", "C22", "C12", "C16", "C26", "C66"))
    nx, ny, stride = c["nx"], c["ny"], 5
    load_d = torch.tensor(load, device=dev)
    sig_d = torch.tensor(sig, device=dev)
    run = lambda ld, sg: EF.fem_frames(nx, ny, nt, dx, dy, dt, c["rho"], C, ld, sg, stride=stride, device=dev)
    for _ in range(max(args.warmup, 0)):
        run(load_d, sig_d)
    torch.cuda.synchronize()
    if args.plain:
        for _ in range(args.steps):
            run(load_d, sig_d)
        torch.cuda.synchronize()
        return None
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    clocks = Clocks(dev.index)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    n0 = lib.ernn_launch_count()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record()
        run(load_d, sig_d)
        ev[k][1].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = (lib.ernn_launch_count() - n0) / args.steps
    ms = dist.max(sum(a.elapsed_time(b) for a, b in ev) / args.steps)
    node_steps = nx * ny * (nt - 2)
    value = dist.world * node_steps / (ms * 1e-3) / 1e9
    # e2e: load and time factors from pinned host memory in, every frame out
    load_h, sig_h = torch.tensor(load).pin_memory(), torch.tensor(sig).pin_memory()
    nt_out = (nt + stride - 1) // stride
    out_h = torch.empty((2, nt_out, nx, ny), dtype=torch.float32).pin_memory()
    e2e = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        e2e[k][0].record()
        fx, fy = run(load_h.to(dev, non_blocking=True), sig_h.to(dev, non_blocking=True))
        out_h[0].copy_(fx, non_blocking=True)
        out_h[1].copy_(fy, non_blocking=True)
        e2e[k][1].record()
    torch.cuda.synchronize()
    e2e_ms = dist.max(sum(a.elapsed_time(b) for a, b in e2e) / args.steps)
    rec = {
        "metric": "Gnode-steps/s (FEM data generator time loop)", "value": round(value, 4),
        "unit": "Gnode-steps/s", "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (the generator's own source and material)",
        "config": {"workload": f"fem301: {nx}x{ny} nodes, {nt} levels (dt {dt:.3e} s), frames every {stride}",
                   "l2": "flushed between timed runs (256 MiB write)"},
        "e2e": {"value": round(dist.world * node_steps / (e2e_ms * 1e-3) / 1e9, 4), "unit": "Gnode-steps/s",
                "h2d_bytes_per_step": load.nbytes + sig.nbytes, "d2h_bytes_per_step": out_h.numel() * 4,
                "ms_per_step": round(e2e_ms, 3)},
        "gpu_launches": int(launches * args.steps), "clocks": clk,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        from oracle import fem as OF
        ns = 60
        t0 = time.perf_counter()
        OF.fem_forward(nx, ny, ns, dx, dy, dt, c["rho"], C, load, sig[:ns], stride=stride, precision="f32")
        cpu_s = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": round(nx * ny * (ns - 2) / cpu_s / 1e9, 6), "unit": "Gnode-steps/s",
                               "cores": 1, "kind": "port",
                               "sample": f"fem301 grid, {ns} of {nt} levels, C restatement of the generator loop"}
    return rec


def run_reference(args, dist):
    """The reference path restated op for op in PyTorch (oracle/torch_ref.py),
    on the host cores with all threads; bounded sample per step."""
    if dist.rank != 0:
        return None
    if args.workload in ("fem301", "multi64"):
        return run_reference_other(args)
    w = standalone("configs").WORKLOADS[args.workload]()
    nts = args.cpu_sample_steps
    for _ in range(max(args.warmup, 0)):
        cpu_sample(args.workload, min(nts, 20), iters=1)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, thr, sample = cpu_sample(args.workload, nts, iters=1)
        vals.append(v)
    wall = time.perf_counter() - t0
    value = statistics.median(vals)
    rec = {
        "impl": "reference",
        "metric": "Gcell-steps/s fwd+adj (hand adjoint, one Adam iteration)",
        "value": round(value, 6), "unit": "Gcell-steps/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(wall * 1e3 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{w.name}: {w.nx}x{w.ny} grid, {w.nt} steps (sampled {nts}), "
                               f"{w.nshots} shot(s), {len(w.rec_cells)} receivers"},
        "cpu_baseline": {"value": round(value, 6), "unit": "Gcell-steps/s", "cores": thr,
                         "kind": "port", "same_config": nts >= w.nt,
                         "sample": sample + " (PyTorch restatement of the reference path, autograd)",
                         **_CPU_EXTRA},
        "e2e": {"value": round(value, 6), "unit": "Gcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if torch.cuda.is_available():
        if w.extra.get("fields"):
            t = fields_reference_iteration(w, w.nt, torch.device("cuda", 0), 2)
            rec["gpu_autograd"] = {"ms_per_iter": round(t * 1e3, 3),
                                   "value": round(w.nx * w.ny * w.nt / t / 1e9, 5), "unit": "Gcell-steps/s"}
        else:
            rec["gpu_autograd"] = gpu_autograd(args, w)
    # evidence that this arm ran nothing of the library: its process never
    # mapped libernn_gb300.so
    rec["native_library_mapped"] = library_mapped()
    return rec


def run_reference_other(args):
    """Reference arm of the non-default workloads: the C restatement of the
    generator loop (fem301), or the restated reference path looped over the
    instances' bounded samples is not provided (multi64)."""
    if args.workload == "multi64":
        return {"impl": "reference", "unavailable": "multi64 has no reference arm here; the default "
                "workload's arm times the reference path"}
    from ernn_gb300 import fem as EF
    from oracle import fem as OF
    c = dict(FEM301)
    x, y, el, bnd, dx, dy = EF.create_structured_triangular_mesh(c["nx"], c["ny"], c["Lx"], c["Ly"])
    t, dt, nt = EF._time_axis(c["nt"], c["t_total"], dx, dy, c["C11"], c["C22"], c["C66"], c["rho"])
    X, Y = np.meshgrid(x, y, indexing="ij")
    load = EF.gaussian_point_load(X, Y, 0.0, 0.0, c["gaussian_param"]).astype(np.float32)
    sig = EF.ricker_wavelet(t, c["source_f0"], c["source_t0"], c["source_amplitude"]).astype(np.float32)
    C = tuple(c[k] for k in ("C11", "C22", "C12", "C16", "C26", "C66"))
    ns = 60
    vals = []
    for k in range(max(args.warmup, 0) + args.steps):
        t0 = time.perf_counter()
        OF.fem_forward(c["nx"], c["ny"], ns, dx, dy, dt, c["rho"], C, load, sig[:ns], stride=5,
                       precision="f32")
        if k >= args.warmup:
            vals.append(c["nx"] * c["ny"] * (ns - 2) / (time.perf_counter() - t0) / 1e9)
    v = statistics.median(vals)
    sample = f"fem301 grid, {ns} of {nt} levels, C restatement of the generator loop, 1 thread"
    return {"impl": "reference", "metric": "Gnode-steps/s (FEM data generator time loop)",
            "value": round(v, 6), "unit": "Gnode-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(c["nx"] * c["ny"] * (nt - 2) / (v * 1e9) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": "fem301"},
            "cpu_baseline": {"value": round(v, 6), "unit": "Gnode-steps/s", "cores": 1, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 6), "unit": "Gnode-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def gpu_autograd(args, w, iters=3):
    """The same restated reference path on the GPU with autograd (the reference's
    plain form on the same device), full workload."""
    Wk, Src = standalone("configs"), standalone("sources")
    from oracle import torch_ref
    dev = torch.device("cuda", 0)
    sig = torch.tensor(Src.hann_burst_signal(w.nt, Wk.DT, w.f0, 5, w.amplitude),
                       dtype=torch.float32, device=dev)[None].repeat(w.nshots, 1)
    pos = [Src.cell_position(i, j, w.nx, w.ny, Wk.H) for (i, j) in w.src_cells]
    load = Src.point_load_maps(w.nx, w.ny, Wk.H, pos, w.gaussian_param, device=dev)
    rec = torch.tensor([[i * w.ny + j for (i, j) in w.rec_cells]] * w.nshots, dtype=torch.int32, device=dev)
    rho = torch.tensor(Wk.RHO, device=dev)
    with torch.no_grad():
        Ct = [torch.tensor(float(c), device=dev) for c in w.C_true]
        ox, oy = torch_ref.propagate(Ct, rho, w.nx, w.ny, w.nt, Wk.H, Wk.DT, sig, load, 1, rec)
    theta = torch.nn.Parameter(torch.tensor(Wk.initial_guess(w) / Wk.scales(w.C_true), dtype=torch.float32, device=dev))
    sc = torch.tensor(Wk.scales(w.C_true), dtype=torch.float32, device=dev)
    opt = torch.optim.Adam([theta], lr=1e-2)

    def it():
        opt.zero_grad()
        C = theta * sc
        px, py = torch_ref.propagate([C[i] for i in range(6)], rho, w.nx, w.ny, w.nt, Wk.H, Wk.DT,
                                     sig, load, 1, rec)
        loss = ((px.double() - ox.double()) ** 2).mean() + ((py.double() - oy.double()) ** 2).mean()
        loss.backward()
        opt.step()
    it()
    torch.cuda.synchronize()
    t = []
    for _ in range(iters):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        it()
        b.record()
        torch.cuda.synchronize()
        t.append(a.elapsed_time(b))
    ms = statistics.median(t)
    return {"ms_per_iter": round(ms, 3), "value": round(w.cell_steps / (ms * 1e-3) / 1e9, 5),
            "unit": "Gcell-steps/s", "peak_mem_gb": round(torch.cuda.max_memory_allocated(dev) / 1e9, 2)}


def main():
    args = parse()
    dist = Dist()
    if args.no_overlap and args.impl == "ernn":
        from ernn_gb300 import _lib
        _lib.launch_overlap(False)
    try:
        if args.impl == "reference":
            rec = run_reference(args, dist)
        elif args.workload == "multi64":
            rec = run_multi(args, dist)
        elif args.workload == "fem301":
            rec = run_fem(args, dist)
        else:
            rec = run_ernn(args, dist)
        if rec is not None and dist.rank == 0:
            print(json.dumps(rec), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
