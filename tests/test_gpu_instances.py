"""Independent instances of uneven sizes and step counts on one canvas (GPU only).

ernn_forward_instances / ernn_adjoint_instances advance every instance with
one launch per time step over a table of the running instances' tiles.  Each
instance's traces and gradient must equal those of the same instance run
alone through ernn_forward / ernn_adjoint on the tiled path (same kernels,
same tile positions relative to the instance), and match the FP64 oracle.
"""
import numpy as np
import pytest
import torch

import ernn_gb300 as E
from ernn_gb300 import _lib, harness as Hn
from ernn_gb300.propagate import Instances
from cases import C_ROT30, H, DT, RHO, gauss_map, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")

# (nx, ny, nt) of each instance: uneven grids (ny % 4 == 0) and step counts
SPECS = [(40, 48, 90), (70, 132, 130), (24, 20, 60), (33, 64, 110)]


def _instances(specs, seed=0, nrec=6):
    """Per-instance problems: constants, signal, source box, receivers."""
    rng = np.random.default_rng(seed)
    out = []
    for (nx, ny, nt) in specs:
        C = (C_ROT30 * rng.uniform(0.9, 1.1, size=6)).astype(np.float32).astype(np.float64)
        t = np.arange(nt) * DT
        sig = (np.sin(2 * np.pi * 2e6 * t + rng.uniform(0, 6)) * np.exp(-((t - 2e-7) / 1.5e-7) ** 2) * 1e10)
        smap = gauss_map(7, 7, H, 0.0, 0.0) * rng.uniform(0.5, 1.5)
        org = (int(rng.integers(0, nx - 7)), int(rng.integers(0, ny - 7)))
        rec = rng.choice(nx * ny, size=nrec, replace=False).astype(np.int32)
        out.append(dict(nx=nx, ny=ny, nt=nt, C=C, sig=sig.astype(np.float32), smap=smap.astype(np.float32),
                        org=org, rec=rec))
    return out


def _canvas(insts, ckpt_k=None):
    ws = [Hn.Workload(f"i{k}", d["nx"], d["ny"], d["nt"], d["C"], [(0, 0)], []) for k, d in enumerate(insts)]
    X, Y, x0, y0 = Hn.canvas_layout(ws)
    S = len(insts)
    nt_max = max(d["nt"] for d in insts)
    sig = np.zeros((S, nt_max), np.float32)
    for k, d in enumerate(insts):
        sig[k, :d["nt"]] = d["sig"]
    smap = np.stack([d["smap"] for d in insts])
    org = np.array([(d["org"][0] + x0[k], d["org"][1] + y0[k]) for k, d in enumerate(insts)], np.int32)
    rec = np.stack([(x0[k] + d["rec"] // d["ny"]) * Y + (y0[k] + d["rec"] % d["ny"])
                    for k, d in enumerate(insts)]).astype(np.int32)
    t = lambda a, dt=torch.float32: torch.as_tensor(a).to(dt).to(DEV).contiguous()
    inst = Instances(x0, y0, [d["nx"] for d in insts], [d["ny"] for d in insts], [d["nt"] for d in insts])
    geom = E.Geometry(nx=X, ny=Y, nt=nt_max, h=H, dt=DT, src_signal=t(sig), src_map=t(smap),
                      src_origin=t(org, torch.int32), stride=1, rec_idx=t(rec, torch.int32),
                      ckpt_k=ckpt_k, instances=inst)
    return geom


def _single(d, ckpt_k=None):
    t = lambda a, dt=torch.float32: torch.as_tensor(a).to(dt).to(DEV).contiguous()
    return E.Geometry(nx=d["nx"], ny=d["ny"], nt=d["nt"], h=H, dt=DT, src_signal=t(d["sig"][None]),
                      src_map=t(d["smap"][None]), src_origin=t(np.array([d["org"]]), torch.int32), stride=1,
                      rec_idx=t(d["rec"][None], torch.int32), ckpt_k=ckpt_k, path=E.PATH_TILED)


def _weights(insts, nt_max, seed=3):
    rng = np.random.default_rng(seed)
    S, R = len(insts), len(insts[0]["rec"])
    wx, wy = rng.standard_normal((S, nt_max, R)), rng.standard_normal((S, nt_max, R))
    for k, d in enumerate(insts):  # frames past an instance's steps carry no weight
        wx[k, d["nt"]:] = 0.0
        wy[k, d["nt"]:] = 0.0
    return wx, wy


def _run_canvas(insts, geom, wx, wy):
    C = torch.tensor(np.stack([d["C"] for d in insts]), dtype=torch.float32, device=DEV, requires_grad=True)
    rho = torch.full((len(insts),), RHO, dtype=torch.float32, device=DEV)
    ux, uy = E.propagate(C, rho, geom)
    L = (ux.double() * torch.as_tensor(wx, device=DEV)).sum() + (uy.double() * torch.as_tensor(wy, device=DEV)).sum()
    L.backward()
    torch.cuda.synchronize()
    return ux.detach().cpu().numpy(), uy.detach().cpu().numpy(), C.grad.double().cpu().numpy()


def _run_single(d, wx, wy, ckpt_k=None):
    C = torch.tensor(d["C"], dtype=torch.float32, device=DEV, requires_grad=True)
    ux, uy = E.propagate(C, torch.tensor(RHO, device=DEV), _single(d, ckpt_k))
    L = (ux.double() * torch.as_tensor(wx, device=DEV)).sum() + (uy.double() * torch.as_tensor(wy, device=DEV)).sum()
    L.backward()
    return ux.detach().cpu().numpy()[0], uy.detach().cpu().numpy()[0], C.grad.double().cpu().numpy()


@pytest.mark.parametrize("ckpt_k", [None, 7, 40])
def test_instances_equal_each_instance_run_alone(ckpt_k):
    insts = _instances(SPECS)
    geom = _canvas(insts, ckpt_k)
    wx, wy = _weights(insts, geom.nt)
    cx, cy, cg = _run_canvas(insts, geom, wx, wy)
    assert E.load_library().ernn_last_path() == E.PATH_TILED
    for k, d in enumerate(insts):
        nt = d["nt"]
        sx, sy, sg = _run_single(d, wx[k:k + 1, :nt], wy[k:k + 1, :nt], ckpt_k)
        # the same kernels over the same tiles of the instance: the same traces
        assert rel(cx[k, :nt], sx) <= 1e-6 and rel(cy[k, :nt], sy) <= 1e-6, (k, rel(cx[k, :nt], sx))
        assert not np.any(cx[k, nt:]) and not np.any(cy[k, nt:])  # past its steps: zero
        # imaging sums grouped per CTA chunk of the table (FP64 across chunks)
        assert rel(cg[k], sg) <= 1e-6, (k, rel(cg[k], sg))


def test_instances_vs_fp64_oracle():
    insts = _instances(SPECS, seed=5)
    geom = _canvas(insts, ckpt_k=25)
    wx, wy = _weights(insts, geom.nt)
    cx, cy, cg = _run_canvas(insts, geom, wx, wy)
    for k, d in enumerate(insts):
        nt = d["nt"]
        case = O.Case(d["nx"], d["ny"], nt, H, DT, RHO, d["C"], d["sig"][None].astype(np.float64),
                      d["smap"][None].astype(np.float64), np.array([d["org"]], np.int32),
                      record=O.RECORD_RECEIVERS, rec_idx=d["rec"][None])
        ox, oy, st = O.forward(case, "f64", keep_states=True)
        gC, _ = O.adjoint(case, st, wx[k:k + 1, :nt], wy[k:k + 1, :nt], "f64")
        assert rel(cx[k:k + 1, :nt], ox) <= 1e-4 and rel(cy[k:k + 1, :nt], oy) <= 1e-4
        assert rel(cg[k], gC) <= 1e-4, (k, rel(cg[k], gC))


def test_instance_layout_is_checked():
    insts = _instances(SPECS[:2])
    geom = _canvas(insts)
    C = torch.tensor(np.stack([d["C"] for d in insts]), dtype=torch.float32, device=DEV)
    rho = torch.full((2,), RHO, dtype=torch.float32, device=DEV)
    i = geom.instances
    bad = [Instances(i.x0, [i.y0[0], i.y0[1] + 2], i.nx, i.ny, i.nt),           # y0 % 4
           Instances([0, 0], [0, 0], i.nx, i.ny, i.nt),                         # overlap
           Instances(i.x0, i.y0, i.nx, i.ny, [i.nt[0], geom.nt + 1])]           # steps > nt
    for b in bad:
        g = E.Geometry(**{**geom.__dict__, "instances": b, "_checked": False})
        with pytest.raises(_lib.ErnnError):
            with torch.no_grad():
                E.propagate(C, rho, g)


def test_canvas_inversion_graph_replay_equals_eager():
    ws = lambda: Hn.multi_instances(5, sides=[128, 192, 128, 256, 192])
    g = Hn.CanvasInversion(ws(), DEV, graph=True, nt=300)   # warm-up steps, then capture
    theta = g.theta.detach().clone()
    loss_g = float(g.step())
    grad_g = g.gradient().detach().double().cpu().numpy()
    e = Hn.CanvasInversion(ws(), DEV, graph=False, nt=300)
    with torch.no_grad():
        e.theta.copy_(theta)
    loss_e = float(e.step())
    grad_e = e.gradient().detach().double().cpu().numpy()
    assert np.isfinite(loss_g) and abs(loss_g - loss_e) <= 1e-6 * abs(loss_e), (loss_g, loss_e)
    assert rel(grad_g, grad_e) <= 1e-6, rel(grad_g, grad_e)
    E.check_device_status()


def test_canvas_set_parts_equal_single_canvases():
    # two canvases of about equal work on their own streams, one graph: each
    # part's loss and gradient equal those of a canvas of the same instances
    # run alone (same kernels, same constants), and the set's gradient comes
    # back in the instances' order
    ws = Hn.multi_instances(6, sides=[128, 192, 128, 256, 192, 128])
    cs = Hn.CanvasSet(ws, DEV, parts=2, graph=True, nt=300)
    assert sorted(k for m in cs.members for k in m) == list(range(len(ws)))
    theta = [p.theta.detach().clone() for p in cs.parts]
    loss = float(cs.step())
    grad = cs.gradient().detach().double().cpu().numpy().reshape(len(ws), 6)
    total = 0.0
    for members, th in zip(cs.members, theta):
        ref = Hn.CanvasInversion([ws[k] for k in members], DEV, graph=False, nt=300,
                                 budget_fraction=0.4 / len(cs.members))
        with torch.no_grad():
            ref.theta.copy_(th)
        total += float(ref.step())
        g = ref.gradient().detach().double().cpu().numpy().reshape(len(members), 6)
        assert rel(grad[members], g) <= 1e-6, rel(grad[members], g)
    assert np.isfinite(loss) and abs(loss - total) <= 1e-6 * abs(total), (loss, total)
    E.check_device_status()


def test_instances_ignore_stale_workspace():
    # Only the instances' ghost rings of the stored and recomputed states are
    # zeroed per call: the rest of the canvas outside the regions may hold
    # anything.  Fill the caching allocator's free blocks with NaN so the
    # next run's tape and scratch come from them: traces and gradients must
    # be bitwise those of a run on fresh memory.
    insts = _instances(SPECS, seed=7)
    geom = _canvas(insts, ckpt_k=25)
    wx, wy = _weights(insts, geom.nt)
    ref = _run_canvas(insts, geom, wx, wy)
    torch.cuda.empty_cache()
    junk = [torch.full((n << 18,), float("nan"), device=DEV) for n in (1, 2, 4, 8, 16, 32, 64, 128) for _ in range(2)]
    torch.cuda.synchronize()
    del junk
    out = _run_canvas(insts, geom, wx, wy)
    for a, b in zip(ref, out):
        assert np.array_equal(a, b)
    E.check_device_status()
