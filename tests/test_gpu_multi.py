"""Many uneven inversions in one CUDA-graph-captured iteration (GPU only).

The captured iteration must give the gradients of the same iteration run
eagerly, with instances served by each kernel path: a 128^2 instance fits the
cluster-resident path, 512^2 runs the plain per-step kernels (fewer tiles than
SMs), 768^2 the tiled TMA kernels.
"""
import numpy as np
import pytest
import torch

from cases import rel
from ernn_gb300 import harness as Hn

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _instances():
    ws = Hn.multi_instances(n=3, sides=[128, 512, 768])
    for w in ws:
        w.nt = 160
    return ws


def test_graph_captured_iteration_matches_eager():
    g = Hn.MultiInversion(_instances(), DEV, graph=True)   # warm-up steps, then capture
    theta = [inv.params.theta.detach().clone() for inv in g.invs]
    loss_g = float(g.step())
    torch.cuda.synchronize()
    grad_g = g.gradient().detach().cpu().numpy().astype(np.float64)
    assert np.isfinite(loss_g) and np.all(np.isfinite(grad_g))

    e = Hn.MultiInversion(_instances(), DEV, graph=False)
    with torch.no_grad():
        for inv, t in zip(e.invs, theta):
            inv.params.theta.copy_(t)
    loss_e = float(e.step())
    grad_e = e.gradient().detach().cpu().numpy().astype(np.float64)
    assert abs(loss_g - loss_e) <= 1e-6 * abs(loss_e), (loss_g, loss_e)
    assert rel(grad_g, grad_e) <= 1e-6, rel(grad_g, grad_e)
    Hn.check_device_status()


def test_grouped_instances_match_separate_runs():
    # two instances of one size run as the shots of one call with per-shot
    # constants; their losses and gradients equal those of separate calls
    def ws():
        out = Hn.multi_instances(n=3, sides=[192, 192, 256])
        for w in out:
            w.nt = 150
        return out
    g = Hn.MultiInversion(ws(), DEV, graph=False, group=True)
    e = Hn.MultiInversion(ws(), DEV, graph=False, group=False)
    assert len(g.groups) == 2 and len(e.groups) == 3
    lg, le = float(g.step()), float(e.step())
    assert abs(lg - le) <= 1e-6 * abs(le), (lg, le)
    gg = g.gradient().detach().cpu().numpy().astype(np.float64)
    ge = e.gradient().detach().cpu().numpy().astype(np.float64)
    assert rel(gg, ge) <= 1e-5, rel(gg, ge)


@pytest.mark.parametrize("make", ["plate", "damage"])
def test_graphed_iteration_matches_eager(make):
    if make == "plate":
        w = Hn.plate128()
        w.nt = 300
    else:
        w = Hn.Workload("damage128", 128, 128, 200, Hn.C_ORTHO.copy(), Hn._top(2, 128, 128, margin=16),
                        Hn._top(16, 128, 128), D_true=Hn.damage_map(128, 128))
    g = Hn.make_inversion(w, DEV)
    g.capture()
    e = Hn.make_inversion(w, DEV)
    param = (lambda inv: inv.params.theta) if make == "plate" else (lambda inv: inv.D)
    with torch.no_grad():
        param(e).copy_(param(g))
    lg = float(g.step())                 # graph replay
    le = float(e.step_eager())
    assert abs(lg - le) <= 1e-6 * abs(le), (lg, le)
    gg = g.gradient().detach().double().cpu().numpy()
    ge = e.gradient().detach().double().cpu().numpy()
    assert rel(gg, ge) <= 1e-6, rel(gg, ge)
    Hn.check_device_status()
