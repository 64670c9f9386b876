"""Fused misfit (ernn_misfit / ernn_misfit_grad through series_misfit) against
the reference's compute_loss methods (golden vectors), the FP64 oracle and
size-independent properties at the damage loop's full size.  GPU only.

Tolerances: the loss sums FP32 squares of FP32 differences in FP64, so it
agrees with the FP64 oracle to ~1e-7 relative (bound 1e-6); gradients are
FP32 products, 1e-6 relative."""
import os

import numpy as np
import pytest
import torch

from cases import rel
from conftest import GOLDEN
from ernn_gb300.misfit import series_misfit
from oracle import misfit as OM

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
LOSS_TOL = 1e-6
GRAD_TOL = 1e-6


def _t(a, grad=False):
    return torch.tensor(np.asarray(a, np.float32), device=DEV, requires_grad=grad)


def _run(px, py, ox, oy, wx, wy, ts, ss):
    ax, ay = _t(px, True), _t(py, True)
    loss = series_misfit(ax, ay, _t(ox), _t(oy), wx, wy, ts, ss)
    loss.backward()
    return float(loss), ax.grad.cpu().numpy(), ay.grad.cpu().numpy()


@pytest.mark.parametrize("tag,wx,use_ss", [("param", 1.0, True), ("damage", 5.0, False)])
def test_matches_reference_compute_loss(tag, wx, use_ss):
    g = np.load(os.path.join(GOLDEN, "misfit.npz"))
    ts, ss = int(g["ts"]), (int(g["ss"]) if use_ss else 1)
    loss, gx, gy = _run(g["px"], g["py"], g["tx"], g["ty"], wx, 1.0, ts, ss)
    ref = float(g[f"{tag}_loss"])
    assert abs(loss - ref) <= 2e-6 * abs(ref), (loss, ref)
    assert rel(gx, g[f"{tag}_gx"]) <= 1e-5 and rel(gy, g[f"{tag}_gy"]) <= 1e-5


CASES = {
    "traces": ((1, 2000, 64), 1, 1),
    "traces_multishot_ts3": ((3, 101, 17), 3, 1),
    "history_ts2": ((1, 41, 30, 33), 2, 1),
    "history_ts2_ss8_ragged": ((2, 23, 45, 37), 2, 8),
    "history_ss3": ((1, 5, 31, 29), 1, 3),
    "frames_below_stride": ((2, 3, 8, 8), 5, 2),
    "single_element": ((1, 1, 1, 1), 1, 1),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("w", [(1.0, 1.0), (5.0, 1.0)])
def test_matches_fp64_oracle(name, w):
    shape, ts, ss = CASES[name]
    rng = np.random.default_rng(len(name))
    px, py, ox, oy = (rng.standard_normal(shape).astype(np.float32) for _ in range(4))
    loss, gx, gy = _run(px, py, ox, oy, w[0], w[1], ts, ss)
    rl, _, _, rgx, rgy = OM.misfit(px, py, ox, oy, w[0], w[1], ts, ss)
    assert abs(loss - rl) <= LOSS_TOL * abs(rl), (loss, rl)
    assert rel(gx, rgx) <= GRAD_TOL and rel(gy, rgy) <= GRAD_TOL
    assert np.array_equal(gx == 0, rgx == 0)  # zero exactly off the counted elements


def test_parts_and_their_gradients():
    rng = np.random.default_rng(1)
    shape = (2, 12, 9, 10)
    px, py, ox, oy = (rng.standard_normal(shape).astype(np.float32) for _ in range(4))
    ax, ay = _t(px, True), _t(py, True)
    loss, ms = series_misfit(ax, ay, _t(ox), _t(oy), 5.0, 1.0, 2, 1, parts=True)
    (0.5 * loss + 3.0 * ms[0] - 2.0 * ms[1]).backward()
    _, mx, my, gx5, gy1 = OM.misfit(px, py, ox, oy, 5.0, 1.0, 2)
    _, _, _, gx1, _ = OM.misfit(px, py, ox, oy, 1.0, 1.0, 2)
    assert abs(float(ms[0]) - mx) <= LOSS_TOL * mx and abs(float(ms[1]) - my) <= LOSS_TOL * my
    assert rel(ax.grad.cpu().numpy(), 0.5 * gx5 + 3.0 * gx1) <= GRAD_TOL
    assert rel(ay.grad.cpu().numpy(), 0.5 * gy1 - 2.0 * gy1) <= GRAD_TOL


def test_reproducible_and_graph_capturable():
    g = torch.Generator(device=DEV).manual_seed(3)
    px, py, ox, oy = (torch.randn((1, 300, 64), device=DEV, generator=g) for _ in range(4))
    a = series_misfit(px, py, ox, oy)
    b = series_misfit(px, py, ox, oy)
    assert torch.equal(a, b)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        series_misfit(px, py, ox, oy)
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        c = series_misfit(px, py, ox, oy)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(a, c)


def test_damage_loop_size_against_torch_fp64():
    # the reference's damage loop: (1, 801, 301, 301) histories, every 2nd frame, 5:1
    g = torch.Generator(device=DEV).manual_seed(4)
    shape = (1, 801, 301, 301)
    px = torch.randn(shape, device=DEV, generator=g, requires_grad=True)
    py = torch.randn(shape, device=DEV, generator=g, requires_grad=True)
    ox = torch.randn(shape, device=DEV, generator=g)
    oy = torch.randn(shape, device=DEV, generator=g)
    loss = series_misfit(px, py, ox, oy, 5.0, 1.0, 2)
    loss.backward()
    with torch.no_grad():
        dx = (px[:, ::2].double() - ox[:, ::2].double())
        dy = (py[:, ::2].double() - oy[:, ::2].double())
        ref = 5.0 * dx.square().mean() + dy.square().mean()
        assert abs(float(loss) - float(ref)) <= LOSS_TOL * float(ref)
        n = dx.numel()
        assert torch.equal(px.grad[:, 1::2], torch.zeros_like(px.grad[:, 1::2]))
        e = (px.grad[:, ::2].double() - 10.0 * dx / n).abs().max() / (10.0 * dx.abs().max() / n)
        assert float(e) <= GRAD_TOL


def test_rejects_bad_inputs():
    a = torch.zeros((1, 4, 6), device=DEV)
    with pytest.raises(RuntimeError, match="CUDA"):
        series_misfit(a.cpu(), a.cpu(), a.cpu(), a.cpu())
    with pytest.raises(ValueError):
        series_misfit(a, a, a, torch.zeros((1, 4, 5), device=DEV))
    with pytest.raises(ValueError):
        series_misfit(a.double(), a.double(), a.double(), a.double())
    with pytest.raises(ValueError):
        series_misfit(a, a, a, a, frame_stride=0)
    with pytest.raises(ValueError):
        series_misfit(a, a, a, a, space_stride=2)  # traces have no grid axes


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_inverter_objectives_match_fixture_losses(tag):
    import ernn_gb300 as E
    g = np.load(os.path.join(GOLDEN, f"param_inversion_{tag}.npz"))
    loss = E.parameter_loss(_t(g["hist_ux"]), _t(g["hist_uy"]), _t(g["target_ux"]), _t(g["target_uy"]),
                            int(g["ts"]), int(g["ss"]))
    assert abs(float(loss) - float(g["loss"])) <= 1e-5 * abs(float(g["loss"]))
    d = np.load(os.path.join(GOLDEN, f"damage_inversion_{tag}.npz"))
    data = series_misfit(_t(d["hist_ux"]), _t(d["hist_uy"]), _t(d["target_ux"]), _t(d["target_uy"]),
                         5.0, 1.0, int(d["ts"]))
    assert abs(float(data) - float(d["loss_data"])) <= 1e-5 * abs(float(d["loss_data"]))
