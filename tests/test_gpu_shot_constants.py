"""Per-shot constants (ERNN_FLAG_SHOT_CONSTANTS): several independent media of
one grid size advance in the same launches, each shot with its own six
constants and density, each getting its own gradient (GPU only).

Checked shot by shot against single-shot FP64 oracle runs, on every kernel path.
"""
import dataclasses

import numpy as np
import pytest
import torch

import ernn_gb300 as E
from cases import random_case, rel
from oracle import oracle as O
from test_gpu_parity import DEV, FWD_TOL, GRAD_TOL, to_geometry, weights

pytestmark = pytest.mark.gpu


def _per_shot(case, seed=5):
    rng = np.random.default_rng(seed)
    S = case.nshots
    C = np.stack([case.C * rng.uniform(0.85, 1.15, size=6) for _ in range(S)])
    C = C.astype(np.float32).astype(np.float64)
    rho = rng.uniform(1450.0, 1700.0, size=S).astype(np.float32).astype(np.float64)
    return C, rho


def _shot(case, s, C, rho):
    return dataclasses.replace(case, C=C[s], rho=float(rho[s]), src_signal=case.src_signal[s:s + 1],
                               src_map=case.src_map[s:s + 1], src_origin=case.src_origin[s:s + 1],
                               rec_idx=None if case.rec_idx is None else case.rec_idx[s:s + 1])


SHAPES = {
    "receivers": dict(nx=40, ny=64, nt=90, S=3, record=O.RECORD_RECEIVERS, nrec=9),
    "dense_stride": dict(nx=33, ny=68, nt=70, S=2, stride=3),
}


@pytest.mark.parametrize("path", [E.PATH_STEP, E.PATH_RESIDENT, E.PATH_TILED])
@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("ckpt_k", [None, 16])
def test_per_shot_constants_vs_single_shot_oracle(path, shape, ckpt_k):
    case = random_case(**SHAPES[shape])
    C, rho = _per_shot(case)
    wx, wy = weights(case)
    geom = to_geometry(case, ckpt_k, path)
    Ct = torch.tensor(C, dtype=torch.float32, device=DEV, requires_grad=True)
    rt = torch.tensor(rho, dtype=torch.float32, device=DEV)
    ox, oy = E.propagate(Ct, rt, geom)
    L = (ox.double() * torch.as_tensor(wx, device=DEV)).sum() + \
        (oy.double() * torch.as_tensor(wy, device=DEV)).sum()
    L.backward()
    assert Ct.grad.shape == (case.nshots, 6)
    assert E._lib.load().ernn_last_path() == path
    for s in range(case.nshots):
        one = _shot(case, s, C, rho)
        rx, ry, st = O.forward(one, "f64", keep_states=True)
        gC, _ = O.adjoint(one, st, wx[s:s + 1], wy[s:s + 1], "f64")
        gx = ox[s:s + 1].detach().cpu().numpy()
        gy = oy[s:s + 1].detach().cpu().numpy()
        assert rel(gx, rx) <= FWD_TOL and rel(gy, ry) <= FWD_TOL, (s, rel(gx, rx), rel(gy, ry))
        g = Ct.grad[s].detach().cpu().numpy()
        assert rel(g, gC) <= GRAD_TOL, (s, rel(g, gC), g, gC)


def test_per_shot_constants_shared_equals_plain_call():
    # identical constants in every shot: the same states as the shared-constant call
    case = random_case(nx=40, ny=64, nt=60, S=2, record=O.RECORD_RECEIVERS, nrec=7)
    geom = to_geometry(case, None, E.PATH_STEP)
    rho = torch.tensor(case.rho, dtype=torch.float32, device=DEV)
    C1 = torch.tensor(case.C, dtype=torch.float32, device=DEV)
    with torch.no_grad():
        a = E.propagate(C1, rho, geom)
        b = E.propagate(C1[None].repeat(2, 1), rho.reshape(1).repeat(2), geom)
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_autotune_picks_an_eligible_path_and_caches():
    from ernn_gb300 import autotune
    case = random_case(nx=64, ny=128, nt=120, S=2, record=O.RECORD_RECEIVERS, nrec=8)
    geom = to_geometry(case, None, E.PATH_AUTO)
    C = torch.tensor(case.C, dtype=torch.float32, device=DEV)
    rho = torch.tensor(case.rho, dtype=torch.float32, device=DEV)
    path, k, rows = autotune.tune(geom, C, rho, probe_steps=40)
    assert path in (E.PATH_STEP, E.PATH_RESIDENT, E.PATH_TILED) and 1 <= k <= case.nt
    assert rows in (16, 32) and (rows == 16 or path == E.PATH_TILED)
    assert autotune.tune(geom, C, rho) == (path, k, rows)  # cached
    geom.path, geom.ckpt_k, geom.tile_rows = path, k, rows
    with torch.no_grad():
        E.propagate(C, rho, geom)
    assert E._lib.load().ernn_last_path() == path


@pytest.mark.parametrize("per_shot", [False, True])
def test_tall_tiles_match_default_tiles(per_shot):
    # 64 x 32 tiles (ERNN_FLAG_TALL_TILES) against the default 64 x 16 on the
    # tiled path: the same forward states (same arithmetic per cell) and the
    # gradient up to the grouping of the FP32 imaging sums
    case = random_case(nx=70, ny=132, nt=90, S=2, record=O.RECORD_RECEIVERS, nrec=9)
    rho = torch.tensor(case.rho, dtype=torch.float32, device=DEV)
    out = []
    for rows in (16, 32):
        geom = to_geometry(case, 30, E.PATH_TILED)
        geom.tile_rows = rows
        C = torch.tensor(case.C, dtype=torch.float32, device=DEV)
        r = rho
        if per_shot:
            C, r = C[None].repeat(2, 1) * torch.tensor([[1.0], [1.05]], device=DEV), rho.reshape(1).repeat(2)
        C = C.clone().requires_grad_(True)
        ux, uy = E.propagate(C, r, geom)
        (ux.double().square().sum() + uy.double().square().sum()).backward()
        out.append((ux.detach().cpu().numpy(), uy.detach().cpu().numpy(), C.grad.double().cpu().numpy()))
    (ax, ay, ag), (bx, by, bg) = out
    assert np.array_equal(ax, bx) and np.array_equal(ay, by)
    assert rel(bg, ag) <= 1e-6, rel(bg, ag)
