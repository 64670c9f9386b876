"""Launch overlap of consecutive step kernels (programmatic dependent launch):
with it on, a step kernel is scheduled while the previous one drains and
waits on the device for the previous step's state.  Results must be bitwise
the same with it on and off, on every loop that chains step launches: the
plain kernels (8- and 32-row tiles, all three modes, checkpoint recompute
interleaved with the adjoint), the tiled kernels and the FEM generator's
levels.  Receivers here never share a cell (a shared cell's adjoint sources
are summed in arrival order).  GPU only."""
import numpy as np
import pytest
import torch

import ernn_gb300 as E
from ernn_gb300 import _lib
from cases import random_case, rel
from oracle import oracle as O
from test_gpu_parity import GRAD_TOL, FWD_TOL, run_gpu, run_oracle, weights

pytestmark = pytest.mark.gpu

CASES = {
    "step_scalar_receivers_ckpt": (dict(nx=45, ny=52, nt=90, S=2, record=O.RECORD_RECEIVERS, nrec=11),
                                   E.PATH_STEP, 13),
    "step_fields_dense": (dict(mode=O.MODE_FIELDS, nx=40, ny=44, nt=60, stride=2), E.PATH_STEP, None),
    "step_fields_ckpt": (dict(mode=O.MODE_FIELDS, nx=37, ny=41, nt=70, stride=3), E.PATH_STEP, 9),
    "step_dfield_ckpt": (dict(mode=O.MODE_DFIELD, nx=41, ny=37, nt=60), E.PATH_STEP, 11),
    "step_32row_fields": (dict(mode=O.MODE_FIELDS, nx=512, ny=520, nt=10, S=2, stride=2), E.PATH_STEP, 4),
    "tiled_scalar_receivers_ckpt": (dict(nx=70, ny=132, nt=80, S=3, record=O.RECORD_RECEIVERS, nrec=40),
                                    E.PATH_TILED, 10),
    "tiled_dfield_dense": (dict(mode=O.MODE_DFIELD, nx=45, ny=76, nt=60), E.PATH_TILED, None),
}


def _both(fn):
    """fn() with the overlap on, then off; the setting is restored."""
    was = _lib.launch_overlap(True)
    try:
        on = fn()
        _lib.launch_overlap(False)
        off = fn()
    finally:
        _lib.launch_overlap(was)
    return on, off


@pytest.mark.parametrize("name", list(CASES))
def test_overlap_is_bitwise_neutral(name):
    kw, path, ckpt = CASES[name]
    case = random_case(**kw)
    wx, wy = weights(case)
    on, off = _both(lambda: run_gpu(case, wx, wy, ckpt_k=ckpt, path=path))
    for a, b in zip(on, off):
        assert np.array_equal(a, b)
    assert _lib.load().ernn_last_path() == path
    if case.nx * case.ny <= 64 * 64:
        rx, ry, rg = run_oracle(case, wx, wy)
        assert rel(on[0], rx) <= FWD_TOL and rel(on[1], ry) <= FWD_TOL
        assert rel(on[2], rg) <= GRAD_TOL


@pytest.mark.parametrize("fields", [False, True])
def test_overlap_bitwise_neutral_fem(fields):
    from ernn_gb300 import fem as EF
    nx, ny, nt, dx = 70, 52, 240, 1e-3
    x = np.linspace(-(nx - 1) * dx / 2, (nx - 1) * dx / 2, nx)
    y = np.linspace(-(ny - 1) * dx / 2, (ny - 1) * dx / 2, ny)
    X, Y = np.meshgrid(x, y, indexing="ij")
    load = EF.gaussian_point_load(X, Y, 0.004, -0.003, 5e5).astype(np.float32)
    sig = EF.ricker_wavelet(np.arange(nt) * 5e-8, 500e3, 2e-6, 1e10).astype(np.float32)
    C = (130.74e9, 11.5e9, 10.49e9, 30.67e9, 3.75e9, 14.77e9)
    Cf = None
    if fields:
        rng = np.random.default_rng(3)
        Cf = (np.asarray(C)[:, None, None] * (1 - 0.3 * rng.random((6, nx, ny)))).astype(np.float32)

    def run():
        fx, fy = EF.fem_frames(nx, ny, nt, dx, dx, 5e-8, 1610.0, C, load, sig, stride=5, C_fields=Cf)
        return fx.cpu().numpy(), fy.cpu().numpy()

    on, off = _both(run)
    assert np.array_equal(on[0], off[0]) and np.array_equal(on[1], off[1])
    assert np.abs(on[1]).max() > 0
