"""FEM data generator on the GPU against the reference solver's output and the
FP64 restatement (GPU only)."""
import os

import numpy as np
import pytest
import torch

from cases import rel
from conftest import GOLDEN
from ernn_gb300 import fem as EF
from ernn_gb300 import formats
from oracle import fem as OF

pytestmark = pytest.mark.gpu
TOL = 5e-5  # FP32 run; the reference's own FP32 run is 1.5e-6 from the FP64 scheme


def _args(g):
    return (int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["dx"]), float(g["dy"]), float(g["dt"]),
            float(g["rho"]), g["C"], g["load"], g["signal"])


@pytest.mark.parametrize("name", ["fem", "fem_cfl"])
def test_fem_frames_match_reference_solver(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    fx, fy = EF.fem_frames(*_args(g))
    rx = np.transpose(g["ux"], (2, 0, 1))
    ry = np.transpose(g["uy"], (2, 0, 1))
    ex, ey = rel(fx.cpu().numpy(), rx), rel(fy.cpu().numpy(), ry)
    assert ex <= TOL and ey <= TOL, (ex, ey)


@pytest.mark.parametrize("stride", [1, 5])
def test_fem_frames_match_fp64_oracle_larger_grid(stride):
    nx, ny, nt = 70, 52, 240
    dx = dy = 1e-3
    x = np.linspace(-(nx - 1) * dx / 2, (nx - 1) * dx / 2, nx)
    y = np.linspace(-(ny - 1) * dy / 2, (ny - 1) * dy / 2, ny)
    X, Y = np.meshgrid(x, y, indexing="ij")
    load = EF.gaussian_point_load(X, Y, 0.004, -0.003, 5e5).astype(np.float32)
    t = np.arange(nt) * 5e-8
    sig = EF.ricker_wavelet(t, 500e3, 2e-6, 1e10).astype(np.float32)
    C = (130.74e9, 11.5e9, 10.49e9, 30.67e9, 3.75e9, 14.77e9)
    fx, fy = EF.fem_frames(nx, ny, nt, dx, dy, 5e-8, 1610.0, C, load, sig, stride=stride)
    ox, oy = OF.fem_forward(nx, ny, nt, dx, dy, 5e-8, 1610.0, C, load, sig, stride=stride)
    assert fx.shape == ox.shape
    ex, ey = rel(fx.cpu().numpy(), ox), rel(fy.cpu().numpy(), oy)
    assert ex <= TOL and ey <= TOL, (ex, ey)


def test_solver_contract_and_data_file(tmp_path):
    g = np.load(os.path.join(GOLDEN, "fem_cfl.npz"))
    kw = {k[4:]: g[k] for k in g.files if k.startswith("arg_")}
    kw = {k: (tuple(float(a) for a in v) if k == "source_position" else
              (int(v) if k in ("nx", "ny", "nt") else float(v))) for k, v in kw.items()}
    x, y, t, ux, uy, tot, mask, src, nodes, elements, info = \
        EF.solve_2d_anisotropic_wave_fem_ricker_fixed(**kw)
    nx, ny, nt = kw["nx"], kw["ny"], int(g["nt"])
    assert ux.shape == (nx, ny, nt) and len(t) == nt
    assert rel(ux, g["ux"]) <= TOL and rel(uy, g["uy"]) <= TOL
    assert np.array_equal(elements, g["elements"]) and info["max_u_boundary"] == 0.0
    path = EF.generate_data_file(str(tmp_path), stride=5, **kw)
    assert "_ds5_" in os.path.basename(path)
    a, b, meta = formats.load_reference_data(path, device="cuda")
    assert meta["primary_stride"] == 5 and a.shape == (1, (nt + 4) // 5, nx, ny)
    assert rel(a[0].cpu().numpy(), np.moveaxis(ux, 2, 0)[::5]) <= 1e-7
    assert np.allclose(meta["t_primary"], t[::5].astype(np.float32))


def test_fem_refuses_cpu_device():
    with pytest.raises(RuntimeError):
        EF.fem_frames(4, 4, 3, 1e-3, 1e-3, 1e-8, 1.0, (1, 1, 1, 1, 1, 1), np.zeros((4, 4)), np.zeros(3),
                      device="cpu")


def test_damaged_plate_matches_reference_solver(tmp_path):
    g = np.load(os.path.join(GOLDEN, "fem_damage.npz"))
    kw = {k[4:]: g[k] for k in g.files if k.startswith("arg_")}
    kw = {k: (tuple(float(a) for a in v) if k == "source_position" else
              (int(v) if k in ("nx", "ny", "nt") else float(v))) for k, v in kw.items()}
    cfg = [{"type": str(tp), "center": tuple(c), "size": float(sz), "reduction_factor": float(f)}
           for tp, c, sz, f in zip(g["damage_types"], g["damage_centers"], g["damage_sizes"],
                                   g["damage_factors"])]
    x, y, t, ux, uy, tot, mask, src, nodes, elements, info = \
        EF.solve_2d_anisotropic_wave_fem_ricker_fixed(damage_configs=cfg, **kw)
    assert np.array_equal(info["damage_mask"], g["damage_mask"])
    assert rel(ux, g["ux"]) <= TOL and rel(uy, g["uy"]) <= TOL, (rel(ux, g["ux"]), rel(uy, g["uy"]))
    path = EF.generate_data_file(str(tmp_path), stride=5, damage_configs=cfg, **kw)
    assert "damage_data_ds5" in os.path.basename(path)
    with np.load(path) as z:
        assert np.array_equal(z["damage_mask"], g["damage_mask"].astype(np.uint8))
        assert int(z["damage_info/total_damaged_points"]) == int(g["damage_mask"].sum())


def _plate(nx, ny, nt):
    """Arguments of fem_frames for a Gaussian load near the centre of an
    nx x ny plate with the constants of the larger-grid test."""
    dx = dy = 1e-3
    x = np.linspace(-(nx - 1) * dx / 2, (nx - 1) * dx / 2, nx)
    y = np.linspace(-(ny - 1) * dy / 2, (ny - 1) * dy / 2, ny)
    X, Y = np.meshgrid(x, y, indexing="ij")
    load = EF.gaussian_point_load(X, Y, 0.004, -0.003, 5e5).astype(np.float32)
    sig = EF.ricker_wavelet(np.arange(nt) * 5e-8, 500e3, 2e-6, 1e10).astype(np.float32)
    C = (130.74e9, 11.5e9, 10.49e9, 30.67e9, 3.75e9, 14.77e9)
    return nx, ny, nt, dx, dy, 5e-8, 1610.0, C, load, sig


def test_fem_frames_match_fp64_oracle_generator_grid():
    """The generator's 301^2 grid, 300 levels, against the FP64 restatement
    of the generator loop."""
    args = _plate(301, 301, 300)
    fx, fy = EF.fem_frames(*args, stride=5)
    ox, oy = OF.fem_forward(*args, stride=5)
    ex, ey = rel(fx.cpu().numpy(), ox), rel(fy.cpu().numpy(), oy)
    assert ex <= TOL and ey <= TOL, (ex, ey)
