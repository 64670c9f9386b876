"""FEM generator host side against the reference solver's run (CPU)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from ernn_gb300 import fem as EF


@pytest.mark.parametrize("name", ["fem", "fem_cfl"])
def test_mesh_time_axis_load_and_signal_match_reference(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    kw = {k[4:]: g[k] for k in g.files if k.startswith("arg_")}
    nx, ny = int(kw["nx"]), int(kw["ny"])
    x, y, el, bnd, dx, dy = EF.create_structured_triangular_mesh(nx, ny, float(kw["Lx"]), float(kw["Ly"]))
    assert np.array_equal(el, g["elements"])
    assert np.array_equal(x, g["x"]) and np.array_equal(y, g["y"])
    assert set(bnd.tolist()) == {j * nx + i for j in range(ny) for i in range(nx)
                                 if i in (0, nx - 1) or j in (0, ny - 1)}
    t, dt, nt = EF._time_axis(int(kw["nt"]), float(kw["t_total"]), dx, dy, float(kw["C11"]),
                              float(kw["C22"]), float(kw["C66"]), float(kw["rho"]))
    assert nt == int(g["nt"]) and np.array_equal(t, g["t"])
    X, Y = np.meshgrid(x, y, indexing="ij")
    pos = kw["source_position"]
    gauss = EF.gaussian_point_load(X, Y, float(pos[0]), float(pos[1]), float(kw["gaussian_param"]))
    assert np.array_equal(gauss.astype(np.float32), g["load"])
    sig = EF.ricker_wavelet(t, float(kw["source_f0"]), float(kw["source_t0"]), float(kw["source_amplitude"]))
    assert np.array_equal(sig.astype(np.float32), g["signal"])


def test_fem_abi_validates_before_device_work():
    import ctypes
    from ernn_gb300 import _lib
    lib = _lib.load()
    p = _lib.ErnnFemProblem(21, 21, 100, 5, 1e-3, 1e-3, 5e-8, 1610.0,
                            (ctypes.c_double * 6)(1e11, 1e10, 1e10, 3e10, 4e9, 1.5e10), 0.7)
    assert lib.ernn_fem_workspace_bytes(ctypes.byref(p)) >= 6 * 21 * 21 * 4
    nul = ctypes.c_void_p(0)
    assert lib.ernn_fem_forward(ctypes.byref(p), nul, nul, nul, nul, nul, nul, 0, nul) == 1
    p.nx = 1
    assert lib.ernn_fem_workspace_bytes(ctypes.byref(p)) == 0
    assert lib.ernn_fem_forward(ctypes.byref(p), ctypes.c_void_p(16), ctypes.c_void_p(16), nul,
                                ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                1 << 20, nul) == 1


def test_damage_regions_and_stiffness_match_reference():
    g = np.load(os.path.join(GOLDEN, "fem_damage.npz"))
    nx, ny = int(g["nx"]), int(g["ny"])
    x, y, *_ = EF.create_structured_triangular_mesh(nx, ny, float(g["arg_Lx"]), float(g["arg_Ly"]))
    X, Y = np.meshgrid(x, y, indexing="ij")
    cfg = [{"type": str(tp), "center": tuple(c), "size": float(sz), "reduction_factor": float(f)}
           for tp, c, sz, f in zip(g["damage_types"], g["damage_centers"], g["damage_sizes"],
                                   g["damage_factors"])]
    mask, info = EF.create_damage_regions(X, Y, cfg)
    assert np.array_equal(mask, g["damage_mask"]) and info["total_damaged_points"] == mask.sum()
    C = EF.apply_damage_to_stiffness(1.0, 2.0, 3.0, 4.0, 5.0, 6.0, mask)
    assert C[1][mask].max() == 1.0 and C[1][~mask].min() == 2.0
