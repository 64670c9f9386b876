"""FEM generator oracle against the reference solver's own output (CPU)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from cases import rel
from oracle import fem as OF


@pytest.mark.parametrize("name", ["fem", "fem_cfl"])
@pytest.mark.parametrize("precision,tol", [("f32", 1e-5), ("f64", 1e-5)])
def test_fem_oracle_matches_reference_solver(name, precision, tol):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    fx, fy = OF.fem_forward(int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["dx"]), float(g["dy"]),
                            float(g["dt"]), float(g["rho"]), g["C"], g["load"], g["signal"],
                            precision=precision)
    rx = np.transpose(g["ux"], (2, 0, 1))
    ry = np.transpose(g["uy"], (2, 0, 1))
    assert rel(fx, rx) <= tol and rel(fy, ry) <= tol, (rel(fx, rx), rel(fy, ry))


def test_fem_oracle_frames_stride_and_edges():
    g = np.load(os.path.join(GOLDEN, "fem.npz"))
    args = (int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["dx"]), float(g["dy"]), float(g["dt"]),
            float(g["rho"]), g["C"], g["load"], g["signal"])
    full_x, _ = OF.fem_forward(*args)
    sub_x, _ = OF.fem_forward(*args, stride=5)
    assert sub_x.shape[0] == (int(g["nt"]) + 4) // 5
    assert np.array_equal(sub_x, full_x[::5])
    assert np.all(full_x[:, 0, :] == 0) and np.all(full_x[:, -1, :] == 0)   # fixed edges
    assert np.all(full_x[:, :, 0] == 0) and np.all(full_x[:, :, -1] == 0)
    assert np.all(full_x[:2] == 0)                                           # u^0 = u^1 = 0


def test_fem_oracle_damaged_plate_matches_reference_solver():
    from ernn_gb300 import fem as EF
    g = np.load(os.path.join(GOLDEN, "fem_damage.npz"))
    C = [float(c) for c in g["C"]]
    Cf = np.stack(EF.apply_damage_to_stiffness(*C, g["damage_mask"], reduction_factor=0.5))
    for precision in ("f32", "f64"):
        fx, fy = OF.fem_forward(int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["dx"]), float(g["dy"]),
                                float(g["dt"]), float(g["rho"]), g["C"], g["load"], g["signal"],
                                precision=precision, C_fields=Cf)
        rx = np.transpose(g["ux"], (2, 0, 1))
        ry = np.transpose(g["uy"], (2, 0, 1))
        assert rel(fx, rx) <= 1e-5 and rel(fy, ry) <= 1e-5, (precision, rel(fx, rx), rel(fy, ry))
    # the damage changes the field: the uniform plate is far from it
    ux0, _ = OF.fem_forward(int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["dx"]), float(g["dy"]),
                            float(g["dt"]), float(g["rho"]), g["C"], g["load"], g["signal"])
    assert rel(ux0, np.transpose(g["ux"], (2, 0, 1))) > 1e-3
