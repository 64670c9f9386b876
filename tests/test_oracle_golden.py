"""Pin the oracle against golden vectors produced by the reference module itself.

The fixtures come from tests/golden/make_golden.py, which imports
Parameter_inversion/Inversion_adam.py and extracts the definitions of
Damage_inversion/Inversion_adam.py, runs them on the CPU in FP32 and in the
FP64 run of the same scheme, and stores inputs, histories and autograd
gradients.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O

# FP64 oracle vs FP64 reference: identical scheme, so agreement to rounding.
# Reference gradients w.r.t. the float32 log-parameters are rounded to float32,
# hence the looser gradient bound.
TOL = {"f64": dict(fwd=1e-12, grad=2e-6), "f32": dict(fwd=1e-5, grad=5e-5)}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def load(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_operator_scalar(tag):
    g = load(f"operator_{tag}.npz")
    Lx, Ly = O.operator(int(g["nx"]), int(g["ny"]), float(g["h"]), g["C"], g["ux"], g["uy"],
                        g["fx"], g["fy"], float(g["rho"]), precision=tag)
    assert rel(Lx, g["Lux"]) < TOL[tag]["fwd"]
    assert rel(Ly, g["Luy"]) < TOL[tag]["fwd"]


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_operator_fields_force_transposed(tag):
    # Damage_inversion/Inversion_adam.py:169-174 adds force.transpose(1, 2).
    g = load(f"operator_{tag}.npz")
    n = int(g["nsq"])
    Lx, Ly = O.operator(n, n, float(g["h"]), g["C_fields"], g["vx"], g["vy"], g["gx"].T,
                        g["gy"].T, float(g["rho"]), mode=O.MODE_FIELDS, precision=tag)
    assert rel(Lx, g["Lux_fields"]) < TOL[tag]["fwd"]
    assert rel(Ly, g["Luy_fields"]) < TOL[tag]["fwd"]
    # and the untransposed force does NOT reproduce the reference
    Lx2, _ = O.operator(n, n, float(g["h"]), g["C_fields"], g["vx"], g["vy"], g["gx"], g["gy"],
                        float(g["rho"]), mode=O.MODE_FIELDS, precision=tag)
    assert rel(Lx2, g["Lux_fields"]) > 1e-3


def _param_case(g):
    return O.Case(int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["h"]), float(g["dt"]),
                  float(g["rho"]), g["C"], g["signal"][None], g["gauss"][None],
                  np.array([[0, 0]]), stride=int(g["stride"]))


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_param_inversion_forward_and_gradient(tag):
    g = load(f"param_inversion_{tag}.npz")
    case = _param_case(g)
    ux, uy, states = O.forward(case, tag, keep_states=True)
    assert ux.shape == g["hist_ux"].shape
    assert rel(ux, g["hist_ux"]) < TOL[tag]["fwd"]
    assert rel(uy, g["hist_uy"]) < TOL[tag]["fwd"]
    ts, ss = int(g["ts"]), int(g["ss"])
    gx = O.history_grad(ux, g["target_ux"], ts, ss)
    gy = O.history_grad(uy, g["target_uy"], ts, ss)
    gC, _ = O.adjoint(case, states, gx, gy, tag)
    # reference gradient is w.r.t. log C: dL/dlogC = C dL/dC (clamp inactive)
    assert rel(gC * g["C"], g["grad_log"]) < TOL[tag]["grad"]
    assert np.all(np.sign(gC * g["C"]) == np.sign(g["grad_log"]))


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_damage_inversion_forward_and_gradient(tag):
    g = load(f"damage_inversion_{tag}.npz")
    case = O.Case(int(g["nx"]), int(g["ny"]), int(g["nt"]), float(g["h"]), float(g["dt"]),
                  float(g["rho"]), g["C_fields"], g["signal"][None], g["gauss"].T[None],
                  np.array([[0, 0]]), stride=int(g["stride"]), mode=O.MODE_FIELDS)
    ux, uy, states = O.forward(case, tag, keep_states=True)
    assert rel(ux, g["hist_ux"]) < TOL[tag]["fwd"]
    assert rel(uy, g["hist_uy"]) < TOL[tag]["fwd"]
    ts = int(g["ts"])
    gx = O.history_grad(ux, g["target_ux"], ts, 1, 5.0)   # 5 MSE(ux) + MSE(uy)
    gy = O.history_grad(uy, g["target_uy"], ts, 1)
    gC, _ = O.adjoint(case, states, gx, gy, tag)
    assert rel(gC * g["C_fields"], g["grad_log"]) < TOL[tag]["grad"]


def test_fp32_vs_fp64_gap_is_small():
    """The FP64 run of the same scheme is the accuracy reference; FP32 sits within 1e-5."""
    g = load("param_inversion_f32.npz")
    case = _param_case(g)
    a, _, _ = O.forward(case, "f32")
    b, _, _ = O.forward(case, "f64")
    assert rel(a, b) < 1e-5
