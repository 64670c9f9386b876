"""Inversion recovers the constants (GPU only).

Plate configuration: 128^2, 1000 steps, orthotropic constants perturbed by up
to 20 % (seeded), 32 top-edge receivers, observations from the same forward at
the true constants plus 0.5 % noise, Adam lr = 1e-2 on normalised constants,
200 iterations through the hand adjoint: every constant must end within 2 %
of its true value (relative to the constant's scale).
"""
import numpy as np
import pytest
import torch

from ernn_gb300 import harness as Hn

pytestmark = pytest.mark.gpu


def test_plate128_recovers_constants_within_two_percent():
    w = Hn.plate128()
    init_err = np.abs(Hn.initial_guess(w) - w.C_true) / Hn.scales(w.C_true)
    C, err, losses = Hn.run_inversion(w, torch.device("cuda:0"), iters=200, lr=1e-2)
    assert np.all(np.isfinite(losses)) and losses[-1] < 0.1 * losses[0]
    assert init_err.max() > 0.05          # the start is genuinely off
    assert err.max() < 0.02, err
    Hn.check_device_status()


def test_rot256_recovers_six_rotated_constants_within_two_percent():
    # configuration 2: the orthotropic plate rotated 30 degrees (all six
    # constants non-zero), 256^2, 2000 steps, checkpoint every 100, 64
    # receivers; Adam lr = 1e-2 on normalised constants through the hand adjoint
    w = Hn.rot256()
    init_err = np.abs(Hn.initial_guess(w) - w.C_true) / Hn.scales(w.C_true)
    C, err, losses = Hn.run_inversion(w, torch.device("cuda:0"), iters=300, lr=1e-2)
    print("rot256 recovery: initial", np.round(init_err, 4), "final", np.round(err, 5),
          "loss", losses[0], "->", losses[-1])
    assert np.all(np.isfinite(losses)) and losses[-1] < 0.1 * losses[0]
    assert init_err.max() > 0.05
    assert err.max() < 0.02, err
    Hn.check_device_status()


def test_damage512_degradation_map_after_100_iterations():
    # configuration 4: D(x, z) from D = 0 over 100 Adam iterations (lr 1e-2)
    # through the D-field adjoint (objective normalised by its initial value);
    # reports the relative error of D inside the damaged ellipses (cells where
    # the true D exceeds 0.05)
    w = Hn.damage512()
    dev = torch.device("cuda:0")
    inv = Hn.DamageInversion(w, dev, lr=1e-2)
    losses = [float(inv.step()) for _ in range(100)]
    D = inv.D.detach().double().cpu().numpy()
    mask = w.D_true > 0.05
    err = float(np.linalg.norm((D - w.D_true)[mask]) / np.linalg.norm(w.D_true[mask]))
    err_all = float(np.linalg.norm(D - w.D_true) / np.linalg.norm(w.D_true))
    print(f"damage512 recovery: D rel err inside ellipses {err:.4f} (all cells {err_all:.4f}), "
          f"loss {losses[0]:.4e} -> {losses[-1]:.4e}")
    assert np.all(np.isfinite(losses)) and losses[-1] < losses[0]
    assert err < 1.0          # moved from D = 0 (error 1) towards the true map
    Hn.check_device_status()
