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
