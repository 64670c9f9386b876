"""The misfit oracle against the reference's own compute_loss methods
(tests/golden/misfit.npz: both inverters on random histories, with autograd
gradients) and against the loss values stored with the inversion fixtures."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import misfit as OM


def _g(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("tag,wx,ss", [("param", 1.0, None), ("damage", 5.0, 1)])
def test_oracle_matches_reference_compute_loss_and_gradient(tag, wx, ss):
    g = _g("misfit.npz")
    ts = int(g["ts"])
    ss = int(g["ss"]) if ss is None else ss
    loss, mx, my, gx, gy = OM.misfit(g["px"], g["py"], g["tx"], g["ty"], wx, 1.0, ts, ss)
    assert abs(loss - float(g[f"{tag}_loss"])) <= 1e-6 * abs(loss)
    for a, b in ((gx, g[f"{tag}_gx"]), (gy, g[f"{tag}_gy"])):
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-7 * np.abs(b).max())
    # the skipped frames and cells carry no gradient
    assert np.all(gx[:, 1::ts] == 0)


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_oracle_matches_inversion_fixture_losses(tag):
    g = _g(f"param_inversion_{tag}.npz")
    loss = OM.misfit(g["hist_ux"], g["hist_uy"], g["target_ux"], g["target_uy"], 1.0, 1.0,
                     int(g["ts"]), int(g["ss"]))[0]
    assert abs(loss - float(g["loss"])) <= (2e-6 if tag == "f32" else 1e-12) * abs(loss)
    d = _g(f"damage_inversion_{tag}.npz")
    data = OM.misfit(d["hist_ux"], d["hist_uy"], d["target_ux"], d["target_uy"], 5.0, 1.0, int(d["ts"]))[0]
    assert abs(data - float(d["loss_data"])) <= (2e-6 if tag == "f32" else 1e-12) * abs(data)


def test_oracle_rejects_space_stride_on_traces():
    a = np.zeros((1, 4, 5))
    with pytest.raises(ValueError):
        OM.misfit(a, a, a, a, ss=2)
