"""Wavefield and trace file formats (CPU)."""
import os

import numpy as np
import pytest
import torch

from ernn_gb300 import formats as EIO


def _fields(nt=7, nx=6, ny=5, seed=0):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((nt, nx, ny)).astype(np.float32),
            rng.standard_normal((nt, nx, ny)).astype(np.float32))


def test_npz_round_trip_and_reference_contract(tmp_path):
    ux, uy = _fields()
    x = np.linspace(-1, 1, 6)
    y = np.linspace(-2, 2, 5)
    t = np.arange(7) * 2.5e-8
    info = {"source_f0": 1e6, "C11": 1.3e11, "source_indices": np.array([3, 4])}
    path = EIO.save_wavefields(str(tmp_path / "anisotropic_ricker_data_ds5_FEM_fixed_bc.npz"),
                               ux, uy, x, y, t, info)
    a, b, meta = EIO.load_reference_data(path, device="cpu")
    assert a.shape == (1, 7, 6, 5) and a.dtype == torch.float32
    assert np.array_equal(a[0].numpy(), ux) and np.array_equal(b[0].numpy(), uy)
    assert meta["primary_stride"] == 5 and meta["noise_added"] is False
    assert np.allclose(meta["t_primary"], t.astype(np.float32))
    assert float(meta["source_info"]["source_f0"]) == 1e6
    assert np.array_equal(meta["source_info"]["source_indices"], [3, 4])


def test_stride_from_name():
    assert EIO.primary_stride("/d/anisotropic_data_ds12_x.mat") == 12
    assert EIO.primary_stride("plain.npz") == EIO.DEFAULT_STRIDE


def test_noise_at_target_snr():
    g = torch.Generator().manual_seed(0)
    s = torch.sin(torch.linspace(0, 60, 200000))
    noisy, noise = EIO.add_noise_snr(s, 20.0, g)
    snr = 10 * torch.log10(torch.mean(s ** 2) / torch.mean(noise ** 2))
    assert abs(float(snr) - 20.0) < 0.05
    assert torch.allclose(noisy - noise, s)


def test_load_with_noise(tmp_path):
    ux, uy = _fields(nt=50, nx=20, ny=20)
    path = EIO.save_wavefields(str(tmp_path / "f_ds2"), ux, uy, np.zeros(20), np.zeros(20), np.zeros(50))
    assert path.endswith(".npz")
    a, b, meta = EIO.load_reference_data(path, add_noise=True, snr_db=30.0, device="cpu",
                                         generator=torch.Generator().manual_seed(1))
    assert meta["noise_added"] and meta["snr_db"] == 30.0 and meta["primary_stride"] == 2
    assert meta["noise_ux"].shape == (1, 50, 20, 20)


def test_hdf5_form_when_available(tmp_path):
    pytest.importorskip("h5py")
    ux, uy = _fields()
    path = EIO.save_wavefields(str(tmp_path / "w_ds5.mat"), ux, uy, np.zeros(6), np.zeros(5), np.zeros(7),
                               {"rho": 1560.0})
    a, b, meta = EIO.load_reference_data(path, device="cpu")
    assert np.array_equal(a[0].numpy(), ux) and float(meta["source_info"]["rho"]) == 1560.0


def test_traces_from_history_and_trace_files(tmp_path):
    S, T, nx, ny = 2, 4, 5, 6
    h = torch.arange(S * T * nx * ny, dtype=torch.float32).reshape(S, T, nx, ny)
    rec = torch.tensor([[0, 7, 29], [5, 6, 12]], dtype=torch.int32)
    tx, ty = EIO.traces_from_history(h, -h, rec)
    assert tx.shape == (S, T, 3)
    for s in range(S):
        for r in range(3):
            i, j = divmod(int(rec[s, r]), ny)
            assert torch.equal(tx[s, :, r], h[s, :, i, j]) and torch.equal(ty[s, :, r], -h[s, :, i, j])
    p = EIO.save_traces(str(tmp_path / "tr"), tx.numpy(), ty.numpy(), rec.numpy(), 3, 5e-9)
    a, b, r2, stride, dt = EIO.load_traces(p, device="cpu")
    assert torch.equal(a, tx) and torch.equal(r2, rec) and stride == 3 and dt == 5e-9


def test_missing_file_raises(tmp_path):
    with pytest.raises(FileNotFoundError):
        EIO.load_reference_data(str(tmp_path / "none_ds5.npz"), device="cpu")


def test_total_variation_matches_definition():
    from ernn_gb300 import total_variation_2d
    f = torch.tensor(np.random.default_rng(3).standard_normal((2, 7, 5)))
    a = f.numpy()
    ref = np.abs(np.diff(a, axis=1)).sum() + np.abs(np.diff(a, axis=2)).sum()
    assert abs(float(total_variation_2d(f)) - ref) <= 1e-12 * ref
