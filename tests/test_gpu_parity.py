"""CUDA path vs the oracle and vs the reference's golden vectors (GPU only).

Tolerances: forward relative L2 error <= 1e-4 against the FP64 run of the
same scheme, gradient relative error <= 1e-4 (the accuracy this library
promises for its FP32 path).  The FP32 CUDA path typically lands near 1e-6.
"""
import ctypes
import os
import sys

import numpy as np
import pytest
import torch

import ernn_gb300 as E
from cases import C_ROT30, random_case, rel
from conftest import GOLDEN
from oracle import oracle as O

pytestmark = pytest.mark.gpu
FWD_TOL = 1e-4
GRAD_TOL = 1e-4
DEV = "cuda:0"


def to_geometry(case: O.Case, ckpt_k=None, path=E.PATH_AUTO) -> E.Geometry:
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(DEV).contiguous()
    return E.Geometry(nx=case.nx, ny=case.ny, nt=case.nt, h=case.h, dt=case.dt,
                      src_signal=t(case.src_signal), src_map=t(case.src_map),
                      src_origin=t(case.src_origin, torch.int32), stride=case.stride,
                      src_comp=case.src_comp,
                      rec_idx=None if case.rec_idx is None else t(case.rec_idx, torch.int32),
                      ckpt_k=ckpt_k, path=path)


def run_gpu(case: O.Case, wx, wy, ckpt_k=None, path=E.PATH_AUTO):
    """Forward + hand adjoint of L = sum(wx*out_x) + sum(wy*out_y) on the GPU."""
    geom = to_geometry(case, ckpt_k, path)
    C = torch.tensor(case.C, dtype=torch.float32, device=DEV, requires_grad=case.mode != O.MODE_DFIELD)
    D = None
    if case.mode == O.MODE_DFIELD:
        D = torch.tensor(case.D, dtype=torch.float32, device=DEV, requires_grad=True)
    rho = torch.tensor(case.rho, dtype=torch.float32, device=DEV)
    ox, oy = E.propagate(C, rho, geom, D=D)
    L = (ox.double() * torch.as_tensor(wx, device=DEV)).sum() + \
        (oy.double() * torch.as_tensor(wy, device=DEV)).sum()
    L.backward()
    g = D.grad if D is not None else C.grad
    return ox.detach().cpu().numpy(), oy.detach().cpu().numpy(), g.detach().cpu().numpy()


def run_oracle(case: O.Case, wx, wy):
    ox, oy, st = O.forward(case, "f64", keep_states=True)
    gC, gD = O.adjoint(case, st, wx, wy, "f64")
    return ox, oy, (gD if case.mode == O.MODE_DFIELD else gC)


def weights(case, seed=11):
    rng = np.random.default_rng(seed)
    shape = case.out_shape()
    return rng.standard_normal(shape), rng.standard_normal(shape)


CASES = {
    "scalar_fields": dict(),
    "scalar_receivers_multishot": dict(record=O.RECORD_RECEIVERS, S=3, nrec=9),
    "dfield_fields": dict(mode=O.MODE_DFIELD, nx=41, ny=37),
    "fields_receivers": dict(mode=O.MODE_FIELDS, record=O.RECORD_RECEIVERS, S=2),
    "odd_small": dict(nx=7, ny=5, nt=40, stride=1, box=3),
    "x_force_stride_gt_nt": dict(src_comp=0, stride=200, nt=60),
    "duplicate_receivers": dict(record=O.RECORD_RECEIVERS, nrec=5, dup_receiver=True),
    "wide_multi_tile": dict(nx=70, ny=97, nt=80, S=2, stride=4),
    # >= 512 tiles of 32 x 32: the 32-row tiles of the plain kernels (smaller
    # problems take 8-row tiles)
    "large_32row_tiles": dict(nx=512, ny=512, nt=18, S=2, stride=3, record=O.RECORD_RECEIVERS, nrec=20),
    "large_32row_fields": dict(mode=O.MODE_FIELDS, nx=512, ny=520, nt=12, S=2, stride=2),
    "large_32row_dfield": dict(mode=O.MODE_DFIELD, nx=520, ny=512, nt=12, S=2, record=O.RECORD_RECEIVERS),
}


@pytest.mark.parametrize("name", list(CASES))
def test_forward_and_gradient_vs_fp64_oracle(name):
    case = random_case(**CASES[name])
    wx, wy = weights(case)
    gx, gy, gg = run_gpu(case, wx, wy, path=E.PATH_STEP)
    rx, ry, rg = run_oracle(case, wx, wy)
    assert rel(gx, rx) <= FWD_TOL and rel(gy, ry) <= FWD_TOL, (rel(gx, rx), rel(gy, ry))
    assert rel(gg, rg) <= GRAD_TOL, rel(gg, rg)


# scalar-constant cases with ny % 4 == 0, served by the cluster-resident path
RESIDENT_CASES = {
    "dense_odd_nx": dict(nx=33, ny=28),
    "receivers_multishot": dict(nx=45, ny=36, record=O.RECORD_RECEIVERS, S=3, nrec=9),
    "x_force_stride1": dict(nx=24, ny=20, nt=70, stride=1, src_comp=0),
    "duplicate_receivers": dict(nx=40, ny=32, record=O.RECORD_RECEIVERS, nrec=6, dup_receiver=True),
    "tall_thin": dict(nx=150, ny=8, nt=90, stride=5),
    "one_row_per_cta": dict(nx=17, ny=12, nt=50),
    "wide": dict(nx=64, ny=256, nt=60, S=2, record=O.RECORD_RECEIVERS, nrec=20),
}


@pytest.mark.parametrize("name", list(RESIDENT_CASES))
def test_resident_path_vs_fp64_oracle(name):
    case = random_case(**RESIDENT_CASES[name])
    wx, wy = weights(case)
    gx, gy, gg = run_gpu(case, wx, wy, path=E.PATH_RESIDENT)
    rx, ry, rg = run_oracle(case, wx, wy)
    assert rel(gx, rx) <= FWD_TOL and rel(gy, ry) <= FWD_TOL, (rel(gx, rx), rel(gy, ry))
    assert rel(gg, rg) <= GRAD_TOL, rel(gg, rg)


# cases with ny % 4 == 0 on the tiled (TMA) per-step kernels: tiles of 64
# columns x 16 rows (32 rows in the degradation-map adjoint), ragged edges in
# both directions, tile boundaries through the source box and through
# receiver cells
TILED_CASES = {
    "dense_ragged": dict(nx=45, ny=76),
    "receivers_multishot": dict(nx=70, ny=132, record=O.RECORD_RECEIVERS, S=3, nrec=40),
    "x_force_stride1": dict(nx=33, ny=68, nt=70, stride=1, src_comp=0),
    "duplicate_receivers": dict(nx=40, ny=64, record=O.RECORD_RECEIVERS, nrec=6, dup_receiver=True),
    "narrow": dict(nx=150, ny=8, nt=90, stride=5),
    "single_tile": dict(nx=32, ny=64, nt=60),
    "tiny": dict(nx=3, ny=4, nt=30, box=2),
    "many_tiles": dict(nx=130, ny=260, nt=50, S=2, record=O.RECORD_RECEIVERS, nrec=30),
    "dfield_dense": dict(mode=O.MODE_DFIELD, nx=45, ny=76),
    "dfield_receivers_multishot": dict(mode=O.MODE_DFIELD, nx=70, ny=132, record=O.RECORD_RECEIVERS,
                                       S=3, nrec=40),
    "dfield_duplicate_receivers": dict(mode=O.MODE_DFIELD, nx=40, ny=64, record=O.RECORD_RECEIVERS,
                                       nrec=6, dup_receiver=True),
    "dfield_x_force_tiny": dict(mode=O.MODE_DFIELD, nx=3, ny=4, nt=30, box=2, src_comp=0),
}


@pytest.mark.parametrize("name", list(TILED_CASES))
def test_tiled_path_vs_fp64_oracle(name):
    case = random_case(**TILED_CASES[name])
    wx, wy = weights(case)
    gx, gy, gg = run_gpu(case, wx, wy, path=E.PATH_TILED)
    rx, ry, rg = run_oracle(case, wx, wy)
    assert rel(gx, rx) <= FWD_TOL and rel(gy, ry) <= FWD_TOL, (rel(gx, rx), rel(gy, ry))
    assert rel(gg, rg) <= GRAD_TOL, rel(gg, rg)


def test_tiled_forward_matches_step_forward():
    # same terms in the same order; the compilers' fused multiply-adds differ
    # between the two kernels, so the states agree to FP32 rounding
    case = random_case(nx=70, ny=132, nt=80, S=2, stride=3)
    wx, wy = weights(case)
    a = run_gpu(case, wx, wy, path=E.PATH_STEP)
    b = run_gpu(case, wx, wy, path=E.PATH_TILED)
    assert rel(a[0], b[0]) <= 1e-5 and rel(a[1], b[1]) <= 1e-5, (rel(a[0], b[0]), rel(a[1], b[1]))


@pytest.mark.parametrize("k", [1, 7, 1000])
def test_tiled_dfield_checkpoint_interval(k):
    case = random_case(mode=O.MODE_DFIELD, nx=40, ny=68, nt=90, S=2, record=O.RECORD_RECEIVERS)
    wx, wy = weights(case)
    ref = run_gpu(case, wx, wy, ckpt_k=None, path=E.PATH_TILED)
    got = run_gpu(case, wx, wy, ckpt_k=k, path=E.PATH_TILED)
    for x, y in zip(ref, got):
        assert np.array_equal(x, y)


def test_tiled_path_rejects_unsupported_problem():
    for kw in (dict(nx=20, ny=18), dict(nx=20, ny=20, mode=O.MODE_FIELDS)):  # ny % 4, six planes
        case = random_case(nt=10, **kw)
        wx, wy = weights(case)
        with pytest.raises(E._lib.ErnnError):
            run_gpu(case, wx, wy, path=E.PATH_TILED)


@pytest.mark.parametrize("path", [E.PATH_STEP, E.PATH_RESIDENT, E.PATH_TILED])
@pytest.mark.parametrize("k", [1, 2, 7, 50, 119, 120, 1000])
def test_checkpoint_interval_does_not_change_results(k, path):
    case = random_case(nt=120, S=2, ny=32, record=O.RECORD_RECEIVERS)
    wx, wy = weights(case)
    ref = run_gpu(case, wx, wy, ckpt_k=None, path=path)
    got = run_gpu(case, wx, wy, ckpt_k=k, path=path)
    # recomputation replays the identical kernels: bit-identical forward outputs
    assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
    if path != E.PATH_RESIDENT:
        assert np.array_equal(ref[2], got[2])
    else:
        # the resident path flushes its FP32 partial sums to FP64 at segment
        # boundaries, so the grouping (not the terms) depends on k
        assert rel(got[2], ref[2]) <= 1e-6


def test_backward_reads_the_tape_as_the_forward_wrote_it():
    """The geometry changed between forward and backward (a longer
    checkpoint interval, a different source signal) does not change how the
    adjoint reads the tape or what the recompute replays: the gradient is that
    of the unchanged run, bit for bit."""
    case = random_case(nt=120, S=2, ny=32, record=O.RECORD_RECEIVERS)
    wx, wy = weights(case)
    ref = run_gpu(case, wx, wy, ckpt_k=10, path=E.PATH_STEP)
    geom = to_geometry(case, 10, E.PATH_STEP)
    C = torch.tensor(case.C, dtype=torch.float32, device=DEV, requires_grad=True)
    rho = torch.tensor(case.rho, dtype=torch.float32, device=DEV)
    ox, oy = E.propagate(C, rho, geom)
    geom.ckpt_k = 40                                     # fewer checkpoints: a smaller tape would pass the size check
    geom.src_signal = torch.zeros_like(geom.src_signal)  # a recompute with this signal would differ
    L = (ox.double() * torch.as_tensor(wx, device=DEV)).sum() + \
        (oy.double() * torch.as_tensor(wy, device=DEV)).sum()
    L.backward()
    assert np.array_equal(C.grad.cpu().numpy(), ref[2])


def test_resident_tiled_and_step_paths_agree():
    case = random_case(nx=64, ny=64, nt=150, S=2, record=O.RECORD_RECEIVERS, nrec=16)
    wx, wy = weights(case)
    a = run_gpu(case, wx, wy, ckpt_k=30, path=E.PATH_STEP)
    r = run_oracle(case, wx, wy)
    for path in (E.PATH_RESIDENT, E.PATH_TILED):
        b = run_gpu(case, wx, wy, ckpt_k=30, path=path)
        for x, y, z in zip(a, b, r):
            # each path against the FP64 run (the plain per-step kernels 2.9e-5
            # on this case, the resident and tiled ones below 1e-5); the FP32
            # paths sum the imaging products in different orders, so they
            # agree to that rounding
            assert rel(x, z) <= 4e-5 and rel(y, z) <= 4e-5, (rel(x, z), rel(y, z))
            assert rel(x, y) <= 4e-5


def test_resident_path_rejects_unsupported_problem():
    case = random_case(nx=20, ny=18, nt=10, mode=O.MODE_DFIELD)  # per-cell mode, ny % 4 != 0
    wx, wy = weights(case)
    with pytest.raises(E._lib.ErnnError):
        run_gpu(case, wx, wy, path=E.PATH_RESIDENT)


@pytest.mark.parametrize("mode", [O.MODE_FIELDS, O.MODE_DFIELD])
def test_checkpointed_percell_modes(mode):
    case = random_case(mode=mode, nt=90, record=O.RECORD_RECEIVERS, S=2)
    wx, wy = weights(case)
    got = run_gpu(case, wx, wy, ckpt_k=13)
    ref = run_oracle(case, wx, wy)
    assert rel(got[2], ref[2]) <= GRAD_TOL


def test_operator_vs_reference_golden():
    for tag in ("f32", "f64"):
        g = np.load(os.path.join(GOLDEN, f"operator_{tag}.npz"))
        t = lambda a: torch.tensor(a, dtype=torch.float32, device=DEV)
        C = [t(v) for v in g["C"]]
        Lx, Ly = E.elastic_operator_with_force(t(g["ux"])[None], t(g["uy"])[None], *C, float(g["h"]),
                                               t(g["fx"])[None], t(g["fy"])[None], float(g["rho"]))
        assert rel(Lx.cpu().numpy()[0], g["Lux"]) < 1e-5
        assert rel(Ly.cpu().numpy()[0], g["Luy"]) < 1e-5
        n = int(g["nsq"])
        Cf = [t(g["C_fields"][i])[None] for i in range(6)]
        # the spatially varying reference adds the transposed force
        Lx, Ly = E.elastic_operator_with_force(t(g["vx"])[None], t(g["vy"])[None], *Cf, float(g["h"]),
                                               t(g["gx"].T)[None], t(g["gy"].T)[None], float(g["rho"]))
        assert rel(Lx.cpu().numpy()[0], g["Lux_fields"]) < 1e-5
        assert rel(Ly.cpu().numpy()[0], g["Luy_fields"]) < 1e-5


def _reference_loss(pred_ux, pred_uy, tx, ty, ts, ss, wx=1.0):
    """compute_loss of Parameter_inversion/Inversion_adam.py:358-391 (wx=5, ss=1:
    Damage_inversion/Inversion_adam.py:441-450)."""
    px = pred_ux[:, ::ts, ::ss, ::ss]
    py = pred_uy[:, ::ts, ::ss, ::ss]
    return wx * torch.mean((px - tx[:, ::ts, ::ss, ::ss]) ** 2) + torch.mean((py - ty[:, ::ts, ::ss, ::ss]) ** 2)


@pytest.mark.parametrize("ckpt_k", [None, 16])
def test_dropin_param_simulator_vs_reference_golden(ckpt_k):
    g = np.load(os.path.join(GOLDEN, "param_inversion_f64.npz"))
    init = dict(C11_init=150e9, C22_init=75e9, C12_init=45e9, C16_init=11e9, C26_init=15e9,
                C66_init=39e9)
    sim = E.CFRPWaveSimulatorRicker((int(g["nx"]), int(g["ny"])), float(g["h"]), float(g["dt"]),
                                    int(g["nt"]), int(g["stride"]), source_component="y",
                                    source_f0=4e6, source_t0=2.5e-7, source_amplitude=1e10,
                                    rho_known=float(g["rho"]), gaussian_param=5e6, ckpt_k=ckpt_k,
                                    **init).to(DEV)
    ux, uy = sim(save_all_steps=False)
    assert ux.shape == g["hist_ux"].shape
    assert rel(ux.detach().cpu().numpy(), g["hist_ux"]) <= FWD_TOL
    assert rel(uy.detach().cpu().numpy(), g["hist_uy"]) <= FWD_TOL
    tx = torch.tensor(g["target_ux"], dtype=torch.float32, device=DEV)
    ty = torch.tensor(g["target_uy"], dtype=torch.float32, device=DEV)
    loss = _reference_loss(ux, uy, tx, ty, int(g["ts"]), int(g["ss"]))
    assert abs(loss.item() - float(g["loss"])) <= 1e-4 * abs(float(g["loss"]))
    loss.backward()
    got = np.array([float(getattr(sim, n).grad) for n in
                    ("log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66")])
    assert rel(got, g["grad_log"]) <= GRAD_TOL, (got, g["grad_log"])


def test_dropin_save_all_steps_matches_every_frame():
    sim = E.CFRPWaveSimulatorRicker((24, 20), 1e-4, 5e-9, 60, 5, source_f0=4e6, source_t0=2.5e-7,
                                    source_amplitude=1e10).to(DEV)
    with torch.no_grad():
        a, _ = sim(save_all_steps=False)
        b, _ = sim(save_all_steps=True)
    assert b.shape[1] == 60 and a.shape[1] == 12
    assert torch.equal(a, b[:, ::5])


def test_dropin_damage_simulator_vs_reference_golden():
    g = np.load(os.path.join(GOLDEN, "damage_inversion_f64.npz"))
    n = int(g["nx"])
    sim = E.SpatiallyVaryingAnisotropicSimulator((n, n), float(g["h"]), float(g["dt"]), int(g["nt"]),
                                                 int(g["stride"]), source_f0=4e6, source_t0=2.5e-7,
                                                 source_amplitude=1e10, total_time=int(g["nt"]) * float(g["dt"]),
                                                 rho_known=float(g["rho"]), gaussian_param=5e6).to(DEV)
    with torch.no_grad():
        for t, name in enumerate(("log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66")):
            getattr(sim, name).copy_(torch.log(torch.tensor(g["C_fields"][t], dtype=torch.float64))[None].float())
    ux, uy = sim(save_all_steps=False)
    assert rel(ux.detach().cpu().numpy(), g["hist_ux"]) <= FWD_TOL
    assert rel(uy.detach().cpu().numpy(), g["hist_uy"]) <= FWD_TOL
    tx = torch.tensor(g["target_ux"], dtype=torch.float32, device=DEV)
    ty = torch.tensor(g["target_uy"], dtype=torch.float32, device=DEV)
    loss = _reference_loss(ux, uy, tx, ty, int(g["ts"]), 1, wx=5.0)
    loss.backward()
    got = np.stack([getattr(sim, n).grad[0].cpu().numpy() for n in
                    ("log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66")])
    assert rel(got, g["grad_log"]) <= GRAD_TOL


def test_dropin_damage_loss_with_tv_vs_reference_golden():
    # the reference run's objective: 5:1 weighted misfit on every ts-th frame
    # plus lambda_tv = 1e-21 times the total variation of the six fields
    g = np.load(os.path.join(GOLDEN, "damage_inversion_tv_f64.npz"))
    n = int(g["nx"])
    sim = E.SpatiallyVaryingAnisotropicSimulator((n, n), float(g["h"]), float(g["dt"]), int(g["nt"]),
                                                 int(g["stride"]), source_f0=4e6, source_t0=2.5e-7,
                                                 source_amplitude=1e10, total_time=int(g["nt"]) * float(g["dt"]),
                                                 rho_known=float(g["rho"]), gaussian_param=5e6).to(DEV)
    names = ("log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66")
    with torch.no_grad():
        for t, name in enumerate(names):
            getattr(sim, name).copy_(torch.log(torch.tensor(g["C_fields"][t], dtype=torch.float64))[None].float())
    ux, uy = sim(save_all_steps=False)
    tx = torch.tensor(g["target_ux"], dtype=torch.float32, device=DEV)
    ty = torch.tensor(g["target_uy"], dtype=torch.float32, device=DEV)
    total, data, tv = E.damage_loss(sim, ux, uy, tx, ty, int(g["ts"]), float(g["lambda_tv"]))
    assert abs(float(data) - float(g["loss_data"])) <= 1e-4 * float(g["loss_data"])
    assert abs(float(tv) - float(g["loss_tv"])) <= 1e-5 * float(g["loss_tv"])
    total.backward()
    got = np.stack([getattr(sim, nm).grad[0].cpu().numpy() for nm in names])
    assert rel(got, g["grad_log"]) <= GRAD_TOL, rel(got, g["grad_log"])


def test_damage_simulator_rejects_non_square_like_reference():
    sim = E.SpatiallyVaryingAnisotropicSimulator((12, 10), 1e-4, 5e-9, 10, 5).to(DEV)
    with pytest.raises(RuntimeError):
        sim()


def test_gradient_vs_central_differences_fp32():
    """Config-2-style check: central differences with h = 1e-3 relative on each
    constant, FP32 forward on the GPU; agreement is limited by FP32 noise of
    the loss difference and the O(h^2) truncation (see the FP64 oracle test
    for the tight bound)."""
    case = random_case(nx=48, ny=40, nt=150, record=O.RECORD_RECEIVERS, nrec=12)
    geom = to_geometry(case, ckpt_k=25)
    rho = torch.tensor(case.rho, device=DEV)
    obs = [o + 0.05 * o.std() * torch.randn_like(o) for o in
           E.propagate(torch.tensor(case.C * 1.02, dtype=torch.float32, device=DEV), rho, geom)]

    def loss(Cv):
        ox, oy = E.propagate(Cv, rho, geom)
        return ((ox.double() - obs[0].double()) ** 2).mean() + ((oy.double() - obs[1].double()) ** 2).mean()

    C = torch.tensor(case.C, dtype=torch.float32, device=DEV, requires_grad=True)
    loss(C).backward()
    g = C.grad.double().cpu().numpy()
    scale = np.abs(g).max()
    with torch.no_grad():
        for t in range(6):
            e = torch.zeros(6, dtype=torch.float64)
            e[t] = case.C[t] * 1e-3
            Cp = (torch.tensor(case.C) + e).float().to(DEV)
            Cm = (torch.tensor(case.C) - e).float().to(DEV)
            de = float((Cp - Cm)[t]) / 2.0
            fd = (loss(Cp).item() - loss(Cm).item()) / (2 * de)
            assert abs(fd - g[t]) <= 2e-3 * scale, (t, fd, g[t])


def test_cpu_tensors_raise_instead_of_falling_back():
    case = random_case(nx=8, ny=8, nt=5)
    geom = to_geometry(case)
    with pytest.raises(RuntimeError):
        E.propagate(torch.tensor(case.C, dtype=torch.float32), torch.tensor(1560.0), geom)


def test_launch_counter_counts_kernels():
    lib = E.load_library()
    case = random_case(nx=16, ny=16, nt=10)
    wx, wy = weights(case)
    n0 = lib.ernn_launch_count()
    run_gpu(case, wx, wy, path=E.PATH_STEP)        # one launch per step and pass
    assert lib.ernn_launch_count() - n0 >= 20
    n0 = lib.ernn_launch_count()
    run_gpu(case, wx, wy, path=E.PATH_RESIDENT)    # one launch per pass
    assert 3 <= lib.ernn_launch_count() - n0 < 20


def test_bounded_wait_gives_up_and_context_survives():
    # a device-side wait that nothing completes returns ERNN_ERR_TIMEOUT after
    # about a second instead of hanging; the context stays usable afterwards
    lib = E._lib.load()
    status = ctypes.c_int32(-1)
    rc = lib.ernn_wait_selftest(ctypes.byref(status), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0 and status.value == 5, (rc, status.value)
    case = random_case(nx=40, ny=64, nt=40)
    wx, wy = weights(case)
    gx, gy, gg = run_gpu(case, wx, wy, path=E.PATH_TILED)
    rx, ry, rg = run_oracle(case, wx, wy)
    assert rel(gx, rx) <= FWD_TOL and rel(gg, rg) <= GRAD_TOL
    E.check_device_status()  # the status words of those calls are clear


@pytest.mark.parametrize("path", [E.PATH_STEP, E.PATH_RESIDENT, E.PATH_TILED])
def test_device_status_word_is_clear_after_calls(path):
    case = random_case(nx=32, ny=32, nt=30, record=O.RECORD_RECEIVERS)
    wx, wy = weights(case)
    run_gpu(case, wx, wy, path=path)
    status = sys.modules[E.ErnnPropagate.__module__]._STATUS
    E.check_device_status()
    assert status.pending == []
    assert E._lib.load().ernn_last_path() == path


@pytest.mark.parametrize("path", [E.PATH_STEP, E.PATH_RESIDENT, E.PATH_TILED])
def test_receiver_traces_equal_gathered_dense_history(path):
    # same seed: identical sources; the receiver mode records frame k = u^{k*stride+1}
    # at the receiver cells, exactly the dense history gathered there
    dense = random_case(nx=40, ny=64, nt=61, stride=3, S=2)
    recs = random_case(nx=40, ny=64, nt=61, stride=3, S=2, record=O.RECORD_RECEIVERS, nrec=12)
    rho = torch.tensor(dense.rho, dtype=torch.float32, device=DEV)
    C = torch.tensor(dense.C, dtype=torch.float32, device=DEV)
    with torch.no_grad():
        hx, hy = E.propagate(C, rho, to_geometry(dense, path=path))
        tx, ty = E.propagate(C, rho, to_geometry(recs, path=path))
    rec_idx = torch.as_tensor(recs.rec_idx, dtype=torch.int32, device=DEV)
    gx, gy = E.formats.traces_from_history(hx, hy, rec_idx)
    assert torch.equal(gx, tx) and torch.equal(gy, ty)


def test_dropin_adam_trajectory_matches_reference_invert():
    # the reference's own loop (CFRPParameterInverterRicker.invert, float32):
    # zero_grad, forward, compute_loss, backward, Adam step, record — six
    # epochs through the drop-in simulator give its losses and constants
    g = np.load(os.path.join(GOLDEN, "param_invert_f32.npz"))
    init = dict(C11_init=150e9, C22_init=75e9, C12_init=45e9, C16_init=11e9, C26_init=15e9,
                C66_init=39e9)
    sim = E.CFRPWaveSimulatorRicker((int(g["nx"]), int(g["ny"])), float(g["h"]), float(g["dt"]),
                                    int(g["nt"]), int(g["stride"]), source_component="y",
                                    source_f0=4e6, source_t0=2.5e-7, source_amplitude=1e10,
                                    rho_known=float(g["rho"]), gaussian_param=5e6, **init).to(DEV)
    tx = torch.tensor(g["target_ux"], dtype=torch.float32, device=DEV)
    ty = torch.tensor(g["target_uy"], dtype=torch.float32, device=DEV)
    opt = torch.optim.Adam(sim.parameters(), lr=float(g["lr"]), betas=(0.9, 0.999), eps=1e-8)
    losses, params = [], []
    for _ in range(int(g["epochs"])):
        opt.zero_grad()
        ux, uy = sim(save_all_steps=False)
        loss = _reference_loss(ux, uy, tx, ty, int(g["ts"]), int(g["ss"]))
        loss.backward()
        opt.step()
        losses.append(loss.item())
        params.append(sim.get_current_params_values()[:6])
    assert rel(np.array(losses), g["loss"]) <= 1e-4, (losses, g["loss"])
    assert rel(np.array(params), g["params"]) <= 1e-6, (params, g["params"])


@pytest.mark.parametrize("fused_objective", [True, False])
def test_damage_loop_trajectory_vs_reference_invert(fused_objective):
    # the reference's own damage loop (SpatiallyVaryingParameterInverter.invert,
    # float32, lr 0.02, TV 1e-21): twelve epochs through the drop-in six-field
    # simulator give its losses and mean constants, with the library's fused
    # objective (damage_loss) or the reference's torch expression
    g = np.load(os.path.join(GOLDEN, "damage_invert_f32.npz"))
    base = dict(C11_init=130.74e9, C22_init=11.50e9, C12_init=10.49e9, C16_init=30.67e9,
                C26_init=3.75e9, C66_init=14.77e9)
    nt = int(g["nt"])
    sim = E.SpatiallyVaryingAnisotropicSimulator(
        (int(g["nx"]), int(g["ny"])), float(g["h"]), float(g["dt"]), nt, int(g["stride"]),
        source_component="y", total_time=nt * float(g["dt"]), rho_known=float(g["rho"]),
        use_log_params=True, source_f0=4e6, source_t0=2.5e-7, source_amplitude=1e10,
        gaussian_param=5e6, **base).to(DEV)
    tx = torch.tensor(g["target_ux"], dtype=torch.float32, device=DEV)
    ty = torch.tensor(g["target_uy"], dtype=torch.float32, device=DEV)
    ts, lam = int(g["ts"]), float(g["lambda_tv"])
    opt = torch.optim.Adam(sim.parameters(), lr=float(g["lr"]), betas=(0.9, 0.999), eps=1e-8)
    losses, means = [], []
    for _ in range(int(g["epochs"])):
        opt.zero_grad()
        ux, uy = sim(save_all_steps=False)
        if fused_objective:
            total, _, _ = E.damage_loss(sim, ux, uy, tx, ty, ts, lam)
        else:
            C = sim.get_material_params()[:6]
            total = _reference_loss(ux, uy, tx, ty, ts, 1, wx=5.0) + \
                lam * sum(E.total_variation_2d(c) for c in C)
        total.backward()
        opt.step()
        losses.append(total.item())
        means.append(sim.get_mean_params()[:6])
    assert rel(np.array(losses), g["loss"]) <= 1e-4, (losses, g["loss"])
    assert rel(np.array(means), g["means"]) <= 1e-6, (means, g["means"])
