"""Size-independent properties of the oracle: finite differences, adjoint identity,
linearity, receiver/record consistency, D-mode equivalence.  All CPU."""
import numpy as np
import pytest

from oracle import oracle as O

C_ROT = np.array([120e9, 30e9, 25e9, 20e9, 8e9, 28e9])


def gauss(nx, ny, h, x0, y0, a=5e6):
    x = np.linspace(-h * (nx - 1) / 2, h * (nx - 1) / 2, nx)
    y = np.linspace(-h * (ny - 1) / 2, h * (ny - 1) / 2, ny)
    X, Y = np.meshgrid(x, y, indexing="ij")
    return a / np.pi * np.exp(-a * ((X - x0) ** 2 + (Y - y0) ** 2))


def make_case(nx=21, ny=17, nt=90, stride=4, mode=O.MODE_SCALAR, record=O.RECORD_FIELDS, S=1,
              seed=0):
    rng = np.random.default_rng(seed)
    h, dt, rho = 1e-4, 5e-9, 1560.0
    sig = rng.standard_normal((S, nt)) * 1e10
    smap = np.stack([gauss(nx, ny, h, (s - S / 2) * 3e-4, 0.0) for s in range(S)])
    org = np.zeros((S, 2), np.int32)
    rec = None
    if record == O.RECORD_RECEIVERS:
        rec = np.stack([np.arange(1, nx, 3) * ny + (ny - 1) for _ in range(S)]).astype(np.int32)
    C, D = C_ROT.copy(), None
    if mode == O.MODE_FIELDS:
        C = C_ROT[:, None, None] * (1 + 0.1 * rng.random((6, nx, ny)))
    if mode == O.MODE_DFIELD:
        D = 0.5 * rng.random((nx, ny))
    return O.Case(nx, ny, nt, h, dt, rho, C, sig, smap, org, stride=stride, mode=mode,
                  record=record, rec_idx=rec, D=D, ref_f32_sum=0)


def loss_and_grad(case, wx, wy):
    ux, uy, st = O.forward(case, "f64", keep_states=True)
    return float((ux * wx).sum() + (uy * wy).sum()), st


@pytest.mark.parametrize("record", [O.RECORD_FIELDS, O.RECORD_RECEIVERS])
def test_scalar_gradient_matches_central_differences(record):
    case = make_case(record=record, S=2)
    rng = np.random.default_rng(1)
    wx = rng.standard_normal(case.out_shape())
    wy = rng.standard_normal(case.out_shape())
    _, st = loss_and_grad(case, wx, wy)
    gC, _ = O.adjoint(case, st, wx, wy)
    def fd(t, rel_step):
        e = np.zeros(6)
        e[t] = case.C[t] * rel_step
        cp, cm = make_case(record=record, S=2), make_case(record=record, S=2)
        cp.C, cm.C = case.C + e, case.C - e
        return (loss_and_grad(cp, wx, wy)[0] - loss_and_grad(cm, wx, wy)[0]) / (2 * e[t])

    scale = np.abs(gC).max()
    for t in range(6):
        f1 = fd(t, 1e-3)                           # h = 1e-3 relative, as the config asks
        f2 = fd(t, 5e-4)
        # central differences carry an O(h^2) truncation error ...
        assert abs(f1 - gC[t]) <= 1e-3 * scale, (t, f1, gC[t])
        # ... which Richardson extrapolation removes, leaving the adjoint exact
        rich = (4 * f2 - f1) / 3
        assert abs(rich - gC[t]) <= 1e-6 * scale, (t, rich, gC[t])


def test_fields_and_dfield_gradients_by_directional_derivative():
    for mode in (O.MODE_FIELDS, O.MODE_DFIELD):
        case = make_case(mode=mode, nx=13, ny=12, nt=60)
        rng = np.random.default_rng(2)
        wx = rng.standard_normal(case.out_shape())
        wy = rng.standard_normal(case.out_shape())
        _, st = loss_and_grad(case, wx, wy)
        gC, gD = O.adjoint(case, st, wx, wy)
        if mode == O.MODE_FIELDS:
            v = rng.standard_normal(case.C.shape) * case.C * 1e-5
            pred = float((gC * v).sum())
            cp, cm = make_case(mode=mode, nx=13, ny=12, nt=60), make_case(mode=mode, nx=13, ny=12, nt=60)
            cp.C, cm.C = case.C + v, case.C - v
        else:
            v = rng.standard_normal(case.D.shape) * 1e-5
            pred = float((gD * v).sum())
            cp, cm = make_case(mode=mode, nx=13, ny=12, nt=60), make_case(mode=mode, nx=13, ny=12, nt=60)
            cp.D, cm.D = case.D + v, case.D - v
        fd = (loss_and_grad(cp, wx, wy)[0] - loss_and_grad(cm, wx, wy)[0]) / 2
        assert abs(fd - pred) <= 1e-6 * abs(pred), (mode, fd, pred)


def test_dfield_equals_fields_with_scaled_constants():
    case = make_case(mode=O.MODE_DFIELD, nx=15, ny=14, nt=50)
    a, b, _ = O.forward(case, "f64")
    fields = (1 - case.D)[None] * case.C[:, None, None]
    c2 = make_case(mode=O.MODE_FIELDS, nx=15, ny=14, nt=50)
    c2.C = fields
    a2, b2, _ = O.forward(c2, "f64")
    assert np.allclose(a, a2, rtol=1e-12, atol=1e-30) and np.allclose(b, b2, rtol=1e-12, atol=1e-30)


def test_linear_in_source_amplitude():
    case = make_case(S=1)
    a, b, _ = O.forward(case, "f64")
    case.src_signal = case.src_signal * 4.0
    a4, b4, _ = O.forward(case, "f64")
    assert np.allclose(a4, 4 * a, rtol=1e-12, atol=0)


def test_receivers_equal_gathered_fields():
    cf = make_case(S=2, record=O.RECORD_FIELDS)
    cr = make_case(S=2, record=O.RECORD_RECEIVERS)
    ux, uy, _ = O.forward(cf, "f64")
    rx, ry, _ = O.forward(cr, "f64")
    flat = ux.reshape(ux.shape[0], ux.shape[1], -1)
    for s in range(2):
        assert np.array_equal(rx[s], flat[s][:, cr.rec_idx[s]])


def test_history_frames_follow_reference_indexing():
    """Frame k holds u^{k*stride+1} (Inversion_adam.py:299-301); stride 1 is every step."""
    c1 = make_case(stride=1, nt=40)
    c4 = make_case(stride=4, nt=40)
    a1, _, _ = O.forward(c1, "f64")
    a4, _, _ = O.forward(c4, "f64")
    assert a4.shape[1] == 10
    assert np.array_equal(a4[0], a1[0, ::4])


def test_adjoint_dot_product_identity():
    """<dL/dC, v> from the adjoint equals the linearised forward response (tangent)."""
    case = make_case(S=1, nt=70)
    rng = np.random.default_rng(5)
    wx = rng.standard_normal(case.out_shape())
    wy = rng.standard_normal(case.out_shape())
    _, st = loss_and_grad(case, wx, wy)
    gC, _ = O.adjoint(case, st, wx, wy)
    v = rng.standard_normal(6) * case.C * 1e-6
    cp, cm = make_case(S=1, nt=70), make_case(S=1, nt=70)
    cp.C, cm.C = case.C + v, case.C - v
    fd = (loss_and_grad(cp, wx, wy)[0] - loss_and_grad(cm, wx, wy)[0]) / 2
    assert abs(fd - gC @ v) <= 1e-7 * abs(gC @ v)


def test_invalid_problem_rejected():
    case = make_case()
    case.h = -1.0
    with pytest.raises(ValueError):
        O.forward(case)


@pytest.mark.parametrize("mode,record,k", [(O.MODE_SCALAR, O.RECORD_RECEIVERS, 7),
                                           (O.MODE_SCALAR, O.RECORD_FIELDS, 90),
                                           (O.MODE_DFIELD, O.RECORD_RECEIVERS, 13),
                                           (O.MODE_FIELDS, O.RECORD_FIELDS, 1)])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_checkpointed_oracle_equals_the_store_all_oracle(mode, record, k, precision):
    # the checkpointed drivers replay the same steps in the same order: the
    # outputs and gradients are bitwise those of the store-all drivers
    case = make_case(mode=mode, record=record, S=2, nt=61)
    rng = np.random.default_rng(2)
    wx = rng.standard_normal(case.out_shape())
    wy = rng.standard_normal(case.out_shape())
    ax, ay, st = O.forward(case, precision, keep_states=True)
    gA, dA = O.adjoint(case, st, wx, wy, precision)
    bx, by, ck = O.forward_ckpt(case, k, precision)
    gB, dB = O.adjoint_ckpt(case, k, ck, wx, wy, precision)
    assert np.array_equal(ax, bx) and np.array_equal(ay, by)
    assert np.array_equal(gA, gB)
    if dA is not None:
        assert np.array_equal(dA, dB)
