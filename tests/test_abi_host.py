"""The C-ABI library loads, exports every entry point of include/ernn.h, and its
host-only calls behave (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

import ernn_gb300 as E
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ernn.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ernn_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = E.load_library()
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding declares a signature for each of them
    assert set(names) <= set(E._lib.SIGNATURES)


def test_c_program_uses_the_abi_without_python(tmp_path):
    """tests/abi_c/ernn_abi_host.c, compiled as strict C99 against
    include/ernn.h and linked to the library, runs the host-side entry points
    (validation, size queries, stability check, error strings) from C."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc absent")
    E.load_library()  # builds the library when it is missing
    libdir = os.path.dirname(E._lib.library_path())
    exe = str(tmp_path / "ernn_abi_host")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "abi_c", "ernn_abi_host.c"),
                    "-L", libdir, "-lernn_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


def test_struct_layout_matches_header():
    # ErnnProblem: 14 int32 then 2 doubles = 72 bytes; ErnnInputs: 7 pointers
    assert ctypes.sizeof(E._lib.ErnnProblem) == 72
    assert ctypes.sizeof(E._lib.ErnnInputs) == 7 * ctypes.sizeof(ctypes.c_void_p)


def test_version_and_error_strings():
    lib = E.load_library()
    assert lib.ernn_abi_version() == 1
    for code in range(0, 7):
        assert lib.ernn_error_string(code)
    assert b"unknown" in lib.ernn_error_string(99)


def _problem(**kw):
    base = dict(nshots=2, nx=64, ny=48, nt=100, stride=5, mode=0, record=1, nrec=8, src_comp=1,
                src_bx=9, src_by=9, ckpt_k=10, path=0, flags=0, h=1e-4, dt=5e-9)
    base.update(kw)
    return E._lib.ErnnProblem(*[base[f] for f, _ in E._lib.ErnnProblem._fields_])


def test_validation_rejects_bad_problems():
    lib = E.load_library()
    assert lib.ernn_validate(ctypes.byref(_problem())) == 0
    bad = [dict(nx=0), dict(nt=0), dict(stride=0), dict(mode=3), dict(record=2),
           dict(nrec=0), dict(src_comp=2), dict(h=0.0), dict(dt=-1.0), dict(ckpt_k=0),
           dict(nshots=0), dict(nx=70000, ny=70000), dict(path=4), dict(path=-1), dict(flags=8),
           dict(flags=1, mode=1),
           # instances on a canvas: scalar constants, receiver traces, canvas < 65536
           dict(flags=2, mode=1), dict(flags=2, record=0), dict(flags=2, nshots=257),
           dict(flags=2, nx=70000, ny=16)]
    for kw in bad:
        assert lib.ernn_validate(ctypes.byref(_problem(**kw))) == 1, kw
    assert lib.ernn_validate(None) == 1


def test_sizes_that_would_wrap_are_refused():
    """A problem whose tape or scratch size would not fit in 64 bits, or whose
    plain step launch would have more blocks than an int counts, is invalid
    and its size queries return 0 (never a wrapped, too small size)."""
    lib = E.load_library()
    huge_tape = dict(nshots=65535, nx=46340, ny=46340, nt=2 ** 30, ckpt_k=2 ** 30)
    many_blocks = dict(nshots=65535, nx=46340, ny=46340, nt=1, ckpt_k=1)
    for kw in (huge_tape, many_blocks):
        p = _problem(**kw)
        assert lib.ernn_validate(ctypes.byref(p)) == 1, kw
        assert lib.ernn_tape_bytes(ctypes.byref(p), 1) == 0
        assert lib.ernn_adjoint_scratch_bytes(ctypes.byref(p)) == 0
    # a large problem within the bounds still gets its exact size
    ok = _problem(nshots=16, nx=1024, ny=1024, nt=4000, ckpt_k=4000)
    assert lib.ernn_validate(ctypes.byref(ok)) == 0
    assert lib.ernn_tape_bytes(ctypes.byref(ok), 1) >= 4000 * 16 * 2 * 1024 * 1024 * 4


def test_instance_regions_are_checked_before_any_device_work():
    """Regions past the canvas (also where x0 + nx overflows 32 bits),
    overlapping or touching regions, and step counts above nt are refused
    on the host.  The inputs are placeholders that are never dereferenced and
    the tape is given as 0 bytes, so valid regions stop at the workspace
    check (ERNN_ERR_WORKSPACE) and bad ones at the region check
    (ERNN_ERR_INVALID), both before any CUDA call."""
    lib = E.load_library()
    p = _problem(flags=2, nshots=2, nx=256, ny=256, nt=100)
    dummy = ctypes.c_void_p(16)  # non-null placeholder, never dereferenced on these paths
    ins = E._lib.ErnnInputs(dummy, None, dummy, dummy, dummy, dummy, dummy)

    def call(x0, y0, nx, ny, nt):
        arr = lambda v: (ctypes.c_int32 * 2)(*v)
        inst = E._lib.ErnnInstances(2, arr(x0), arr(y0), arr(nx), arr(ny), arr(nt))
        return lib.ernn_forward_instances(ctypes.byref(p), ctypes.byref(ins), ctypes.byref(inst), dummy, dummy,
                                          dummy, 0, 1, None)
    assert call((0, 20), (0, 0), (10, 10), (16, 16), (100, 60)) == 2  # valid: only the tape is short
    bad = [((0, 2 ** 31 - 8), (0, 0), (10, 16), (16, 16), (100, 100)),   # x0 + nx wraps
           ((0, 0), (0, 2 ** 31 - 4), (10, 10), (16, 8), (100, 100)),    # y0 + ny wraps
           ((0, 250), (0, 0), (10, 10), (16, 16), (100, 100)),           # past the canvas
           ((0, 10), (0, 0), (10, 10), (16, 16), (100, 100)),            # no ghost row between
           ((0, 20), (0, 0), (10, 10), (16, 16), (100, 101))]            # more steps than nt
    for args in bad:
        assert call(*args) == 1, args


def test_instance_workspace_holds_one_canvas_plane():
    # with instances the state is one canvas plane, not one per shot, and the
    # tape and scratch hold the tile table (and the scratch a zero state)
    lib = E.load_library()
    plain = _problem(flags=1, ckpt_k=100)
    inst = _problem(flags=2, ckpt_k=100)
    assert lib.ernn_validate(ctypes.byref(inst)) == 0
    state1 = (2 * 64 * 48 * 4 + 255) // 256 * 256
    t_plain = lib.ernn_tape_bytes(ctypes.byref(plain), 0)
    t_inst = lib.ernn_tape_bytes(ctypes.byref(inst), 0)
    # two state levels of two shots vs of one plane, plus the table
    assert t_inst - 2 * state1 < t_plain - 2 * 2 * state1 + 256 * 1024
    assert lib.ernn_adjoint_scratch_bytes(ctypes.byref(inst)) > 0


def test_workspace_sizes_follow_checkpoint_plan():
    lib = E.load_library()
    state = 2 * 2 * 64 * 48 * 4  # shots * comps * cells * float
    align = lambda v: (v + 255) // 256 * 256
    # segmented: 10 segments -> 9 checkpoints of two states
    p = _problem(ckpt_k=10)
    t = lib.ernn_tape_bytes(ctypes.byref(p), 1)
    assert t == 256 + 2 * align(state) + 9 * 2 * align(state)
    assert lib.ernn_tape_bytes(ctypes.byref(p), 0) == 256 + 2 * align(state)
    # store-all when k >= nt
    p = _problem(ckpt_k=100)
    assert lib.ernn_tape_bytes(ctypes.byref(p), 1) == 256 + 2 * align(state) + 100 * align(state)
    s_seg = lib.ernn_adjoint_scratch_bytes(ctypes.byref(_problem(ckpt_k=10)))
    s_all = lib.ernn_adjoint_scratch_bytes(ctypes.byref(_problem(ckpt_k=100)))
    # segmented: two recompute segments and two lam segments of k = 10 states;
    # store-all: no recompute segments, two lam segments of min(nt, 128) = 100
    assert s_seg - s_all == (2 * 10 + 2 * 10 - 2 * 100) * align(state)
    assert lib.ernn_tape_bytes(ctypes.byref(_problem(nx=0)), 1) == 0


def test_stability_check():
    c = E.materials.orthotropic_xz(130e9, 12e9, 6e9, 5.5e9)
    v = E.materials.check_stability(c, 1560.0, 1e-4, 5e-9)
    assert 0.1 < v < 1.0
    # the stability number scales with dt^2
    v2 = E.materials.check_stability(c, 1560.0, 1e-4, 10e-9)
    assert abs(v2 / v - 4.0) < 1e-9
    with pytest.raises(ValueError):
        E.materials.check_stability(c, 1560.0, 1e-4, 20e-9)
    # 1D limit: C11 only, q = v^2 dt^2 / h^2 -> number = q * 4 / 4
    one = np.array([1.0, 0, 0, 0, 0, 0])
    assert abs(E.materials.check_stability(one, 1.0, 1.0, 0.5) - 0.25) < 1e-12


def test_numpy_stability_number_equals_the_library_check():
    # the benchmark's reference arm draws its initial guesses with the numpy
    # restatement (it must not load the library): both must accept and reject
    # the same materials
    rng = np.random.default_rng(5)
    base = E.materials.rotate(E.materials.orthotropic_xz(130e9, 12e9, 6e9, 5.5e9), 30.0)
    for k in range(40):
        c = base * rng.uniform(0.5, 1.5, size=6)
        dt = rng.choice([5e-9, 9e-9, 14e-9])
        number, indefinite = E.configs.stability_number(c, 1560.0, 1e-4, dt)
        try:
            v = E.materials.check_stability(c, 1560.0, 1e-4, dt)
            assert not indefinite and number <= 1.0
            assert abs(v - number) <= 1e-12 * v
        except ValueError:
            assert indefinite or number > 1.0


def test_reference_arm_loads_no_library():
    # bench.py's reference arm builds its workload from the numpy-only
    # configurations, loaded by file path in a fresh process
    import subprocess
    import sys
    code = ("import bench; w = bench.standalone('configs').rot256(); "
            "g = bench.standalone('configs').initial_guess(w); bench.standalone('sources'); "
            "print(bench.library_mapped(), len(g))")
    out = subprocess.run([sys.executable, "-c", code], cwd=os.path.dirname(os.path.dirname(__file__)),
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["False", "6"]


def test_rotation_properties():
    c = E.materials.orthotropic_xz(130e9, 12e9, 6e9, 5.5e9)
    assert np.allclose(E.materials.rotate(c, 0), c)
    r90 = E.materials.rotate(c, 90)
    assert np.allclose(r90[[0, 1, 2, 5]], c[[1, 0, 2, 5]], rtol=1e-12, atol=1e-3)
    r30 = E.materials.rotate(c, 30)
    assert np.all(np.abs(r30) > 1e9)          # all six non-zero
    # rotation invariants of the 2D stiffness: C_iijj = C11 + C22 + 2 C12, C_ijij = C11 + C22 + 2 C66
    inv1 = lambda v: v[0] + v[1] + 2 * v[2]
    inv2 = lambda v: v[0] + v[1] + 2 * v[5]
    assert abs(inv1(r30) - inv1(c)) < 1e-3 * inv1(c)
    assert abs(inv2(r30) - inv2(c)) < 1e-3 * inv2(c)
    assert np.allclose(E.materials.rotate(E.materials.rotate(c, 30), -30), c, rtol=1e-12, atol=1e-2)


def test_sources():
    t = np.arange(2000) * 5e-9
    b = E.sources.tone_burst(t, 1e6, 5)
    assert b[0] == 0 and np.all(b[t > 5e-6] == 0) and np.abs(b).max() > 0.9
    r = E.sources.ricker_wavelet(t, 1e6, 1e-6, 2.0)
    assert abs(r[200] - 2.0) < 1e-12  # peak at t0
    dense = torch.zeros(2, 20, 16)
    dense[0, 3:6, 4:9] = 1.0
    dense[1, 10:12, 0:3] = 2.0
    m, o = E.sources.crop_box(dense)
    assert m.shape == (2, 3, 5)
    assert o.tolist() == [[3, 4], [10, 0]]
    assert float(m[1].sum()) == 12.0


def test_geometry_validation_on_host():
    geom = E.Geometry(nx=8, ny=8, nt=4, h=1e-4, dt=5e-9, src_signal=torch.zeros(1, 4),
                      src_map=torch.zeros(1, 2, 2), src_origin=torch.zeros(1, 2, dtype=torch.int32),
                      rec_idx=torch.tensor([[0, 64]], dtype=torch.int32))
    with pytest.raises(ValueError):
        geom.check(torch.device("cpu"))   # receiver 64 is outside the 8x8 grid
    geom = E.Geometry(nx=8, ny=8, nt=5, h=1e-4, dt=5e-9, src_signal=torch.zeros(1, 4),
                      src_map=torch.zeros(1, 2, 2), src_origin=torch.zeros(1, 2, dtype=torch.int32))
    with pytest.raises(ValueError):
        geom.check(torch.device("cpu"))   # signal length != nt


def test_product_path_refuses_cpu_tensors():
    geom = E.Geometry(nx=8, ny=8, nt=4, h=1e-4, dt=5e-9, src_signal=torch.zeros(1, 4),
                      src_map=torch.zeros(1, 2, 2), src_origin=torch.zeros(1, 2, dtype=torch.int32))
    with pytest.raises(RuntimeError, match="CUDA"):
        E.propagate(torch.ones(6), torch.tensor(1.0), geom)


def test_device_status_validates_before_any_device_call():
    lib = E._lib.load()
    p = _problem()
    st = ctypes.c_int32(0)
    assert lib.ernn_device_status(None, ctypes.c_void_p(16), 0, ctypes.byref(st), None) == 1
    assert lib.ernn_device_status(ctypes.byref(p), None, 0, ctypes.byref(st), None) == 1
    assert lib.ernn_device_status(ctypes.byref(p), ctypes.c_void_p(16), 2, ctypes.byref(st), None) == 1
    assert lib.ernn_device_status(ctypes.byref(p), ctypes.c_void_p(16), 0, None, None) == 1
    assert lib.ernn_wait_selftest(None, None) == 1
    assert lib.ernn_last_path() in (0, 1, 2, 3)


def test_launch_overlap_switch_is_a_host_setting():
    was = E._lib.launch_overlap(False)
    try:
        assert E._lib.launch_overlap(True) is False
        assert E._lib.launch_overlap(True) is True
    finally:
        E._lib.launch_overlap(was)


def test_fused_adam_refuses_cpu_parameters():
    from ernn_gb300.optim import FusedAdam
    p = torch.zeros(4, requires_grad=True)
    p.grad = torch.ones(4)
    with pytest.raises(RuntimeError, match="CUDA"):
        FusedAdam([p]).step()


def test_series_misfit_validates_on_the_host():
    from ernn_gb300.misfit import series_misfit
    a = torch.zeros((1, 4, 6))
    with pytest.raises(RuntimeError, match="CUDA"):
        series_misfit(a, a, a, a)
    with pytest.raises(ValueError):
        series_misfit(torch.zeros(3), torch.zeros(3), torch.zeros(3), torch.zeros(3))


def test_abi_refuses_series_and_fem_grids_beyond_its_bounds():
    """Host-side refusals made before any CUDA call: a misfit series whose
    element count would wrap 64 bits, a FEM grid whose per-level launch
    would exceed the 65535 blocks of grid y."""
    lib = E.load_library()
    dummy = ctypes.c_void_p(16)  # non-null placeholder, never dereferenced on these paths
    huge = E._lib.ErnnSeries(2 ** 40, 2 ** 30, 2 ** 20, 2 ** 20, 1, 1, 1.0, 1.0)
    assert lib.ernn_misfit(ctypes.byref(huge), dummy, dummy, dummy, dummy, dummy, dummy,
                           lib.ernn_misfit_workspace_bytes(), None) == 1
    assert lib.ernn_misfit_grad(ctypes.byref(huge), dummy, dummy, dummy, dummy, None, dummy, dummy, None) == 1
    ok = E._lib.ErnnSeries(2, 10, 1, 64, 1, 1, 1.0, 1.0)
    assert lib.ernn_misfit(ctypes.byref(ok), dummy, dummy, dummy, dummy, dummy, dummy, 0, None) == 2
    C6 = (ctypes.c_double * 6)(1e9, 1e9, 1e9, 0.0, 0.0, 1e9)
    tall = E._lib.ErnnFemProblem(524289, 3, 10, 1, 1e-3, 1e-3, 1e-8, 1.0, C6, 0.7)
    assert lib.ernn_fem_forward(ctypes.byref(tall), dummy, dummy, None, dummy, dummy, dummy, 2 ** 40, None) == 1
    fits = E._lib.ErnnFemProblem(524280, 3, 10, 1, 1e-3, 1e-3, 1e-8, 1.0, C6, 0.7)
    assert lib.ernn_fem_forward(ctypes.byref(fits), dummy, dummy, None, dummy, dummy, dummy, 0, None) == 2


def test_fused_adam_rejects_bad_hyper_parameters():
    from ernn_gb300.optim import FusedAdam
    p = torch.zeros(3, requires_grad=True)
    for kw in (dict(lr=-1.0), dict(betas=(1.0, 0.9)), dict(betas=(0.9, 1.0)), dict(eps=-1.0),
               dict(weight_decay=-0.1)):
        with pytest.raises(ValueError):
            FusedAdam([p], **kw)
