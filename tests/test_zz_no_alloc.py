"""The allocation-free forward entry point, ernn_forward_static.

Some callers of this library cannot call cudaMalloc around a propagation:
code that runs while another framework is capturing a CUDA graph on the
stream (an allocation there would break the capture), real-time loops that
cannot afford the device synchronisation an allocation may bring, and FFI
hosts that carry no device allocator.  ernn_forward_static keeps its
wavefield scratch in an 8 MiB device array owned by the library.

Here it is called through the C ABI and compared with ernn_forward on the
per-step kernels: the same kernels in the same order on the same inputs, so
the outputs must be bitwise equal, on two calls in a row (the second call
reuses the array the first one left behind).  One case is also checked
directly against the FP64 oracle at the forward tolerance of the parity
tests.  This file is collected last so that a run stopping at the first
failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest
import torch

import ernn_gb300 as E
from ernn_gb300 import _lib
from cases import random_case, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
FWD_TOL = 1e-4   # forward tolerance of the parity tests (relative L2 against FP64)
LIMIT = 8 << 20  # bytes of the library's static array


def _tensors(case, per_shot_C=None):
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(DEV).contiguous()
    C = case.C if per_shot_C is None else per_shot_C
    rho = np.array([case.rho]) if per_shot_C is None else np.full(case.nshots, case.rho)
    keep = dict(C=t(C), rho=t(rho), sig=t(case.src_signal), smap=t(case.src_map),
                org=t(case.src_origin, torch.int32),
                rec=None if case.rec_idx is None else t(case.rec_idx, torch.int32),
                D=None if case.D is None else t(case.D))
    p = lambda x: None if x is None else ctypes.c_void_p(x.data_ptr())
    ins = _lib.ErnnInputs(p(keep["C"]), p(keep["D"]), p(keep["rho"]), p(keep["sig"]), p(keep["smap"]),
                          p(keep["org"]), p(keep["rec"]))
    return keep, ins


def _problem(case, flags=0, path=_lib.PATH_STEP):
    nrec = 0 if case.rec_idx is None else case.rec_idx.shape[1]
    return _lib.ErnnProblem(case.nshots, case.nx, case.ny, case.nt, case.stride, case.mode,
                            case.record, nrec, case.src_comp, case.src_map.shape[1],
                            case.src_map.shape[2], case.nt, path, flags, case.h, case.dt)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _forward(lib, prob, ins, shape):
    """ernn_forward without a tape (the library's allocating entry point)."""
    tape_bytes = lib.ernn_tape_bytes(ctypes.byref(prob), 0)
    tape = torch.empty(tape_bytes, dtype=torch.uint8, device=DEV)
    out_x = torch.empty(shape, device=DEV)
    out_y = torch.empty(shape, device=DEV)
    rc = lib.ernn_forward(ctypes.byref(prob), ctypes.byref(ins), ctypes.c_void_p(out_x.data_ptr()),
                          ctypes.c_void_p(out_y.data_ptr()), ctypes.c_void_p(tape.data_ptr()),
                          ctypes.c_size_t(tape_bytes), 0, _stream())
    assert rc == 0, lib.ernn_error_string(rc)
    return out_x, out_y


def _static(lib, prob, ins, shape):
    out_x = torch.full(shape, float("nan"), device=DEV)
    out_y = torch.full(shape, float("nan"), device=DEV)
    rc = lib.ernn_forward_static(ctypes.byref(prob), ctypes.byref(ins), ctypes.c_void_p(out_x.data_ptr()),
                                 ctypes.c_void_p(out_y.data_ptr()), _stream())
    return rc, out_x, out_y


def _per_shot_constants(case, seed=3):
    rng = np.random.default_rng(seed)
    return np.stack([case.C * rng.uniform(0.9, 1.1, size=6) for _ in range(case.nshots)])


CASES = {
    "fields_multishot": (dict(nx=48, ny=40, nt=120, stride=3, S=2), False),
    "receivers_multishot": (dict(nx=37, ny=29, nt=90, S=3, record=O.RECORD_RECEIVERS, nrec=11), False),
    "dfield": (dict(nx=30, ny=30, nt=60, mode=O.MODE_DFIELD), False),
    "six_planes": (dict(nx=26, ny=31, nt=50, mode=O.MODE_FIELDS, record=O.RECORD_RECEIVERS, nrec=5), False),
    "per_shot_constants": (dict(nx=40, ny=36, nt=80, S=3, record=O.RECORD_RECEIVERS, nrec=9), True),
}


@pytest.mark.parametrize("name", list(CASES))
def test_static_forward_equals_forward_twice(name):
    kw, per_shot = CASES[name]
    lib = E.load_library()
    case = random_case(**kw)
    C = _per_shot_constants(case) if per_shot else None
    keep, ins = _tensors(case, C)
    prob = _problem(case, flags=_lib.FLAG_SHOT_CONSTANTS if per_shot else 0)
    shape = case.out_shape()
    ref_x, ref_y = _forward(lib, prob, ins, shape)
    for _ in range(2):
        rc, out_x, out_y = _static(lib, prob, ins, shape)
        assert rc == 0, lib.ernn_error_string(rc)
        torch.cuda.synchronize()
        assert lib.ernn_last_path() == _lib.PATH_STEP
        assert torch.equal(out_x, ref_x) and torch.equal(out_y, ref_y)


def test_static_forward_vs_fp64_oracle():
    lib = E.load_library()
    case = random_case(nx=44, ny=38, nt=150, stride=2, S=2, record=O.RECORD_RECEIVERS, nrec=13)
    keep, ins = _tensors(case)
    prob = _problem(case, path=_lib.PATH_AUTO)
    rx, ry, _ = O.forward(case, "f64")
    for _ in range(2):
        rc, out_x, out_y = _static(lib, prob, ins, case.out_shape())
        assert rc == 0, lib.ernn_error_string(rc)
        gx, gy = out_x.cpu().numpy(), out_y.cpu().numpy()
        assert rel(gx, rx) <= FWD_TOL and rel(gy, ry) <= FWD_TOL, (rel(gx, rx), rel(gy, ry))


def _static_bytes(nshots, nx, ny, ncoef=1):
    a = lambda v: (v + 255) // 256 * 256
    return a(64 * ncoef) + 2 * a(nshots * 2 * nx * ny * 4)


def test_static_forward_at_its_size_limit():
    # the largest square grid whose two state levels fit the array, and the
    # next size up, which must be rejected with ERNN_ERR_WORKSPACE
    side = 724
    assert _static_bytes(1, side, side) <= LIMIT < _static_bytes(1, side + 1, side)
    lib = E.load_library()
    case = random_case(nx=side, ny=side, nt=6, stride=2, record=O.RECORD_RECEIVERS, nrec=17)
    keep, ins = _tensors(case)
    prob = _problem(case)
    ref_x, ref_y = _forward(lib, prob, ins, case.out_shape())
    for _ in range(2):
        rc, out_x, out_y = _static(lib, prob, ins, case.out_shape())
        assert rc == 0, lib.ernn_error_string(rc)
        torch.cuda.synchronize()
        assert torch.equal(out_x, ref_x) and torch.equal(out_y, ref_y)
    prob.nx = side + 1
    out = torch.empty(1, device=DEV)
    rc = lib.ernn_forward_static(ctypes.byref(prob), ctypes.byref(ins), ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(out.data_ptr()), _stream())
    assert rc == 2  # ERNN_ERR_WORKSPACE


def test_static_forward_rejects_other_kernel_paths():
    lib = E.load_library()
    case = random_case(nx=32, ny=32, nt=4)
    keep, ins = _tensors(case)
    out = torch.empty(case.out_shape(), device=DEV)
    for path in (_lib.PATH_RESIDENT, _lib.PATH_TILED):
        prob = _problem(case, path=path)
        rc = lib.ernn_forward_static(ctypes.byref(prob), ctypes.byref(ins), ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), _stream())
        assert rc == 6  # ERNN_ERR_UNSUPPORTED
