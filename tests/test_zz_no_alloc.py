"""The allocation-free forward entry point, ernn_forward_static.

Some callers of this library cannot call cudaMalloc around a propagation
(code running while another framework captures a CUDA graph, real-time loops
that cannot afford an allocation's device synchronisation, FFI hosts with no
device allocator).  ernn_forward_static keeps its wavefield scratch in an
8 MiB device array owned by the library.  Here it is called through the C ABI
and compared with ernn_forward on the same inputs, on two calls in a row (the
second call reuses the scratch the first one left behind).  This file is
collected last so that a run stopping at the first failure has run every
other test first.
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
TOL = 1e-4   # forward tolerance of the parity tests


def _tensors(case):
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(DEV).contiguous()
    keep = dict(C=t(case.C), rho=t(np.array([case.rho])), sig=t(case.src_signal), smap=t(case.src_map),
                org=t(case.src_origin, torch.int32),
                rec=None if case.rec_idx is None else t(case.rec_idx, torch.int32),
                D=None if case.D is None else t(case.D))
    p = lambda x: None if x is None else ctypes.c_void_p(x.data_ptr())
    ins = _lib.ErnnInputs(p(keep["C"]), p(keep["D"]), p(keep["rho"]), p(keep["sig"]), p(keep["smap"]),
                          p(keep["org"]), p(keep["rec"]))
    return keep, ins


def _problem(case):
    nrec = 0 if case.rec_idx is None else case.rec_idx.shape[1]
    return _lib.ErnnProblem(case.nshots, case.nx, case.ny, case.nt, case.stride, case.mode,
                            case.record, nrec, case.src_comp, case.src_map.shape[1],
                            case.src_map.shape[2], case.nt, _lib.PATH_STEP, 0, case.h, case.dt)


@pytest.mark.parametrize("kw", [dict(nx=48, ny=40, nt=120, stride=3, S=2),
                                dict(nx=37, ny=29, nt=90, S=3, record=O.RECORD_RECEIVERS, nrec=11),
                                dict(nx=30, ny=30, nt=60, mode=O.MODE_DFIELD)])
def test_static_forward_matches_forward_twice(kw):
    lib = E.load_library()
    case = random_case(**kw)
    keep, ins = _tensors(case)
    prob = _problem(case)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    shape = case.out_shape()
    tape_bytes = lib.ernn_tape_bytes(ctypes.byref(prob), 0)
    tape = torch.empty(tape_bytes, dtype=torch.uint8, device=DEV)
    ref_x = torch.empty(shape, device=DEV)
    ref_y = torch.empty(shape, device=DEV)
    rc = lib.ernn_forward(ctypes.byref(prob), ctypes.byref(ins), ctypes.c_void_p(ref_x.data_ptr()),
                          ctypes.c_void_p(ref_y.data_ptr()), ctypes.c_void_p(tape.data_ptr()),
                          ctypes.c_size_t(tape_bytes), 0, stream)
    assert rc == 0
    for _ in range(2):
        out_x = torch.full(shape, float("nan"), device=DEV)
        out_y = torch.full(shape, float("nan"), device=DEV)
        rc = lib.ernn_forward_static(ctypes.byref(prob), ctypes.byref(ins),
                                     ctypes.c_void_p(out_x.data_ptr()),
                                     ctypes.c_void_p(out_y.data_ptr()), stream)
        assert rc == 0, lib.ernn_error_string(rc)
        torch.cuda.synchronize()
        assert rel(out_x.cpu().numpy(), ref_x.cpu().numpy()) <= TOL
        assert rel(out_y.cpu().numpy(), ref_y.cpu().numpy()) <= TOL


def test_static_forward_rejects_problems_beyond_its_scratch():
    lib = E.load_library()
    case = random_case(nx=48, ny=40, nt=4)
    keep, ins = _tensors(case)
    prob = _problem(case)
    prob.nx, prob.ny = 1024, 1024            # 2 levels x 2 x 4 MiB > 8 MiB
    out = torch.empty(1, device=DEV)
    rc = lib.ernn_forward_static(ctypes.byref(prob), ctypes.byref(ins), ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 2  # ERNN_ERR_WORKSPACE
