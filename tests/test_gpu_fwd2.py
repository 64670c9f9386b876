"""Two-step tiled forward (u^{i+1} and u^{i+2} in one launch) in the
recompute segments of the checkpointed adjoint: gradients against the FP64
oracle and against the plain per-step kernels, on segment lengths that pair
every step (even) or leave a single step (odd), ragged and tiny grids, loads
on the grid edge, several shots and per-shot constants.  GPU only."""
import numpy as np
import pytest
import torch

import ernn_gb300 as E
from cases import C_ROT30, random_case, rel
from oracle import oracle as O
from test_gpu_parity import DEV, FWD_TOL, GRAD_TOL, run_gpu, run_oracle, to_geometry, weights

pytestmark = pytest.mark.gpu

CASES = {
    "receivers_multishot_even": (dict(nx=70, ny=132, nt=80, S=3, record=O.RECORD_RECEIVERS, nrec=40), 10),
    "receivers_multishot_odd": (dict(nx=70, ny=132, nt=80, S=3, record=O.RECORD_RECEIVERS, nrec=40), 9),
    "dense_ragged": (dict(nx=45, ny=76, nt=70), 7),
    "x_force_stride1": (dict(nx=33, ny=68, nt=70, stride=1, src_comp=0), 12),
    "narrow": (dict(nx=150, ny=8, nt=90, stride=5), 11),
    "tiny": (dict(nx=3, ny=4, nt=30, box=2), 6),
    "single_tile": (dict(nx=16, ny=64, nt=40), 5),
    "segment_of_two": (dict(nx=40, ny=64, nt=40, record=O.RECORD_RECEIVERS, nrec=6), 2),
}


@pytest.mark.parametrize("name", list(CASES))
def test_two_step_recompute_vs_oracle_and_plain(name):
    kw, ckpt = CASES[name]
    case = random_case(**kw)
    wx, wy = weights(case)
    gx, gy, gg = run_gpu(case, wx, wy, ckpt_k=ckpt, path=E.PATH_TILED)
    rx, ry, rg = run_oracle(case, wx, wy)
    assert rel(gx, rx) <= FWD_TOL and rel(gy, ry) <= FWD_TOL
    assert rel(gg, rg) <= GRAD_TOL, rel(gg, rg)
    sx, sy, sg = run_gpu(case, wx, wy, ckpt_k=ckpt, path=E.PATH_STEP)
    assert rel(gg, sg) <= 1e-5, rel(gg, sg)


def test_two_step_recompute_per_shot_constants():
    S = 4
    case = random_case(nx=64, ny=128, nt=60, S=S, record=O.RECORD_RECEIVERS, nrec=12)
    geom = to_geometry(case, ckpt_k=8, path=E.PATH_TILED)
    rng = np.random.default_rng(2)
    Cs = np.stack([C_ROT30 * rng.uniform(0.9, 1.1, 6) for _ in range(S)]).astype(np.float32)
    wx, wy = weights(case)
    C = torch.tensor(Cs, device=DEV, requires_grad=True)
    rho = torch.full((S,), float(case.rho), device=DEV)
    ox, oy = E.propagate(C, rho, geom)
    ((ox.double() * torch.as_tensor(wx, device=DEV)).sum() +
     (oy.double() * torch.as_tensor(wy, device=DEV)).sum()).backward()
    assert E._lib.load().ernn_last_path() == E.PATH_TILED
    for s in range(S):
        one = O.Case(case.nx, case.ny, case.nt, case.h, case.dt, case.rho, Cs[s].astype(np.float64),
                     case.src_signal[s:s + 1], case.src_map[s:s + 1], case.src_origin[s:s + 1],
                     stride=case.stride, mode=case.mode, record=case.record,
                     rec_idx=case.rec_idx[s:s + 1], src_comp=case.src_comp)
        _, _, rg = run_oracle(one, wx[s:s + 1], wy[s:s + 1])
        assert rel(C.grad[s].cpu().numpy(), rg) <= GRAD_TOL, (s, rel(C.grad[s].cpu().numpy(), rg))
