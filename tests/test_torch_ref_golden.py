"""The PyTorch restatement of the reference path (the benchmark's reference arm)
reproduces the reference's golden vectors on the CPU."""
import os

import numpy as np
import torch

from conftest import GOLDEN
from oracle import torch_ref


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def test_operator_matches_reference():
    g = np.load(os.path.join(GOLDEN, "operator_f32.npz"))
    t = lambda a: torch.tensor(a, dtype=torch.float32)
    C = [t(v) for v in g["C"]]
    Lx, Ly = torch_ref.operator(t(g["ux"])[None], t(g["uy"])[None], C, float(g["h"]),
                                t(g["fx"])[None], t(g["fy"])[None], t(float(g["rho"])))
    assert rel(Lx[0].numpy(), g["Lux"]) < 1e-6
    assert rel(Ly[0].numpy(), g["Luy"]) < 1e-6


def test_forward_and_autograd_gradient_match_reference():
    g = np.load(os.path.join(GOLDEN, "param_inversion_f32.npz"))
    nx, ny, nt, st = int(g["nx"]), int(g["ny"]), int(g["nt"]), int(g["stride"])
    logC = torch.tensor(np.log(g["C"]), dtype=torch.float32, requires_grad=True)
    C = [torch.exp(logC[i]) for i in range(6)]
    ux, uy = torch_ref.propagate(C, torch.tensor(float(g["rho"])), nx, ny, nt, float(g["h"]),
                                 float(g["dt"]), torch.tensor(g["signal"], dtype=torch.float32)[None],
                                 torch.tensor(g["gauss"], dtype=torch.float32)[None], stride=st)
    assert rel(ux.detach().numpy(), g["hist_ux"]) < 1e-5
    ts, ss = int(g["ts"]), int(g["ss"])
    tx = torch.tensor(g["target_ux"], dtype=torch.float32)
    ty = torch.tensor(g["target_uy"], dtype=torch.float32)
    loss = torch.mean((ux[:, ::ts, ::ss, ::ss] - tx[:, ::ts, ::ss, ::ss]) ** 2) + \
        torch.mean((uy[:, ::ts, ::ss, ::ss] - ty[:, ::ts, ::ss, ::ss]) ** 2)
    loss.backward()
    assert rel(logC.grad.numpy(), g["grad_log"]) < 5e-5
