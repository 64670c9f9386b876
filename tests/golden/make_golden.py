"""Generate the golden vectors in tests/golden/ from the reference module itself.

Run where the reference is checked out, giving its location as the first
argument or in the ERNN_REFERENCE environment variable:
  python tests/golden/make_golden.py <reference checkout>
The reference is imported unmodified:
  * Parameter_inversion/Inversion_adam.py is imported as a module with stub
    modules for matplotlib and h5py (absent here, unused on this path);
  * Parameter_inversion/FEM_generate_data.py likewise (its solver runs on the
    CPU here; plots are stubbed);
  * Damage_inversion/Inversion_adam.py selects a GPU at import time
    (Inversion_adam.py:36-43), so only its definitions are extracted with `ast`
    and executed with `device` bound to the CPU.

Each fixture stores the exact inputs the reference used (constants after
exp/clamp, the Gaussian load map, the source signal) and its outputs
(operator values, forward histories, loss, autograd gradients), in FP32 and in
the FP64 run of the same scheme (torch default dtype float64).
"""
from __future__ import annotations

import ast
import importlib.util
import os
import sys
import types
from unittest import mock

import numpy as np
import torch

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ERNN_REFERENCE")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: make_golden.py <reference checkout>  (or set ERNN_REFERENCE)")
OUT = os.path.dirname(os.path.abspath(__file__))
sys.dont_write_bytecode = True


def _stub_plotting():
    for name in ["matplotlib", "matplotlib.pyplot", "matplotlib.ticker", "matplotlib.colors",
                 "matplotlib.patches", "matplotlib.collections", "mpl_toolkits",
                 "mpl_toolkits.axes_grid1", "h5py"]:
        sys.modules.setdefault(name, mock.MagicMock(name=name))


def load_param_module():
    _stub_plotting()
    path = os.path.join(REF, "Parameter_inversion", "Inversion_adam.py")
    spec = importlib.util.spec_from_file_location("ref_param_inversion", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_damage_defs():
    path = os.path.join(REF, "Damage_inversion", "Inversion_adam.py")
    tree = ast.parse(open(path).read(), filename=path)
    keep = {"gaussian_point_load", "ricker_wavelet", "conv2d_fixed",
            "_general_anisotropic_elastic_operator_with_force_spatially_varying",
            "total_variation_2d", "SpatiallyVaryingAnisotropicSimulator",
            "SpatiallyVaryingParameterInverter"}
    body = [n for n in tree.body
            if isinstance(n, (ast.FunctionDef, ast.ClassDef)) and n.name in keep]
    ns = {"torch": torch, "nn": torch.nn, "F": torch.nn.functional, "np": np,
          "optim": torch.optim, "os": os, "device": torch.device("cpu")}
    exec(compile(ast.Module(body=body, type_ignores=[]), path, "exec"), ns)
    return types.SimpleNamespace(**{k: ns[k] for k in keep})


# --------------------------------------------------------------------------
H, DT, RHO = 1e-4, 5e-9, 1610.0
TRUE = dict(C11=160.06e9, C22=70.86e9, C12=48.04e9, C16=9.48e9, C26=16.27e9, C66=37.64e9)
INIT = dict(C11=150e9, C22=75e9, C12=45e9, C16=11e9, C26=15e9, C66=39e9)
SRC = dict(source_f0=4e6, source_t0=2.5e-7, source_amplitude=1e10, gaussian_param=5e6)


def param_case(P, dtype, domain=(24, 20), nt=150, stride=5, ts=2, ss=3):
    torch.set_default_dtype(dtype)
    try:
        def make(C):
            return P.CFRPWaveSimulatorRicker(
                domain, H, DT, nt, stride, source_component="y", rho_known=RHO,
                source_position=(0.0, 0.0),
                C11_init=C["C11"], C22_init=C["C22"], C12_init=C["C12"],
                C16_init=C["C16"], C26_init=C["C26"], C66_init=C["C66"], **SRC)
        true_sim = make(TRUE)
        with torch.no_grad():
            tx, ty = true_sim()
        sim = make(INIT)
        inv = P.CFRPParameterInverterRicker(sim, tx, ty, secondary_time_stride=ts,
                                            secondary_space_stride=ss)
        ux, uy = sim(save_all_steps=False)
        loss = inv.compute_loss(ux, uy)
        loss.backward()
        C = sim.get_material_params()
        names = ["log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66"]
        return dict(
            nx=domain[0], ny=domain[1], nt=nt, stride=stride, ts=ts, ss=ss, h=H, dt=DT,
            rho=float(sim.rho), C=np.array([float(c) for c in C[:6]], np.float64),
            C_true=np.array([float(c) for c in true_sim.get_material_params()[:6]]),
            gauss=sim.gaussian_dist.detach().double().numpy(),
            signal=sim.source_signal.detach().double().numpy()[0],
            hist_ux=ux.detach().double().numpy(), hist_uy=uy.detach().double().numpy(),
            target_ux=tx.double().numpy(), target_uy=ty.double().numpy(),
            loss=float(loss), grad_log=np.array([float(getattr(sim, n).grad) for n in names]))
    finally:
        torch.set_default_dtype(torch.float32)


def invert_case(P, domain=(24, 20), nt=150, stride=5, ts=2, ss=3, epochs=6, lr=1e-2):
    """The reference's own inversion loop, CFRPParameterInverterRicker.invert
    (Parameter_inversion/Inversion_adam.py:393-483), for a few Adam epochs in
    float32: its loss and constants after every epoch."""
    torch.set_default_dtype(torch.float32)
    def make(C):
        return P.CFRPWaveSimulatorRicker(
            domain, H, DT, nt, stride, source_component="y", rho_known=RHO,
            source_position=(0.0, 0.0),
            C11_init=C["C11"], C22_init=C["C22"], C12_init=C["C12"],
            C16_init=C["C16"], C26_init=C["C26"], C66_init=C["C66"], **SRC)
    with torch.no_grad():
        tx, ty = make(TRUE)()
    sim = make(INIT)
    inv = P.CFRPParameterInverterRicker(sim, tx, ty, secondary_time_stride=ts,
                                        secondary_space_stride=ss)
    inv.get_results = lambda *a, **k: None  # the summary printout is not part of the loop
    inv.invert(max_epochs=epochs, lr=lr)
    h = inv.history
    return dict(nx=domain[0], ny=domain[1], nt=nt, stride=stride, ts=ts, ss=ss, h=H, dt=DT, rho=RHO,
                epochs=epochs, lr=lr, target_ux=tx.double().numpy(), target_uy=ty.double().numpy(),
                loss=np.array(h["loss"]),
                params=np.array([h[k] for k in ("C11", "C22", "C12", "C16", "C26", "C66")]).T)


def operator_case(P, Dm, dtype, nx=19, ny=16, nsq=17, seed=3):
    torch.set_default_dtype(dtype)
    try:
        g = torch.Generator().manual_seed(seed)
        ux = torch.randn(1, nx, ny, generator=g) * 1e-3
        uy = torch.randn(1, nx, ny, generator=g) * 1e-3
        fx = torch.randn(1, nx, ny, generator=g) * 1e16
        fy = torch.randn(1, nx, ny, generator=g) * 1e16
        Cs = [torch.tensor(v, dtype=torch.float32) for v in TRUE.values()]
        rho = torch.tensor(RHO, dtype=torch.float32)
        Lx, Ly = P._general_anisotropic_elastic_operator_with_force(ux, uy, *Cs, H, fx, fy, rho)
        # The spatially varying operator adds the force transposed
        # (Damage_inversion/Inversion_adam.py:169-174), so it only accepts square
        # grids; its case uses its own square fields and an asymmetric force.
        n = nsq
        vx = torch.randn(1, n, n, generator=g) * 1e-3
        vy = torch.randn(1, n, n, generator=g) * 1e-3
        gx = torch.randn(1, n, n, generator=g) * 1e16
        gy = torch.randn(1, n, n, generator=g) * 1e16
        base = torch.tensor(list(TRUE.values()), dtype=torch.float32).view(6, 1, 1)
        fields = (base * (1 + 0.2 * torch.rand(6, n, n, generator=g))).to(torch.float32)
        Lxf, Lyf = Dm._general_anisotropic_elastic_operator_with_force_spatially_varying(
            vx, vy, *[fields[t:t + 1] for t in range(6)], H, gx, gy, rho)
        d = lambda a: a.detach().double().numpy()
        return dict(nx=nx, ny=ny, h=H, rho=RHO, C=np.array([float(c) for c in Cs]),
                    ux=d(ux[0]), uy=d(uy[0]), fx=d(fx[0]), fy=d(fy[0]),
                    Lux=d(Lx[0]), Luy=d(Ly[0]), nsq=n, C_fields=d(fields), vx=d(vx[0]),
                    vy=d(vy[0]), gx=d(gx[0]), gy=d(gy[0]), Lux_fields=d(Lxf[0]),
                    Luy_fields=d(Lyf[0]))
    finally:
        torch.set_default_dtype(torch.float32)


def damage_case(Dm, dtype, domain=(20, 20), nt=120, stride=5, ts=2, seed=7, lambda_tv=0.0):
    torch.set_default_dtype(dtype)
    try:
        base = dict(C11_init=130.74e9, C22_init=11.50e9, C12_init=10.49e9, C16_init=30.67e9,
                    C26_init=3.75e9, C66_init=14.77e9)
        def make():
            return Dm.SpatiallyVaryingAnisotropicSimulator(
                domain, H, DT, nt, stride, source_component="y", total_time=nt * DT,
                rho_known=RHO, use_log_params=True, **base, **SRC)
        healthy = make()
        with torch.no_grad():
            tx, ty = healthy()
        sim = make()
        g = torch.Generator().manual_seed(seed)
        with torch.no_grad():
            for n in ["log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66"]:
                p = getattr(sim, n)
                p.add_(0.08 * torch.randn(p.shape, generator=g))
        inv = Dm.SpatiallyVaryingParameterInverter(sim, tx, ty, secondary_time_stride=ts,
                                                   lambda_tv=lambda_tv)
        ux, uy = sim(save_all_steps=False)
        loss, loss_data, loss_tv = inv.compute_loss(ux, uy)
        loss.backward()
        C = sim.get_material_params()
        names = ["log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66"]
        d = lambda a: a.detach().double().numpy()
        return dict(
            nx=domain[0], ny=domain[1], nt=nt, stride=stride, ts=ts, h=H, dt=DT,
            rho=float(sim.rho), C_fields=np.stack([d(c[0]) for c in C[:6]]),
            gauss=d(sim.gaussian_dist), signal=d(sim.source_signal)[0],
            hist_ux=d(ux), hist_uy=d(uy), target_ux=d(tx), target_uy=d(ty), loss=float(loss),
            loss_data=float(loss_data), loss_tv=float(loss_tv), lambda_tv=lambda_tv,
            grad_log=np.stack([d(getattr(sim, n).grad[0]) for n in names]))
    finally:
        torch.set_default_dtype(torch.float32)


def load_fem_module(folder="Parameter_inversion"):
    _stub_plotting()
    path = os.path.join(REF, folder, "FEM_generate_data.py")
    spec = importlib.util.spec_from_file_location(f"ref_fem_generate_{folder}", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    # the solvers draw figures on their way; they are not part of the path
    for name in dir(mod):
        if name.startswith(("plot_", "visualize_")):
            setattr(mod, name, lambda *a, **k: None)
    return mod


FEM_CASES = {
    # CFL below 0.5: the requested dt is kept
    "fem": dict(nx=21, ny=21, Lx=0.02, Ly=0.02, nt=201, t_total=10e-6, source_amplitude=1e10,
                source_f0=500e3, source_t0=2e-6, gaussian_param=5e5, C11=130.74e9, C22=11.50e9,
                C12=10.49e9, C16=30.67e9, C26=3.75e9, C66=14.77e9, rho=1610.0,
                source_position=(0.0, 0.0)),
    # CFL above 0.5 and an off-centre source: the generator shortens dt
    "fem_cfl": dict(nx=17, ny=13, Lx=0.016, Ly=0.012, nt=61, t_total=6e-6, source_amplitude=1e10,
                    source_f0=500e3, source_t0=2e-6, gaussian_param=5e5, C11=130.74e9,
                    C22=11.50e9, C12=10.49e9, C16=30.67e9, C26=3.75e9, C66=14.77e9, rho=1610.0,
                    source_position=(0.002, -0.001)),
}


DAMAGE_FEM = dict(FEM_CASES["fem"], damage_configs=[
    {"type": "circle", "center": (0.004, 0.003), "size": 0.003, "reduction_factor": 0.5},
    {"type": "square", "center": (-0.005, -0.004), "size": 0.002, "reduction_factor": 0.7}])


def fem_case(F, kw):
    """The reference FEM generator run on the CPU in float32 (it moves
    everything to float32 tensors itself); plotting is stubbed and its output
    folder goes to a temporary directory."""
    import tempfile
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            x, y, t, ux, uy, tot, mask, src_idx, nodes, elements, info = \
                F.solve_2d_anisotropic_wave_fem_ricker_fixed(device=torch.device("cpu"), **kw)
        finally:
            os.chdir(cwd)
    X, Y = np.meshgrid(x, y, indexing="ij")
    gauss = F.gaussian_point_load(X, Y, kw["source_position"][0], kw["source_position"][1],
                                  kw["gaussian_param"])
    sig = np.array([F.ricker_wavelet(tn, kw["source_f0"], kw["source_t0"], kw["source_amplitude"])
                    for tn in t])
    extra = {}
    if "damage_mask" in info:
        cfg = kw["damage_configs"]
        extra = dict(damage_mask=info["damage_mask"],
                     damage_types=np.array([c["type"] for c in cfg]),
                     damage_centers=np.array([c["center"] for c in cfg], dtype=np.float64),
                     damage_sizes=np.array([c["size"] for c in cfg], dtype=np.float64),
                     damage_factors=np.array([c["reduction_factor"] for c in cfg], dtype=np.float64))
        kw = {k: v for k, v in kw.items() if k != "damage_configs"}
    return dict(nx=kw["nx"], ny=kw["ny"], nt=len(t), dt=float(t[1] - t[0]), t=t, x=x, y=y, **extra,
                dx=kw["Lx"] / (kw["nx"] - 1), dy=kw["Ly"] / (kw["ny"] - 1), rho=kw["rho"],
                C=np.array([kw[k] for k in ("C11", "C22", "C12", "C16", "C26", "C66")]),
                load=gauss.astype(np.float32), signal=sig.astype(np.float32),
                ux=ux.astype(np.float32), uy=uy.astype(np.float32), elements=elements,
                requested=np.array([kw["nt"], kw["t_total"]]),
                **{f"arg_{k}": np.asarray(v) for k, v in kw.items()})


def damage_invert_case(Dm, domain=(20, 20), nt=120, stride=5, ts=2, epochs=12, lr=0.02,
                       lambda_tv=1e-21):
    """The reference's own damage loop, SpatiallyVaryingParameterInverter.invert
    (Damage_inversion/Inversion_adam.py:465-557), for a few Adam epochs in
    float32 at its learning rate and TV weight (:827-830): targets from the
    same simulator with every constant halved inside a disc of radius 3 cells
    around cell (12, 8); loss history and mean constants after every epoch."""
    torch.set_default_dtype(torch.float32)
    base = dict(C11_init=130.74e9, C22_init=11.50e9, C12_init=10.49e9, C16_init=30.67e9,
                C26_init=3.75e9, C66_init=14.77e9)
    def make():
        return Dm.SpatiallyVaryingAnisotropicSimulator(
            domain, H, DT, nt, stride, source_component="y", total_time=nt * DT,
            rho_known=RHO, use_log_params=True, **base, **SRC)
    true = make()
    ii, jj = np.meshgrid(np.arange(domain[0]), np.arange(domain[1]), indexing="ij")
    disc = torch.tensor(((ii - 12) ** 2 + (jj - 8) ** 2 <= 9)[None], dtype=torch.float32)
    with torch.no_grad():
        for n in ["log_C11", "log_C22", "log_C12", "log_C16", "log_C26", "log_C66"]:
            getattr(true, n).add_(disc * float(np.log(0.5)))
        tx, ty = true()
    sim = make()
    inv = Dm.SpatiallyVaryingParameterInverter(sim, tx, ty, secondary_time_stride=ts, lambda_tv=lambda_tv)
    inv.get_results = lambda *a, **k: None  # the summary printout is not part of the loop
    inv.invert(max_epochs=epochs, lr=lr)
    h = inv.history
    return dict(nx=domain[0], ny=domain[1], nt=nt, stride=stride, ts=ts, h=H, dt=DT, rho=RHO,
                epochs=epochs, lr=lr, lambda_tv=lambda_tv, disc=disc.numpy()[0],
                target_ux=tx.double().numpy(), target_uy=ty.double().numpy(),
                loss=np.array(h["loss"]), loss_data=np.array(h["loss_data"]),
                means=np.array([h[k] for k in ("C11_mean", "C22_mean", "C12_mean", "C16_mean",
                                               "C26_mean", "C66_mean")]).T)


def misfit_case(P, Dm, shape=(1, 9, 13, 11), ts=2, ss=3, seed=5):
    """The two inverters' compute_loss (Parameter_inversion/Inversion_adam.py:358-391,
    Damage_inversion/Inversion_adam.py:441-463, without TV) on random float32
    histories, with the gradients of each loss to the predicted histories."""
    torch.set_default_dtype(torch.float32)
    g = torch.Generator().manual_seed(seed)
    px, py, tx, ty = (torch.randn(shape, generator=g) for _ in range(4))
    out = dict(px=px.numpy(), py=py.numpy(), tx=tx.numpy(), ty=ty.numpy(), ts=ts, ss=ss)
    for tag, inv in (("param", P.CFRPParameterInverterRicker(None, tx, ty, secondary_time_stride=ts,
                                                            secondary_space_stride=ss)),
                     ("damage", Dm.SpatiallyVaryingParameterInverter(None, tx, ty, secondary_time_stride=ts,
                                                                     lambda_tv=0.0))):
        ax, ay = px.clone().requires_grad_(True), py.clone().requires_grad_(True)
        loss = inv.compute_loss(ax, ay)
        loss = loss[0] if isinstance(loss, tuple) else loss
        loss.backward()
        out[f"{tag}_loss"] = float(loss)
        out[f"{tag}_gx"] = ax.grad.numpy()
        out[f"{tag}_gy"] = ay.grad.numpy()
    return out


def main():
    torch.manual_seed(0)
    P = load_param_module()
    Dm = load_damage_defs()
    for tag, dtype in (("f32", torch.float32), ("f64", torch.float64)):
        np.savez_compressed(os.path.join(OUT, f"operator_{tag}.npz"), **operator_case(P, Dm, dtype))
        np.savez_compressed(os.path.join(OUT, f"param_inversion_{tag}.npz"), **param_case(P, dtype))
        np.savez_compressed(os.path.join(OUT, f"damage_inversion_{tag}.npz"), **damage_case(Dm, dtype))
        # the reference run's regularisation weight (Damage_inversion/Inversion_adam.py:827)
        np.savez_compressed(os.path.join(OUT, f"damage_inversion_tv_{tag}.npz"),
                            **damage_case(Dm, dtype, lambda_tv=1e-21))
    np.savez_compressed(os.path.join(OUT, "param_invert_f32.npz"), **invert_case(P))
    np.savez_compressed(os.path.join(OUT, "misfit.npz"), **misfit_case(P, Dm))
    np.savez_compressed(os.path.join(OUT, "damage_invert_f32.npz"), **damage_invert_case(Dm))
    F = load_fem_module()
    torch.set_default_dtype(torch.float32)
    for name, kw in FEM_CASES.items():
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **fem_case(F, kw))
    FD = load_fem_module("Damage_inversion")
    np.savez_compressed(os.path.join(OUT, "fem_damage.npz"), **fem_case(FD, DAMAGE_FEM))
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    main()
