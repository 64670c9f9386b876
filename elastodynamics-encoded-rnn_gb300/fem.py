"""FEM data generator on the GPU: the step before the ERNN path.

`solve_2d_anisotropic_wave_fem_ricker_fixed` keeps the signature and the
return tuple of the reference generator
(Parameter_inversion/FEM_generate_data.py:196-590): the same mesh, CFL
adjustment of dt / nt, Ricker source with a Gaussian nodal load, lumped mass,
fixed edges and 0.7-scaled displacement fields (nx, ny, nt).  The time loop
runs in `ernn_fem_forward` (one fused node-gather kernel per step, no atomics);
`stride` > 1 keeps only every stride-th time level on the device, which is
what `generate_data_file` saves (the generator's `_ds<stride>` files,
FEM_generate_data.py:901-946).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _lib
from . import formats


def gaussian_point_load(x, y, x0, y0, a=150):
    """(a / pi) exp(-a r^2) (FEM_generate_data.py:51-66)."""
    r2 = (x - x0) ** 2 + (y - y0) ** 2
    return (a / np.pi) * np.exp(-a * r2)


def ricker_wavelet(t, f0, t0, amplitude=1.0):
    """A (1 - 2 (pi f0 tau)^2) exp(-(pi f0 tau)^2), tau = t - t0 (FEM_generate_data.py:69-88)."""
    s = (np.pi * f0 * (np.asarray(t) - t0)) ** 2
    return amplitude * (1 - 2 * s) * np.exp(-s)


def calculate_fwhm(a):
    return 2 * np.sqrt(np.log(2) / a)


def calculate_wave_velocities_anisotropic(C11, C22, C12, C16, C26, C66, rho):
    """(vp, vs, anisotropy) estimates the generator's CFL check uses (FEM_generate_data.py:96-112)."""
    vp = np.sqrt(max(C11, C22) / rho)
    vs = np.sqrt(C66 / rho)
    return vp, vs, abs(C11 - C22) / (C11 + C22)


def create_structured_triangular_mesh(nx, ny, Lx, Ly):
    """(x, y, elements, boundary_nodes, dx, dy) of the checkerboard triangular
    mesh, node id j*nx + i (FEM_generate_data.py:117-185)."""
    dx, dy = Lx / (nx - 1), Ly / (ny - 1)
    x = np.linspace(-Lx / 2, Lx / 2, nx)
    y = np.linspace(-Ly / 2, Ly / 2, ny)
    i, j = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), indexing="xy")
    n0 = j * nx + i
    n1, n2, n3 = n0 + 1, n0 + nx + 1, n0 + nx
    even = ((i + j) % 2 == 0)
    lower = np.where(even[..., None], np.stack([n0, n1, n2], -1), np.stack([n0, n1, n3], -1))
    upper = np.where(even[..., None], np.stack([n0, n2, n3], -1), np.stack([n1, n2, n3], -1))
    elements = np.stack([lower, upper], axis=2).reshape(-1, 3).astype(np.int64)
    b = np.zeros((ny, nx), dtype=bool)
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = True
    boundary = np.flatnonzero(b.reshape(-1)).astype(np.int64)
    return x, y, elements, boundary, dx, dy


def _time_axis(nt, t_total, dx, dy, C11, C22, C66, rho):
    """The generator's dt and its CFL adjustment (FEM_generate_data.py:274-292)."""
    vp, vs, _ = calculate_wave_velocities_anisotropic(C11, C22, 0, 0, 0, C66, rho)
    dt = t_total / (nt - 1)
    t = np.linspace(0, t_total, nt)
    vmax = max(vp, vs)
    if vmax * dt / min(dx, dy) > 0.5:
        dt_stable = 0.5 * min(dx, dy) / vmax
        nt = int(t_total / dt_stable) + 1
        dt = t_total / (nt - 1)
        t = np.linspace(0, t_total, nt)
    return t, dt, nt


def create_damage_regions(X, Y, damage_configs):
    """(damage_mask, damage_info): union of circles (|r - c| <= size) and squares
    (|x - cx|, |y - cy| <= size) on the node grid
    (Damage_inversion/FEM_generate_data.py:121-180)."""
    mask = np.zeros_like(X, dtype=bool)
    regions = []
    for k, cfg in enumerate(damage_configs):
        cx, cy = cfg["center"]
        if cfg["type"] == "circle":
            region = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) <= cfg["size"]
        elif cfg["type"] == "square":
            region = (np.abs(X - cx) <= cfg["size"]) & (np.abs(Y - cy) <= cfg["size"])
        else:
            raise ValueError(f"Unknown damage type: {cfg['type']}")
        mask |= region
        regions.append({"id": k, "type": cfg["type"], "center": cfg["center"], "size": cfg["size"],
                        "reduction_factor": cfg.get("reduction_factor", 0.5),
                        "n_points": int(region.sum())})
    info = {"regions": regions, "total_damaged_points": int(mask.sum()),
            "damage_percentage": 100 * mask.sum() / mask.size}
    return mask, info


def apply_damage_to_stiffness(C11, C22, C12, C16, C26, C66, damage_mask, reduction_factor=0.5):
    """Six (nx, ny) constant fields, multiplied by `reduction_factor` on the
    damaged nodes (Damage_inversion/FEM_generate_data.py:183-214).  The
    generator calls it with 0.5 whatever the regions' own factors are."""
    out = []
    for c in (C11, C22, C12, C16, C26, C66):
        f = np.full(damage_mask.shape, c, dtype=np.float64)
        f[damage_mask] *= reduction_factor
        out.append(f)
    return tuple(out)


def fem_frames(nx, ny, nt, dx, dy, dt, rho, C, load, signal, stride=1, out_scale=0.7, device=None,
               C_fields=None):
    """Device frames (nt_out, nx, ny) per component from the library's time
    loop; `load` (nx, ny) and `signal` (nt,) as arrays or tensors; `C_fields`
    None or (6, nx, ny) per-node constants (each element takes those of the
    node nearest its centroid)."""
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    if torch.device(device).type != "cuda":
        raise RuntimeError("the FEM generator runs only on a CUDA device through libernn_gb300.so")
    lib = _lib.load()
    p = _lib.ErnnFemProblem(nx, ny, nt, stride, dx, dy, dt, rho,
                            (ctypes.c_double * 6)(*[float(c) for c in C]), out_scale)
    ld = torch.as_tensor(load, dtype=torch.float32, device=device).contiguous()
    sg = torch.as_tensor(signal, dtype=torch.float32, device=device).contiguous()
    if tuple(ld.shape) != (nx, ny) or tuple(sg.shape) != (nt,):
        raise ValueError("load must be (nx, ny) and signal (nt,)")
    cf = None
    if C_fields is not None:
        cf = torch.as_tensor(np.asarray(C_fields, dtype=np.float32) if not torch.is_tensor(C_fields)
                             else C_fields, dtype=torch.float32, device=device).contiguous()
        if tuple(cf.shape) != (6, nx, ny):
            raise ValueError("C_fields must be (6, nx, ny)")
    nt_out = (nt + stride - 1) // stride
    with torch.cuda.device(device):
        fx = torch.empty((nt_out, nx, ny), dtype=torch.float32, device=device)
        fy = torch.empty_like(fx)
        nbytes = lib.ernn_fem_workspace_bytes(ctypes.byref(p))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
        rc = lib.ernn_fem_forward(ctypes.byref(p), ctypes.c_void_p(ld.data_ptr()),
                                  ctypes.c_void_p(sg.data_ptr()),
                                  ctypes.c_void_p(None if cf is None else cf.data_ptr()),
                                  ctypes.c_void_p(fx.data_ptr()),
                                  ctypes.c_void_p(fy.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                                  ctypes.c_size_t(nbytes), stream)
        _lib.check("ernn_fem_forward", rc)
    return fx, fy


def solve_2d_anisotropic_wave_fem_ricker_fixed(nx=301, ny=301, Lx=0.4, Ly=0.4, nt=1001,
                                               t_total=30e-6, source_amplitude=1e13,
                                               source_f0=170e3, source_t0=6e-6,
                                               gaussian_param=5e8, C11=16.5e10, C22=6.2e10,
                                               C12=5.0e10, C16=0.0, C26=0.0, C66=3.96e10,
                                               rho=7100.0, source_position=(0.0, 0.0),
                                               device=None, stride=1, damage_configs=False):
    """The reference generator's contract: returns (x, y, t, u_x, u_y,
    total_displacement, source_mask, source_indices, nodes, elements,
    source_info), u_x / u_y (nx, ny, nt_out) numpy float32 scaled by 0.7,
    nt_out = nt with stride 1 (every time level, as the reference returns).
    `damage_configs` (a list, or None for the damaged-plate generator's
    default circle) switches to the damaged-plate generator
    (Damage_inversion/FEM_generate_data.py:770-1224): stiffness halved on the
    damaged nodes, each element taking the constants of the node nearest its
    centroid; source_info then carries damage_mask, damage_info, damage_configs."""
    x, y, elements, boundary, dx, dy = create_structured_triangular_mesh(nx, ny, Lx, Ly)
    t, dt, nt = _time_axis(nt, t_total, dx, dy, C11, C22, C66, rho)
    x0, y0 = source_position
    X, Y = np.meshgrid(x, y, indexing="ij")
    gauss = gaussian_point_load(X, Y, x0, y0, gaussian_param)
    signal = ricker_wavelet(t, source_f0, source_t0, source_amplitude)
    C = (C11, C22, C12, C16, C26, C66)
    C_fields, damage = None, None
    if damage_configs is not False:
        if damage_configs is None:  # the damaged-plate generator's default
            damage_configs = [{"type": "circle", "center": (0.1, 0.1), "size": 0.02,
                               "reduction_factor": 0.5}]
        mask, dinfo = create_damage_regions(X, Y, damage_configs)
        C_fields = np.stack(apply_damage_to_stiffness(*C, mask, reduction_factor=0.5))
        damage = {"damage_mask": mask, "damage_info": dinfo, "damage_configs": damage_configs}
    fx, fy = fem_frames(nx, ny, nt, dx, dy, dt, rho, C, gauss, signal, stride=stride, device=device,
                        C_fields=C_fields)
    ux = fx.permute(1, 2, 0).cpu().numpy()
    uy = fy.permute(1, 2, 0).cpu().numpy()
    total = np.sqrt(ux ** 2 + uy ** 2)
    last_x = ux[boundary % nx, boundary // nx, -1]
    last_y = uy[boundary % nx, boundary // nx, -1]
    vp, vs, aniso = calculate_wave_velocities_anisotropic(C11, C22, C12, C16, C26, C66, rho)
    jj, ii = np.divmod(np.arange(nx * ny), nx)
    nodes = np.stack([x[ii], y[jj]], axis=1)
    source_mask = gauss > 0.01 * np.max(gauss)
    source_indices = [int(np.argmin(np.abs(y - y0))) * nx + int(np.argmin(np.abs(x - x0)))]
    info = {"source_amplitude": source_amplitude, "source_f0": source_f0, "source_t0": source_t0,
            "gaussian_param": gaussian_param, "fwhm": calculate_fwhm(gaussian_param),
            "C11": C11, "C22": C22, "C12": C12, "C16": C16, "C26": C26, "C66": C66, "rho": rho,
            "vp_approx": vp, "vs_approx": vs, "anisotropy_factor": aniso,
            "boundary_condition": "fixed",
            "max_u_boundary": float(max(np.abs(last_x).max(), np.abs(last_y).max()))}
    if damage is not None:
        info.update(damage)
    return x, y, t, ux, uy, total, source_mask, source_indices, nodes, elements, info


def generate_data_file(output_dir, stride=5, device=None, **kw):
    """Run the generator and save its `_ds<stride>` wavefield file
    (FEM_generate_data.py:901-946): datasets ux, uy (nt_ds, nx, ny), x, y,
    t[::stride], source_info.  HDF5 when h5py is installed, else .npz with the
    same names.  Returns the path written."""
    x, y, t, ux, uy, _, _, _, _, _, info = solve_2d_anisotropic_wave_fem_ricker_fixed(
        device=device, stride=stride, **kw)
    os.makedirs(output_dir, exist_ok=True)
    damaged = "damage_mask" in info
    name = f"anisotropic_ricker_{'damage_' if damaged else ''}data_ds{stride}_FEM_fixed_bc"
    extra = {}
    if damaged:  # Damage_inversion/FEM_generate_data.py:1656-1672
        d = info["damage_info"]
        extra = {"damage_mask": info["damage_mask"].astype(np.uint8),
                 "damage_info/total_damaged_points": d["total_damaged_points"],
                 "damage_info/damage_percentage": d["damage_percentage"]}
        for r in d["regions"]:
            for key in ("type", "center", "size", "reduction_factor", "n_points"):
                extra[f"damage_info/region_{r['id']}/{key}"] = np.asarray(r[key])
    info = {k: v for k, v in info.items() if k not in ("damage_mask", "damage_info", "damage_configs")}
    path = os.path.join(output_dir, name + (".mat" if formats.h5py is not None else ".npz"))
    return formats.save_wavefields(path, np.moveaxis(ux, 2, 0), np.moveaxis(uy, 2, 0), x, y,
                                   t[::stride], info, extra)
