"""Data formats on either side of the propagation path.

Wavefield files: the FEM generator writes the time-subsampled displacement
fields as datasets `ux`, `uy` of shape (nt_ds, nx, ny) float32, coordinate
vectors `x`, `y`, the subsampled times `t` and a group `source_info` of
scalars and arrays, into a file whose name carries the subsampling stride as
`_ds<stride>` (Parameter_inversion/FEM_generate_data.py:901-946).  The
inversion scripts read it back with `load_reference_data`
(Parameter_inversion/Inversion_adam.py:514-587): fields as (1, nt_ds, nx, ny)
float32 tensors on the compute device, optional noise at a given SNR, and a
metadata dictionary.  The same layout is read and written here through h5py
when it is importable, and otherwise as an `.npz` archive holding the same
names (`source_info/<key>` for the group members), so data prepared on a
machine with HDF5 and data prepared without it feed the same loader.

Receiver traces: `(S, nt_out, R)` per component, the output of the
RECORD_RECEIVERS mode, stored with the flat receiver cells and the time axis.
"""
from __future__ import annotations

import os
import re

import numpy as np
import torch

try:  # optional: the HDF5 form of the files
    import h5py  # type: ignore
except ImportError:  # pragma: no cover - depends on the machine
    h5py = None

_STRIDE = re.compile(r"_ds(\d+)")
DEFAULT_STRIDE = 5  # Inversion_adam.py:575 when the name carries none


def primary_stride(path: str) -> int:
    """Subsampling stride from a `_ds<stride>` file name (5 when absent)."""
    m = _STRIDE.search(os.path.basename(path))
    return int(m.group(1)) if m else DEFAULT_STRIDE


def _is_hdf5(path: str) -> bool:
    with open(path, "rb") as f:
        return f.read(8) == b"\x89HDF\r\n\x1a\n"


def save_wavefields(path: str, ux, uy, x, y, t, source_info: dict | None = None,
                    extra: dict | None = None) -> str:
    """Write (nt_ds, nx, ny) fields in the generator's layout.  HDF5 when
    h5py is present and the name does not end in `.npz`, else `.npz` (the
    suffix is added when missing).  `extra` maps further dataset paths
    ("damage_mask", "damage_info/region_0/size", ...) to values, as the
    damaged-plate generator writes them.  Returns the path written."""
    ux = np.asarray(ux, dtype=np.float32)
    uy = np.asarray(uy, dtype=np.float32)
    if ux.ndim != 3 or ux.shape != uy.shape:
        raise ValueError("ux and uy must both be (nt_ds, nx, ny)")
    info = dict(source_info or {})
    if h5py is not None and not path.endswith(".npz"):
        with h5py.File(path, "w") as f:
            f.create_dataset("ux", data=ux, chunks=(1,) + ux.shape[1:])
            f.create_dataset("uy", data=uy, chunks=(1,) + uy.shape[1:])
            f.create_dataset("x", data=np.asarray(x, dtype=np.float32))
            f.create_dataset("y", data=np.asarray(y, dtype=np.float32))
            f.create_dataset("t", data=np.asarray(t, dtype=np.float32))
            g = f.create_group("source_info")
            for k, v in info.items():
                g.create_dataset(k, data=v if np.isscalar(v) else np.asarray(v))
            for k, v in (extra or {}).items():
                f.create_dataset(k, data=v if np.isscalar(v) else np.asarray(v))
        return path
    if not path.endswith(".npz"):
        path = path + ".npz"
    arrays = {"ux": ux, "uy": uy, "x": np.asarray(x, dtype=np.float32),
              "y": np.asarray(y, dtype=np.float32), "t": np.asarray(t, dtype=np.float32)}
    for k, v in info.items():
        arrays[f"source_info/{k}"] = np.asarray(v)
    for k, v in (extra or {}).items():
        arrays[k] = np.asarray(v)
    np.savez(path, **arrays)
    return path


def read_wavefields(path: str):
    """(ux, uy, x, y, t, source_info) as numpy arrays from either form."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"wavefield file not found: {path}")
    if _is_hdf5(path):
        if h5py is None:
            raise ImportError(f"{path} is HDF5 and h5py is not installed; convert it to .npz "
                              "with save_wavefields on a machine that has h5py")
        with h5py.File(path, "r") as f:
            out = [f[k][:] for k in ("ux", "uy", "x", "y", "t")]
            info = {k: f["source_info"][k][()] for k in f["source_info"].keys()} \
                if "source_info" in f else {}
        return (*out, info)
    with np.load(path, allow_pickle=False) as z:
        out = [z[k] for k in ("ux", "uy", "x", "y", "t")]
        info = {}
        for k in z.files:
            if k.startswith("source_info/"):
                v = z[k]
                info[k.split("/", 1)[1]] = v[()] if v.ndim == 0 else v
    return (*out, info)


def add_noise_snr(signal: torch.Tensor, snr_db: float, generator: torch.Generator | None = None):
    """Gaussian noise at a target SNR over the whole tensor: noise power =
    mean(signal^2) / 10^(snr_db/10) (Parameter_inversion/Inversion_adam.py:108-129).
    Returns (noisy, noise)."""
    power = torch.mean(signal ** 2)
    noise_power = power / (10.0 ** (snr_db / 10.0))
    noise = torch.randn(signal.shape, generator=generator, device=signal.device,
                        dtype=signal.dtype) * torch.sqrt(noise_power)
    return signal + noise, noise


def load_reference_data(path: str, add_noise: bool = False, snr_db: float = 20.0,
                        device=None, generator: torch.Generator | None = None):
    """The reference loader's contract: (ux, uy, metadata), fields (1, nt_ds,
    nx, ny) float32 on `device` (default: the current CUDA device when there
    is one), copied from pinned host memory; metadata keys x_original,
    y_original, t_primary, source_info, primary_stride, noise_added (+ snr_db,
    noise_ux, noise_uy with noise)."""
    ux, uy, x, y, t, info = read_wavefields(path)
    if device is None:
        device = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
    ux_t = to_device(ux[None], device)
    uy_t = to_device(uy[None], device)
    meta = {"x_original": x, "y_original": y, "t_primary": t, "source_info": info,
            "primary_stride": primary_stride(path)}
    if add_noise:
        ux_t, nx_ = add_noise_snr(ux_t, snr_db, generator)
        uy_t, ny_ = add_noise_snr(uy_t, snr_db, generator)
        meta.update(noise_added=True, snr_db=snr_db, noise_ux=nx_.cpu().numpy(),
                    noise_uy=ny_.cpu().numpy())
    else:
        meta["noise_added"] = False
    return ux_t, uy_t, meta


def to_device(a, device) -> torch.Tensor:
    """float32 host array -> device tensor through pinned memory (asynchronous
    copy on the current stream when the device is a GPU)."""
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))
    dev = torch.device(device)
    if dev.type != "cuda":
        return t.clone()
    return t.pin_memory().to(dev, non_blocking=True)


def traces_from_history(ux_hist: torch.Tensor, uy_hist: torch.Tensor, rec_idx: torch.Tensor):
    """Receiver traces (S, nt_out, R) from dense histories (S, nt_out, nx, ny)
    at flat cells rec_idx (S, R) (i*ny + j): the values the RECORD_RECEIVERS
    mode records for the same problem."""
    S, T = ux_hist.shape[:2]
    idx = rec_idx.long().to(ux_hist.device)[:, None, :].expand(S, T, rec_idx.shape[1])
    return (ux_hist.reshape(S, T, -1).gather(2, idx), uy_hist.reshape(S, T, -1).gather(2, idx))


def save_traces(path: str, tr_x, tr_y, rec_idx, stride: int, dt: float) -> str:
    """Receiver traces with their cells and time axis (frame k = step k*stride+1)."""
    if not path.endswith(".npz"):
        path = path + ".npz"
    np.savez(path, tr_x=np.asarray(tr_x, np.float32), tr_y=np.asarray(tr_y, np.float32),
             rec_idx=np.asarray(rec_idx, np.int32), stride=np.int32(stride), dt=np.float64(dt))
    return path


def load_traces(path: str, device=None):
    """(tr_x, tr_y, rec_idx, stride, dt) with the traces on `device`."""
    with np.load(path, allow_pickle=False) as z:
        tr_x, tr_y, rec = z["tr_x"], z["tr_y"], z["rec_idx"]
        stride, dt = int(z["stride"]), float(z["dt"])
    if device is None:
        device = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
    return to_device(tr_x, device), to_device(tr_y, device), \
        torch.as_tensor(rec, dtype=torch.int32, device=device), stride, dt
