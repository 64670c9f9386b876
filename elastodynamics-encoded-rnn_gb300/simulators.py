"""Drop-in nn.Modules with the reference's call surface, running on the CUDA path.

CFRPWaveSimulatorRicker mirrors Parameter_inversion/Inversion_adam.py:132-307
and SpatiallyVaryingAnisotropicSimulator mirrors
Damage_inversion/Inversion_adam.py:198-393: same constructor arguments, the
same parameters (log_C11 ... log_C66), buffers (rho, gaussian_dist,
source_signal), get_material_params() and forward(save_all_steps) ->
(ux_fields, uy_fields) of shape (1, nt_out, nx, ny).  Only forward's body
differs: the time loop and its gradient run in libernn_gb300.so through
ErnnPropagate, so the reference's invert() loops (zero_grad, forward,
compute_loss, backward, Adam.step) work unchanged.

DegradationSimulator and ShotGatherSimulator are the receiver-trace and
stiffness-degradation forms of the benchmark configurations.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn as nn

from . import sources as S
from .misfit import series_misfit
from .propagate import Geometry, propagate


def _default_device():
    return torch.device("cuda:0" if torch.cuda.is_available() else "cpu")


class _GeometryCache:
    """Source box cropped from the dense load, rebuilt when the buffer changes."""

    def __init__(self):
        self.key = None
        self.box = None

    def get(self, dense: torch.Tensor):
        key = (dense.data_ptr(), dense._version, dense.device, tuple(dense.shape))
        if key != self.key:
            self.box = S.crop_box(dense)
            self.key = key
        return self.box


class CFRPWaveSimulatorRicker(nn.Module):
    """Anisotropic elastic simulator with six scalar constants and a Ricker source
    (Parameter_inversion/Inversion_adam.py:132-307)."""

    def __init__(self, domain_shape, h, dt, nt, primary_time_stride,
                 source_component='y',
                 source_f0=100e3,
                 source_t0=6e-6,
                 source_amplitude=1.0,
                 C11_init=100e9, C22_init=10e9, C12_init=8e9,
                 C16_init=25e9, C26_init=3e9, C66_init=12e9,
                 rho_known=1600.0, gaussian_param=5e6,
                 source_position=(0.0, 0.0),
                 ckpt_k=None):
        super().__init__()
        self.domain_shape = tuple(domain_shape)
        self.h = h
        self.dt = dt
        self.nt = nt
        self.primary_time_stride = primary_time_stride
        self.source_component = source_component
        self.source_f0 = source_f0
        self.source_t0 = source_t0
        self.source_amplitude = source_amplitude
        self.gaussian_param = gaussian_param
        self.source_position = source_position
        # checkpoint interval of the hand adjoint (None: keep every state)
        self.ckpt_k = ckpt_k

        f32 = torch.float32
        self.log_C11 = nn.Parameter(torch.log(torch.tensor(C11_init, dtype=f32)))
        self.log_C22 = nn.Parameter(torch.log(torch.tensor(C22_init, dtype=f32)))
        self.log_C12 = nn.Parameter(torch.log(torch.tensor(C12_init, dtype=f32)))
        self.log_C16 = nn.Parameter(torch.log(torch.tensor(C16_init, dtype=f32)))
        self.log_C26 = nn.Parameter(torch.log(torch.tensor(C26_init, dtype=f32)))
        self.log_C66 = nn.Parameter(torch.log(torch.tensor(C66_init, dtype=f32)))
        self.register_buffer('rho', torch.tensor(rho_known, dtype=f32))
        self.rho_known = rho_known
        self.C11_bounds = (1e9, 10000e9)
        self.C22_bounds = (1e9, 10000e9)
        self.C12_bounds = (1e9, 10000e9)
        self.C16_bounds = (1e9, 10000e9)
        self.C26_bounds = (1e9, 10000e9)
        self.C66_bounds = (1e9, 10000e9)

        nx, ny = self.domain_shape
        X, Y = S.centered_grid(nx, ny, h, device=_default_device())
        x0, y0 = source_position
        self.gaussian_distribution = S.gaussian_point_load(X, Y, x0, y0, gaussian_param)
        self.register_buffer('gaussian_dist', self.gaussian_distribution)
        self._generate_ricker_source_signal()
        self._box = _GeometryCache()

    def _generate_ricker_source_signal(self):
        t = np.arange(self.nt) * self.dt
        signal = S.ricker_wavelet(t, self.source_f0, self.source_t0, self.source_amplitude)
        self.register_buffer('source_signal', torch.tensor(signal, dtype=torch.float32).unsqueeze(0))

    def get_material_params(self):
        """Clamped exp(log C) (Parameter_inversion/Inversion_adam.py:223-232)."""
        C11 = torch.clamp(torch.exp(self.log_C11), *self.C11_bounds)
        C22 = torch.clamp(torch.exp(self.log_C22), *self.C22_bounds)
        C12 = torch.clamp(torch.exp(self.log_C12), *self.C12_bounds)
        C16 = torch.clamp(torch.exp(self.log_C16), *self.C16_bounds)
        C26 = torch.clamp(torch.exp(self.log_C26), *self.C26_bounds)
        C66 = torch.clamp(torch.exp(self.log_C66), *self.C66_bounds)
        return C11, C22, C12, C16, C26, C66, self.rho

    def get_current_params_values(self):
        C11, C22, C12, C16, C26, C66, rho = self.get_material_params()
        return (C11.item() / 1e9, C22.item() / 1e9, C12.item() / 1e9,
                C16.item() / 1e9, C26.item() / 1e9, C66.item() / 1e9, rho.item())

    def _load_map(self):
        return self.gaussian_dist.unsqueeze(0)

    def geometry(self, save_all_steps=False) -> Geometry:
        nx, ny = self.domain_shape
        smap, origin = self._box.get(self._load_map())
        return Geometry(nx=nx, ny=ny, nt=self.nt, h=self.h, dt=self.dt,
                        src_signal=self.source_signal.contiguous(), src_map=smap,
                        src_origin=origin,
                        stride=1 if save_all_steps else self.primary_time_stride,
                        src_comp=0 if self.source_component == 'x' else 1,
                        ckpt_k=self.ckpt_k)

    def forward(self, save_all_steps=False):
        """Returns ux_fields, uy_fields of shape (1, nt_output, nx, ny)."""
        C11, C22, C12, C16, C26, C66, rho = self.get_material_params()
        C = torch.stack([C11, C22, C12, C16, C26, C66])
        return propagate(C, rho, self.geometry(save_all_steps))


class SpatiallyVaryingAnisotropicSimulator(nn.Module):
    """Six per-cell constant fields (Damage_inversion/Inversion_adam.py:198-393).

    The reference's spatially varying operator adds the force transposed
    (Damage_inversion/Inversion_adam.py:169-174), which only works on square
    grids; this module passes the transposed load to reproduce it and raises
    the same kind of error for non-square grids."""

    def __init__(self, domain_shape, h, dt, nt, primary_time_stride,
                 source_component='y',
                 source_f0=100e3,
                 source_t0=10e-6,
                 source_amplitude=1e10,
                 total_time=60e-6,
                 C11_init=130.74e9,
                 C22_init=11.50e9,
                 C12_init=10.49e9,
                 C16_init=30.67e9,
                 C26_init=3.75e9,
                 C66_init=14.77e9,
                 rho_known=1610.0,
                 gaussian_param=5e6,
                 use_log_params=True,
                 ckpt_k=None):
        super().__init__()
        self.domain_shape = tuple(domain_shape)
        self.h = h
        self.dt = dt
        self.nt = nt
        self.total_time = total_time
        self.primary_time_stride = primary_time_stride
        self.use_log_params = use_log_params
        self.source_component = source_component
        self.source_f0 = source_f0
        self.source_t0 = source_t0
        self.source_amplitude = source_amplitude
        self.gaussian_param = gaussian_param
        self.ckpt_k = ckpt_k
        nx, ny = self.domain_shape
        f32 = torch.float32
        if use_log_params:
            self.log_C11 = nn.Parameter(torch.full((1, nx, ny), np.log(C11_init), dtype=f32))
            self.log_C22 = nn.Parameter(torch.full((1, nx, ny), np.log(C22_init), dtype=f32))
            self.log_C12 = nn.Parameter(torch.full((1, nx, ny), np.log(C12_init), dtype=f32))
            self.log_C16 = nn.Parameter(torch.full((1, nx, ny), np.log(abs(C16_init) + 1e6), dtype=f32))
            self.log_C26 = nn.Parameter(torch.full((1, nx, ny), np.log(abs(C26_init) + 1e6), dtype=f32))
            self.log_C66 = nn.Parameter(torch.full((1, nx, ny), np.log(C66_init), dtype=f32))
        else:
            self.C11 = nn.Parameter(torch.full((1, nx, ny), C11_init, dtype=f32))
            self.C22 = nn.Parameter(torch.full((1, nx, ny), C22_init, dtype=f32))
            self.C12 = nn.Parameter(torch.full((1, nx, ny), C12_init, dtype=f32))
            self.C16 = nn.Parameter(torch.full((1, nx, ny), C16_init, dtype=f32))
            self.C26 = nn.Parameter(torch.full((1, nx, ny), C26_init, dtype=f32))
            self.C66 = nn.Parameter(torch.full((1, nx, ny), C66_init, dtype=f32))
        self.register_buffer('rho', torch.tensor(rho_known, dtype=f32))
        self.rho_known = rho_known
        self.C11_bounds = (50e9, 250e9)
        self.C22_bounds = (5e9, 50e9)
        self.C12_bounds = (5e9, 50e9)
        self.C16_bounds = (0, 60e9)
        self.C26_bounds = (0, 20e9)
        self.C66_bounds = (5e9, 30e9)
        X, Y = S.centered_grid(nx, ny, h, device=_default_device())
        self.gaussian_distribution = S.gaussian_point_load(X, Y, 0.0, 0.0, gaussian_param)
        self.register_buffer('gaussian_dist', self.gaussian_distribution)
        self._generate_ricker_source_signal()
        self._box = _GeometryCache()

    def _generate_ricker_source_signal(self):
        t = np.arange(self.nt) * self.dt
        signal = S.ricker_wavelet(t, self.source_f0, self.source_t0, self.source_amplitude)
        self.register_buffer('source_signal', torch.tensor(signal, dtype=torch.float32).unsqueeze(0))

    def get_material_params(self):
        """Clamped per-cell constants (Damage_inversion/Inversion_adam.py:304-322)."""
        if self.use_log_params:
            C11 = torch.clamp(torch.exp(self.log_C11), *self.C11_bounds)
            C22 = torch.clamp(torch.exp(self.log_C22), *self.C22_bounds)
            C12 = torch.clamp(torch.exp(self.log_C12), *self.C12_bounds)
            C16 = torch.clamp(torch.exp(self.log_C16), *self.C16_bounds)
            C26 = torch.clamp(torch.exp(self.log_C26), *self.C26_bounds)
            C66 = torch.clamp(torch.exp(self.log_C66), *self.C66_bounds)
        else:
            C11 = torch.clamp(self.C11, *self.C11_bounds)
            C22 = torch.clamp(self.C22, *self.C22_bounds)
            C12 = torch.clamp(self.C12, *self.C12_bounds)
            C16 = torch.clamp(self.C16, *self.C16_bounds)
            C26 = torch.clamp(self.C26, *self.C26_bounds)
            C66 = torch.clamp(self.C66, *self.C66_bounds)
        return C11, C22, C12, C16, C26, C66, self.rho

    def get_mean_params(self):
        C11, C22, C12, C16, C26, C66, rho = self.get_material_params()
        return (C11.mean().item() / 1e9, C22.mean().item() / 1e9, C12.mean().item() / 1e9,
                C16.mean().item() / 1e9, C26.mean().item() / 1e9, C66.mean().item() / 1e9,
                rho.item())

    def geometry(self, save_all_steps=False) -> Geometry:
        nx, ny = self.domain_shape
        if nx != ny:
            raise RuntimeError(
                f"The size of tensor a ({ny}) must match the size of tensor b ({nx}): the "
                "spatially varying operator adds the force transposed and needs a square grid")
        smap, origin = self._box.get(self.gaussian_dist.t().unsqueeze(0))
        return Geometry(nx=nx, ny=ny, nt=self.nt, h=self.h, dt=self.dt,
                        src_signal=self.source_signal.contiguous(), src_map=smap,
                        src_origin=origin,
                        stride=1 if save_all_steps else self.primary_time_stride,
                        src_comp=0 if self.source_component == 'x' else 1,
                        ckpt_k=self.ckpt_k)

    def forward(self, save_all_steps=False):
        C11, C22, C12, C16, C26, C66, rho = self.get_material_params()
        C = torch.cat([C11, C22, C12, C16, C26, C66], dim=0)
        return propagate(C, rho, self.geometry(save_all_steps))


class ShotGatherSimulator(nn.Module):
    """Scalar constants, many shots, receiver traces (the benchmark configurations).

    constants: (6,) tensor of physical constants or a callable returning one
    (e.g. a normalised parameterisation).  Returns (ux_traces, uy_traces) of
    shape (S, nt_out, R)."""

    def __init__(self, geometry: Geometry, rho: float):
        super().__init__()
        self.geom = geometry
        self.register_buffer('rho', torch.tensor(rho, dtype=torch.float32))

    def forward(self, C):
        return propagate(C, self.rho, self.geom)


class DegradationSimulator(nn.Module):
    """C_ij(x) = (1 - D(x)) C0_ij with a learnable degradation map D (the
    stiffness-degradation configuration).  Returns receiver traces or the
    dense history, depending on the geometry."""

    def __init__(self, geometry: Geometry, C0, rho: float, D_init=None):
        super().__init__()
        self.geom = geometry
        self.register_buffer('C0', torch.as_tensor(np.asarray(C0, dtype=np.float32)))
        self.register_buffer('rho', torch.tensor(rho, dtype=torch.float32))
        D0 = torch.zeros((geometry.nx, geometry.ny)) if D_init is None else torch.as_tensor(D_init)
        self.D = nn.Parameter(D0.to(torch.float32).clone())

    def forward(self):
        return propagate(self.C0, self.rho, self.geom, D=self.D)


def total_variation_2d(field: torch.Tensor) -> torch.Tensor:
    """Sum of the absolute forward differences of a (batch, nx, ny) field along
    both grid axes (Damage_inversion/Inversion_adam.py:179-195)."""
    return (torch.sum(torch.abs(field[:, 1:, :] - field[:, :-1, :])) +
            torch.sum(torch.abs(field[:, :, 1:] - field[:, :, :-1])))


def damage_loss(sim: SpatiallyVaryingAnisotropicSimulator, pred_ux, pred_uy, target_ux, target_uy,
                secondary_time_stride: int = 1, lambda_tv: float = 0.0):
    """The damage inversion's objective, as its inverter computes it
    (Damage_inversion/Inversion_adam.py:420-422, 441-463): every
    `secondary_time_stride`-th frame of the (1, nt_out, nx, ny) histories,
    5:1 weighted mean squared errors of u_x and u_y, plus lambda_tv times the
    total variation of the six constant fields of `sim`.  Targets are the
    full-rate histories.  The data term is one fused pass of the library
    (FP64 sums, float64 result) whose gradient is the adjoint source.
    Returns (total, data, tv)."""
    data = series_misfit(pred_ux, pred_uy, target_ux, target_uy, 5.0, 1.0, secondary_time_stride)
    tv = 0.0
    if lambda_tv > 0:
        C = sim.get_material_params()[:6]
        tv = lambda_tv * sum(total_variation_2d(c) for c in C)
    return data + tv, data, tv


def parameter_loss(pred_ux, pred_uy, target_ux, target_uy, secondary_time_stride: int = 1,
                   secondary_space_stride: int = 1):
    """The parameter inversion's objective, as its inverter computes it
    (Parameter_inversion/Inversion_adam.py:339-342, 358-391): [:, ::ts, ::ss,
    ::ss] of the (1, nt_out, nx, ny) histories and of the full-rate targets,
    mean squared error of u_x plus that of u_y; one fused pass of the
    library (FP64 sums, float64 result)."""
    return series_misfit(pred_ux, pred_uy, target_ux, target_uy, 1.0, 1.0, secondary_time_stride,
                         secondary_space_stride)
