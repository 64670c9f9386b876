"""Benchmark configurations and the material algebra they need (numpy only).

This module imports nothing from the package and nothing that loads the
CUDA library, so the benchmark's reference arm can load it by file path and
build the same workloads, initial guesses and scales as the library's own
arm without mapping libernn_gb300.so into its process.

Workloads (synthetic inputs; no dataset is involved):
  plate128   128x128, 1000 steps, orthotropic, 1 source, 32 top-edge receivers
  rot256     256x256, 2000 steps, orthotropic rotated 30 deg, 1 source,
             64 top-edge receivers, checkpoint every 100 steps
  shots1024  1024x1024, 4000 steps, rotated 30 deg, 16 top-edge sources,
             256 receivers per shot
  damage512  512x512, 3000 steps, C = (1 - D) C0, 8 top sources, 128
             receivers on the top and bottom edges
  fields301  the reference's damage loop on its generator's grid (six
             per-cell constant fields)
  multi64    64 independent inversions, side drawn from {128, 192, ..., 768},
             5.2 x side steps, C0 scaled by U(0.8, 1.2) per constant and
             rotated by U(0, 90) degrees, 1 source and 32 receivers each
dx = dz = 0.1 mm, dt = 5 ns, rho = 1560 kg/m^3, 5-cycle Hann 1 MHz tone-burst
vertical force (Gaussian point load of the reference's source model, a = 5e6
m^-2) on the top edge (y = ny - 1).

Constants are ordered (C11, C22, C12, C16, C26, C66) in the reference's x-y
naming; the x-z names of the configurations map one to one (C11 -> C11,
C33 -> C22, C13 -> C12, C15 -> C16, C35 -> C26, C55 -> C66).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

H, DT, RHO = 1e-4, 5e-9, 1560.0

# Voigt index of the symmetric pair (a, b) in 2D: xx -> 0 (1), yy -> 1 (2), xy -> 2 (6)
_V = {(0, 0): 0, (1, 1): 1, (0, 1): 2, (1, 0): 2}


def voigt_matrix(c6):
    """3x3 Voigt matrix [[C11, C12, C16], [C12, C22, C26], [C16, C26, C66]]."""
    C11, C22, C12, C16, C26, C66 = (float(v) for v in c6)
    return np.array([[C11, C12, C16], [C12, C22, C26], [C16, C26, C66]])


def from_voigt(M):
    return np.array([M[0, 0], M[1, 1], M[0, 1], M[0, 2], M[1, 2], M[2, 2]])


def rotate(c6, theta_deg):
    """Constants of the material rotated by theta in the plane (tensor rotation
    C'_ijkl = R_ia R_jb R_kc R_ld C_abcd)."""
    M = voigt_matrix(c6)
    C = np.zeros((2, 2, 2, 2))
    for i in range(2):
        for j in range(2):
            for k in range(2):
                for l in range(2):
                    C[i, j, k, l] = M[_V[(i, j)], _V[(k, l)]]
    t = np.deg2rad(theta_deg)
    R = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
    Cr = np.einsum("ia,jb,kc,ld,abcd->ijkl", R, R, R, R, C)
    Mr = np.zeros((3, 3))
    for (i, j), p in _V.items():
        for (k, l), q in _V.items():
            Mr[p, q] = Cr[i, j, k, l]
    return from_voigt(Mr)


def orthotropic_xz(C11, C33, C13, C55, C15=0.0, C35=0.0):
    """x-z constants of the benchmark configurations, returned in (C11, C22, C12, C16, C26, C66) order."""
    return np.array([C11, C33, C13, C15, C35, C55], dtype=np.float64)


def stability_number(c6, rho, h, dt, n=128):
    """Stability of the leapfrog scheme for scalar constants: max over the
    Fourier modes exp(i(tx i + ty j)), tx, ty in [0, pi] on an (n+1)^2 grid
    and both signs of the mixed term, of the largest eigenvalue of the
    symbol of -(dt^2 / (rho h^2)) h^2 A divided by 4 (stable for values <= 1),
    and whether the symbol is indefinite somewhere (a stiffness that is not
    positive-definite).  The same test as the library's ernn_check_stability."""
    C11, C22, C12, C16, C26, C66 = (float(v) for v in c6)
    q = dt * dt / (rho * h * h)
    t = np.pi * np.arange(n + 1) / n
    tx, ty = np.meshgrid(t, t, indexing="ij")
    a = 4.0 * np.sin(tx / 2) * np.sin(tx / 2)
    b = 4.0 * np.sin(ty / 2) * np.sin(ty / 2)
    worst, indefinite = 0.0, False
    for sgn in (-1.0, 1.0):
        d = sgn * np.sin(tx) * np.sin(ty)
        mxx = C11 * a + C66 * b + 2 * C16 * d
        myy = C66 * a + C22 * b + 2 * C26 * d
        mxy = C16 * a + C26 * b + (C12 + C66) * d
        tr, det = mxx + myy, mxx * myy - mxy * mxy
        disc = np.sqrt(np.maximum(tr * tr / 4 - det, 0.0))
        lmax, lmin = tr / 2 + disc, tr / 2 - disc
        indefinite = indefinite or bool(np.any(lmin < -1e-9 * np.abs(lmax)))
        worst = max(worst, float(np.max(q * lmax / 4.0)))
    return worst, indefinite


def top_edge_positions(n, nx, margin=0):
    """n cell indices along x evenly spaced on [margin, nx-1-margin]."""
    if n == 1:
        return [nx // 2]
    return [int(round(v)) for v in np.linspace(margin, nx - 1 - margin, n)]


C_ORTHO = orthotropic_xz(130e9, 12e9, 6e9, 5.5e9)  # C11, C33, C13, C55 (GPa), C15 = C35 = 0


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nt: int
    C_true: np.ndarray
    src_cells: list            # [(i, j)] per shot
    rec_cells: list            # [(i, j)] shared by every shot
    ckpt_k: int | None = None
    stride: int = 1
    f0: float = 1e6
    amplitude: float = 1e10
    gaussian_param: float = 5e6
    D_true: np.ndarray | None = None
    extra: dict = field(default_factory=dict)
    path: int = 0              # kernel path of the library (PATH_AUTO by default)

    @property
    def nshots(self):
        return len(self.src_cells)

    @property
    def cell_steps(self):
        return self.nshots * self.nx * self.ny * self.nt


def _top(n, nx, ny, margin=2):
    return [(i, ny - 1) for i in top_edge_positions(n, nx, margin)]


def plate128():
    return Workload("plate128", 128, 128, 1000, C_ORTHO.copy(), [(64, 127)], _top(32, 128, 128))


def rot256(ckpt_k=100):
    C = rotate(C_ORTHO, 30.0)
    return Workload("rot256", 256, 256, 2000, C, [(128, 255)], _top(64, 256, 256), ckpt_k=ckpt_k)


def shots1024(ckpt_k=None, nt=4000):
    C = rotate(C_ORTHO, 30.0)
    src = _top(16, 1024, 1024, margin=32)
    return Workload("shots1024", 1024, 1024, nt, C, src, _top(256, 1024, 1024), ckpt_k=ckpt_k)


def damage_map(nx, ny, seed=0, n=3):
    """True degradation D in [0, 0.6]: three Gaussian ellipses with seeded
    centres, axes sigma in [1, 4] mm and peak depths in [0.2, 0.6] of the depth."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * H
    y = np.arange(ny) * H
    X, Y = np.meshgrid(x, y, indexing="ij")
    D = np.zeros((nx, ny))
    for _ in range(n):
        cx = rng.uniform(0.2, 0.8) * x[-1]
        depth = rng.uniform(0.2, 0.6) * y[-1]
        cy = y[-1] - depth                      # depth measured from the top edge
        sx, sy = rng.uniform(1e-3, 4e-3, size=2)
        peak = rng.uniform(0.3, 0.6)
        D = np.maximum(D, peak * np.exp(-0.5 * (((X - cx) / sx) ** 2 + ((Y - cy) / sy) ** 2)))
    return np.clip(D, 0.0, 0.6)


def damage512(ckpt_k=None, nt=3000):
    rec = _top(64, 512, 512) + [(i, 0) for i in top_edge_positions(64, 512, 2)]
    return Workload("damage512", 512, 512, nt, C_ORTHO.copy(), _top(8, 512, 512, margin=16), rec,
                    ckpt_k=ckpt_k, D_true=damage_map(512, 512))


# The damage loop of the reference (Damage_inversion/Inversion_adam.py:815-1000)
# on its generator's grid: 301^2 nodes over 0.4 m, 4001 steps over 120 us,
# history every 5 steps, loss on every 2nd frame with TV 1e-21, Adam lr 0.02
# on the six log-constant fields; run through the drop-in
# SpatiallyVaryingAnisotropicSimulator (six-field mode).
FIELDS301 = dict(nx=301, L=0.4, nt=4001, total_time=120e-6, stride=5, ts=2, lambda_tv=1e-21,
                 lr=0.02, C0=(130.74e9, 11.50e9, 10.49e9, 30.67e9, 3.75e9, 14.77e9), rho=1610.0,
                 f0=100e3, t0=10e-6, amplitude=1e10, gaussian_param=5e6)


def fields301():
    c = FIELDS301
    return Workload("fields301", c["nx"], c["nx"], c["nt"], np.asarray(c["C0"]), [(c["nx"] // 2, c["nx"] // 2)],
                    [], stride=c["stride"], f0=c["f0"], amplitude=c["amplitude"],
                    gaussian_param=c["gaussian_param"], extra={"fields": True, "restart": True})


WORKLOADS = {"plate128": plate128, "rot256": rot256, "shots1024": shots1024,
             "damage512": damage512, "fields301": fields301}


def initial_guess(w: Workload, seed=0, spread=0.2, max_draws=100):
    """Each constant perturbed uniformly by +-spread (seeded).  Perturbing the
    six constants of a rotated material independently can leave a stiffness
    that is not positive-definite (the time loop then diverges): such draws
    are rejected, as are draws the leapfrog step cannot carry, and redrawn
    from the same seeded stream."""
    rng = np.random.default_rng(seed)
    for _ in range(max_draws):
        C = w.C_true * rng.uniform(1 - spread, 1 + spread, size=6)
        number, indefinite = stability_number(C, RHO, H, DT)
        if number <= 1.0 and not indefinite:
            return C
    raise ValueError("no stable initial guess found")


def scales(C_true):
    C = np.abs(np.asarray(C_true, np.float64))
    return np.where(C > 0, C, 0.05 * C.max())


def multi_instances(n=64, seed=0, sides=None):
    """Workloads of the uneven multi-inversion configuration (seeded)."""
    rng = np.random.default_rng(seed)
    if sides is None:
        sides = rng.choice(np.arange(128, 769, 64), size=n)
    out = []
    for i, side in enumerate(sides):
        side = int(side)
        C0 = C_ORTHO * rng.uniform(0.8, 1.2, size=6)
        C = rotate(C0, float(rng.uniform(0.0, 90.0)))
        nt = int(round(5.2 * side))
        out.append(Workload(f"inst{i}_{side}", side, side, nt, C, [(side // 2, side - 1)],
                            _top(32, side, side)))
    return out
