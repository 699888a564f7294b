"""Synthetic MT workloads the solver is measured and tested on.

Pure numpy: nothing here loads the native library, so the CPU reference arm
of the benchmark and the checkers can build the same inputs (conductivity,
stations, frequencies, observed data) as the GPU arm without it.

The model and survey rules follow the reference's drivers:
  domain and station refinement radius   examples/real_inversion_octree.cpp:298-379
  air conductivity 1e-8 S/m              examples/halfspace_1d_test.cpp:89-92
  5 % noise on Zxy / Zyx, err = 0.05|Z|  examples/commemi_3d1a/generate_data.cpp:230-251
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

MU0 = 4.0e-7 * math.pi
SIGMA_AIR = 1e-8
SIGMA_BG = 0.01          # primary-field halfspace (forward_solver_fv.cpp:34,121)


def skin_depth(freq, sigma):
    return math.sqrt(2.0 / (2.0 * math.pi * freq * MU0 * sigma))


def station_grid(n, spacing):
    c = (np.arange(n) - (n - 1) / 2.0) * spacing
    xx, yy = np.meshgrid(c, c, indexing="xy")
    return np.stack([xx.ravel(), yy.ravel(), np.zeros(n * n)], axis=1)


def driver_domain(stations, freqs, half_width, sigma0, max_level, radius=None):
    """Domain [-hw, hw]^2 x [-3 delta, delta] (delta = skin depth at the lowest
    frequency in sigma0) and the station refinement radius of the driver."""
    fmin = float(np.min(freqs))
    dmax = skin_depth(fmin, sigma0)
    domain = (-half_width, half_width, -half_width, half_width, -3.0 * dmax, dmax)
    if radius is None:
        st = np.asarray(stations)
        d = np.sqrt(((st[:, None, :2] - st[None, :, :2]) ** 2).sum(-1))
        d = d[d > 100]
        min_sp = float(d.min()) if d.size else 1000.0
        finest = 2.0 * half_width / 2.0 ** max_level
        radius = max(3.0 * finest, min_sp, 2000.0)
        radius = min(radius, dmax * 0.1)
    return domain, radius


def layered_block_sigma(x, y, z):
    """10/100/1000 ohm-m layers (interfaces -1 km, -10 km) with a 0.5 ohm-m block
    x in [-0.5, 0.5] km, y in [-1, 1] km, z in [-2.25, -0.25] km."""
    s = np.where(z > -1000.0, 0.1, np.where(z > -10000.0, 0.01, 0.001))
    blk = (np.abs(x) <= 500.0) & (np.abs(y) <= 1000.0) & (z <= -250.0) & (z >= -2250.0)
    return np.where(blk, 2.0, s)


def halfspace_sigma(rho):
    return lambda x, y, z: np.full_like(np.asarray(z, dtype=np.float64), 1.0 / rho)


def cell_sigma(cell_type, cx, cy, cz, earth_fn):
    """Air cells 1e-8 S/m, earth cells earth_fn(cx, cy, cz)."""
    s = np.where(np.asarray(cell_type) == 0, earth_fn(cx, cy, cz), SIGMA_AIR)
    return np.ascontiguousarray(s, dtype=np.float64)


def random_layered_blocks(seed, n_blocks=None):
    """A seeded layered earth with 1-3 conductive/resistive blocks (block
    resistivity log-uniform in 0.1-1000 ohm-m, sizes 0.5-5 km), as earth_fn."""
    rng = np.random.default_rng(seed)
    nl = int(rng.integers(2, 4))
    tops = np.sort(-rng.uniform(300.0, 15000.0, nl - 1))[::-1]     # interfaces, descending
    rho_l = 10.0 ** rng.uniform(0.0, 3.0, nl)
    nb = int(rng.integers(1, 4)) if n_blocks is None else int(n_blocks)
    blocks = []
    for _ in range(nb):
        size = rng.uniform(500.0, 5000.0, 3)
        cx, cy = rng.uniform(-3000.0, 3000.0, 2)
        ztop = -rng.uniform(100.0, 3000.0)
        blocks.append((cx - size[0] / 2, cx + size[0] / 2, cy - size[1] / 2, cy + size[1] / 2,
                       ztop - size[2], ztop, 10.0 ** rng.uniform(-1.0, 3.0)))

    def earth(x, y, z):
        x = np.asarray(x); y = np.asarray(y); z = np.asarray(z)
        rho = np.full(z.shape, rho_l[-1])
        for i in range(nl - 2, -1, -1):          # deepest interface first
            rho = np.where(z > tops[i], rho_l[i], rho)
        for (x0, x1, y0, y1, z0, z1, r) in blocks:
            inside = (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1) & (z >= z0) & (z <= z1)
            rho = np.where(inside, r, rho)
        return 1.0 / rho
    return earth


def halfspace_data(stations, freqs, seed=42, rho=100.0):
    """Observed impedances of the 1-D halfspace with seeded 5 % complex noise
    on every component, errors 5 % of |Z| on Zxy and Zyx (Zxx, Zyy carry no
    weight, as unset components in the reference)."""
    ns, nf = len(stations), len(freqs)
    rng = np.random.default_rng(seed)
    om = 2 * math.pi * np.asarray(freqs, np.float64)
    z1 = np.sqrt(1j * om * MU0 / (1.0 / rho))
    obs = np.zeros((ns, nf, 4), np.complex128)
    obs[:, :, 1] = z1[None, :]
    obs[:, :, 2] = -z1[None, :]
    err = np.zeros((ns, nf, 4))
    err[:, :, 1:3] = 0.05 * np.abs(z1)[None, :, None]
    noise = rng.normal(size=(ns, nf, 4)) + 1j * rng.normal(size=(ns, nf, 4))
    obs = obs + 0.05 * np.abs(obs) * noise / math.sqrt(2)
    return obs, err


def noisy_data(Z, seed=42, level=0.05):
    """5 % noise as the reference's synthetic-data generator: mt19937-style
    seeded Gaussian noise scaled by 0.05|Z| on Zxy and Zyx, err = 0.05|Z|
    (Z given as [ns, nf, 4])."""
    rng = np.random.default_rng(seed)
    obs = np.array(Z, dtype=np.complex128, copy=True)
    err = np.zeros(obs.shape)
    for k in (1, 2):
        a = np.abs(obs[:, :, k])
        err[:, :, k] = level * a
        obs[:, :, k] += level * a * (rng.normal(size=a.shape) + 1j * rng.normal(size=a.shape)) / math.sqrt(2)
    return obs, err


@dataclass(frozen=True)
class SurveySpec:
    """Mesh and survey parameters of a named configuration."""
    name: str
    min_level: int
    max_level: int
    n_side: int
    spacing: float
    freqs: tuple
    half_width: float = 50000.0


C1 = SurveySpec("C1 halfspace", 3, 5, 5, 2000.0, (1.0,))
C2 = SurveySpec("C2 layered+block", 6, 7, 11, 1000.0, tuple(np.logspace(-2, 2, 8).tolist()))
C5 = SurveySpec("C5 layered+block at scale", 6, 8, 20, 1000.0, tuple(np.logspace(-3, 3, 24).tolist()))
# one mesh per frequency (skin-depth refinement at that frequency only),
# log10 sigma of earth cells perturbed by N(0, 0.3^2)
C3 = SurveySpec("C3 per-frequency meshes", 6, 7, 11, 1000.0, tuple(np.logspace(-3, 3, 16).tolist()))
C3_NOISE_STD = 0.3


def station_sources(ns, rng, level=0.05):
    """Adjoint sources of the per-station Jacobian rows: source s has
    w^2 conj(r) at station s only, r a synthetic 5 % residual of a unit-scale
    response on the off-diagonal impedances (Zxy, Zyx) with unit weight.
    Returns wr [ns][ns][4] complex."""
    wr = np.zeros((ns, ns, 4), np.complex128)
    for k in (1, 2):
        r = level * (rng.normal(size=ns) + 1j * rng.normal(size=ns)) / math.sqrt(2)
        wr[np.arange(ns), np.arange(ns), k] = np.conj(r)
    return wr
