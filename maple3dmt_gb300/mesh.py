"""Octree meshes and synthetic surveys for the forward solve.

`build_octree` calls the native leaf builder (include/m3d_mesh.h), a p4est
stand-in that follows the refinement rules of the reference's
OctreeMesh::setup (src/octree/octree_mesh.cpp:25-63).  The survey helpers
apply the domain and refinement-radius rules of the reference driver
(examples/real_inversion_octree.cpp:298-379) to the workloads the solver is
measured on.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi, _loader

from .workloads import (MU0, SIGMA_AIR, driver_domain, layered_block_sigma, skin_depth,  # noqa: F401
                        station_grid)


@dataclass
class Leaves:
    """Leaf list of an octree: the mesh input of the solver."""
    domain: tuple
    min_level: int
    max_level: int
    level: np.ndarray      # int32 [nc]
    qxyz: np.ndarray       # int32 [nc, 3] lower corners, root length 2**19
    cx: np.ndarray         # float64 [nc]
    cy: np.ndarray
    cz: np.ndarray
    cell_type: np.ndarray  # int32 [nc] 0 earth, 1 air

    @property
    def n_cells(self) -> int:
        return int(self.level.shape[0])


def build_octree(domain, min_level, max_level, stations, freqs, *, station_refine_radius,
                 station_refine_level=None, sigma_bg=0.01, max_interest_depth=0.0,
                 air_surface_thickness=2000.0, air_mid_thickness=8000.0,
                 air_upper_thickness=20000.0, transition_padding=0.0, regions=(),
                 lib=None) -> Leaves:
    lib = lib or _loader.load()
    st = np.ascontiguousarray(np.asarray(stations, dtype=np.float64).reshape(-1, 3))
    fr = np.ascontiguousarray(np.asarray(freqs, dtype=np.float64).reshape(-1))
    p = _abi.MeshParams()
    for i in range(6):
        p.domain[i] = float(domain[i])
    p.min_level = int(min_level)
    p.max_level = int(max_level)
    p.station_refine_radius = float(station_refine_radius)
    p.station_refine_level = int(max_level if station_refine_level is None else station_refine_level)
    p.sigma_bg = float(sigma_bg)
    p.max_interest_depth = float(max_interest_depth)
    p.air_surface_thickness = float(air_surface_thickness)
    p.air_mid_thickness = float(air_mid_thickness)
    p.air_upper_thickness = float(air_upper_thickness)
    p.transition_padding = float(transition_padding)
    if st.shape[0]:
        p.station_bbox[0] = float(st[:, 0].min()); p.station_bbox[1] = float(st[:, 0].max())
        p.station_bbox[2] = float(st[:, 1].min()); p.station_bbox[3] = float(st[:, 1].max())
    reg = np.ascontiguousarray(np.asarray(regions, dtype=np.float64).reshape(-1, 8))
    p.n_regions = int(reg.shape[0])
    p.regions = reg.ctypes.data_as(_abi.c_double_p) if reg.shape[0] else None
    h = C.c_void_p()
    rc = lib.m3d_octree_build(C.byref(p), st.ctypes.data_as(_abi.c_double_p), int(st.shape[0]),
                              fr.ctypes.data_as(_abi.c_double_p), int(fr.shape[0]), C.byref(h))
    if rc != 0:
        raise RuntimeError(f"m3d_octree_build failed with code {rc}")
    try:
        nc = lib.m3d_octree_num_cells(h)
        level = np.zeros(nc, np.int32)
        q = np.zeros((nc, 3), np.int32)
        cx = np.zeros(nc); cy = np.zeros(nc); cz = np.zeros(nc)
        ty = np.zeros(nc, np.int32)
        ip = lambda a: a.ctypes.data_as(_abi.c_int_p)  # noqa: E731
        dp = lambda a: a.ctypes.data_as(_abi.c_double_p)  # noqa: E731
        rc = lib.m3d_octree_get(h, ip(level), ip(q), dp(cx), dp(cy), dp(cz), ip(ty))
        if rc != 0:
            raise RuntimeError(f"m3d_octree_get failed with code {rc}")
        balanced = lib.m3d_octree_is_balanced(h)
    finally:
        lib.m3d_octree_destroy(h)
    if not balanced:
        raise RuntimeError("octree leaf builder produced an unbalanced tree")
    return Leaves(tuple(float(d) for d in domain), int(min_level), int(max_level),
                  level, q, cx, cy, cz, ty)


@dataclass
class Survey:
    """A synthetic MT survey: mesh, conductivity, stations and frequencies."""
    name: str
    leaves: Leaves
    sigma: np.ndarray          # [nc] S/m
    sigma_bg: float
    stations: np.ndarray       # [ns, 3]
    freqs: np.ndarray          # [nf] Hz
    meta: dict = field(default_factory=dict)


def assign_sigma(leaves: Leaves, earth_fn) -> np.ndarray:
    """Air cells get 1e-8 S/m (examples/halfspace_1d_test.cpp:89-92); earth cells earth_fn."""
    s = np.where(leaves.cell_type == 0, earth_fn(leaves.cx, leaves.cy, leaves.cz), SIGMA_AIR)
    return np.ascontiguousarray(s, dtype=np.float64)


def halfspace_survey(*, half_width=50000.0, min_level=3, max_level=5, n_side=5, spacing=2000.0,
                     freqs=(1.0,), rho=100.0, lib=None) -> Survey:
    """Uniform 100 ohm-m halfspace under 1e-8 S/m air, 5x5 stations at 2 km, 1 Hz."""
    st = station_grid(n_side, spacing)
    fr = np.asarray(freqs, dtype=np.float64)
    sigma0 = 0.01
    domain, radius = driver_domain(st, fr, half_width, sigma0, max_level)
    lv = build_octree(domain, min_level, max_level, st, fr, station_refine_radius=radius,
                      sigma_bg=sigma0, lib=lib)
    sig = assign_sigma(lv, lambda x, y, z: np.full_like(z, 1.0 / rho))
    return Survey("halfspace", lv, sig, sigma0, st, fr,
                  {"station_refine_radius": radius, "rho": rho})


def layered_block_survey(*, half_width=50000.0, min_level=5, max_level=7, n_side=11,
                         spacing=1000.0, freqs=None, radius=None, noise_std=0.0, seed=0,
                         lib=None) -> Survey:
    """Three-layer earth plus conductive block, 11x11 stations at 1 km, 8 frequencies
    log-spaced 0.01-100 Hz; optional seeded Gaussian noise on log10 sigma of earth cells."""
    st = station_grid(n_side, spacing)
    fr = np.logspace(-2, 2, 8) if freqs is None else np.asarray(freqs, dtype=np.float64)
    sigma0 = 0.01
    domain, radius = driver_domain(st, fr, half_width, sigma0, max_level, radius)
    lv = build_octree(domain, min_level, max_level, st, fr, station_refine_radius=radius,
                      sigma_bg=sigma0, lib=lib)
    sig = assign_sigma(lv, layered_block_sigma)
    if noise_std > 0:
        rng = np.random.default_rng(seed)
        earth = lv.cell_type == 0
        sig[earth] = sig[earth] * 10.0 ** rng.normal(0.0, noise_std, int(earth.sum()))
    return Survey("layered_block", lv, sig, sigma0, st, fr,
                  {"station_refine_radius": radius})


def c3_surveys(freqs=None, *, min_level=None, max_level=None, seed=11, lib=None, workers=8) -> list:
    """C3: one survey per frequency, each mesh refined for that frequency's
    skin depth alone (so the meshes differ in size), the C2 earth with log10
    sigma of earth cells perturbed by seeded N(0, 0.3^2) noise, 121 stations
    on an 11 x 11 grid at 1 km.  The meshes are built on `workers` host
    threads (the leaf builder is native code and runs outside the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    from . import workloads
    sp = workloads.C3
    fr = np.asarray(sp.freqs if freqs is None else freqs, dtype=np.float64).reshape(-1)
    lib = lib or _loader.load()

    def one(i):
        return layered_block_survey(min_level=sp.min_level if min_level is None else min_level,
                                    max_level=sp.max_level if max_level is None else max_level,
                                    n_side=sp.n_side, spacing=sp.spacing, freqs=np.array([fr[i]]),
                                    noise_std=workloads.C3_NOISE_STD, seed=seed + i, lib=lib)
    with ThreadPoolExecutor(max_workers=max(1, min(workers, len(fr)))) as ex:
        return list(ex.map(one, range(len(fr))))


def c5_survey(*, seed=7, rho_start=100.0, lib=None) -> Survey:
    """C5, the inversion iteration at scale: octree levels 6/8 (about 3.1 M
    edges), 400 stations on a 20x20 grid at 1 km, 24 frequencies log-spaced
    0.001-1000 Hz.  `sigma` is the starting model (a 100 ohm-m halfspace under
    air); meta["sigma_true"] is the seeded random layered-plus-blocks model
    the synthetic data come from."""
    from . import workloads
    sp = workloads.C5
    sv = layered_block_survey(min_level=sp.min_level, max_level=sp.max_level, n_side=sp.n_side,
                              spacing=sp.spacing, freqs=np.asarray(sp.freqs), lib=lib)
    lv = sv.leaves
    true = workloads.cell_sigma(lv.cell_type, lv.cx, lv.cy, lv.cz, workloads.random_layered_blocks(seed))
    start = workloads.cell_sigma(lv.cell_type, lv.cx, lv.cy, lv.cz, workloads.halfspace_sigma(rho_start))
    return Survey("c5", lv, start, sv.sigma_bg, sv.stations, sv.freqs,
                  {**sv.meta, "sigma_true": true, "seed": seed, "rho_start": rho_start})


def small_survey(*, min_level=2, max_level=4, n_side=2, spacing=4000.0, freqs=(0.5,),
                 half_width=20000.0, block=True, lib=None) -> Survey:
    """A few-thousand-edge mesh with hanging faces, for parity tests."""
    st = station_grid(n_side, spacing)
    fr = np.asarray(freqs, dtype=np.float64)
    sigma0 = 0.01
    dmax = skin_depth(float(fr.min()), sigma0)
    domain = (-half_width, half_width, -half_width, half_width, -1.5 * dmax, 0.5 * dmax)
    lv = build_octree(domain, min_level, max_level, st, fr, station_refine_radius=3000.0,
                      sigma_bg=sigma0, lib=lib)

    def earth(x, y, z):
        s = np.where(z > -2000.0, 0.02, 0.005)
        if block:
            b = (np.abs(x) < 3000) & (np.abs(y) < 3000) & (z < -500) & (z > -4000)
            s = np.where(b, 0.5, s)
        return s
    sig = assign_sigma(lv, earth)
    return Survey("small", lv, sig, sigma0, st, fr, {})


def leaves_struct(lv: Leaves):
    """ctypes m3d_leaves over the arrays of `lv` (keep `lv` alive while it is used)."""
    s = _abi.Leaves()
    for i in range(6):
        s.domain[i] = float(lv.domain[i])
    s.min_level = int(lv.min_level)
    s.max_level = int(lv.max_level)
    s.n_cells = int(lv.n_cells)
    for name in ("level", "cell_type"):
        a = getattr(lv, name)
        assert a.dtype == np.int32 and a.flags.c_contiguous
        setattr(s, name, a.ctypes.data_as(_abi.c_int_p))
    for name in ("cx", "cy", "cz"):
        a = getattr(lv, name)
        assert a.dtype == np.float64 and a.flags.c_contiguous
        setattr(s, name, a.ctypes.data_as(_abi.c_double_p))
    return s


def host_layout(lv: Leaves, lib=None) -> dict:
    """The solver's host layout (edges, stiffness S, hanging pairs) as numpy arrays."""
    lib = lib or _loader.load()
    st = leaves_struct(lv)
    h = C.c_void_p()
    rc = lib.m3d_layout_build(C.byref(st), C.byref(h))
    if rc != 0:
        raise RuntimeError(f"m3d_layout_build failed with code {rc}")
    try:
        ne, nf, nc, nn, nnz, nh = (C.c_int() for _ in range(6))
        lib.m3d_layout_sizes(h, C.byref(ne), C.byref(nf), C.byref(nc), C.byref(nn), C.byref(nnz),
                             C.byref(nh))
        ne, nf, nc, nn, nnz, nh = (v.value for v in (ne, nf, nc, nn, nnz, nh))
        xyz = np.zeros((ne, 3)); ln = np.zeros(ne); d = np.zeros(ne, np.int32)
        ad = np.zeros(ne); dead = np.zeros(ne, np.int32)
        n1 = np.zeros(ne, np.int32); n2 = np.zeros(ne, np.int32)
        ip = lambda a: a.ctypes.data_as(_abi.c_int_p)  # noqa: E731
        dp = lambda a: a.ctypes.data_as(_abi.c_double_p)  # noqa: E731
        lib.m3d_layout_edges(h, dp(xyz), dp(ln), ip(d), dp(ad), ip(dead), ip(n1), ip(n2))
        ptr = np.zeros(ne + 1, np.int32); idx = np.zeros(nnz, np.int32); val = np.zeros(nnz)
        lib.m3d_layout_stiffness(h, ip(ptr), ip(idx), dp(val))
        hp = np.zeros((nh, 3), np.int32)
        if nh:
            lib.m3d_layout_hanging(h, ip(hp))
    finally:
        lib.m3d_layout_destroy(h)
    return dict(n_edges=ne, n_faces=nf, n_cells=nc, n_nodes=nn, xyz=xyz, length=ln, direction=d,
                dual_area=ad, dead=dead, node1=n1, node2=n2, s_ptr=ptr, s_idx=idx, s_val=val,
                hanging=hp)
