"""CPU checkers for the GPU solve.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.  It wraps two libraries:

* ``libm3d_oracle.so`` - the C restatement in m3d_oracle.c (built with gcc
  here and on any machine that runs the tests);
* ``_ref/libm3d_ref.so`` - the reference's own solver sources compiled by
  build_ref.sh (only where the reference tree is present).
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "libm3d_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libm3d_ref.so")

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement (IEEE order kept: -ffp-contract=off)."""
    src = os.path.join(HERE, "m3d_oracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-shared",
                           "-o", tmp, src, "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(reference_root: str = "/root/reference") -> str | None:
    """Compile the reference's own sources into _ref/ when its tree is present."""
    if not os.path.isdir(os.path.join(reference_root, "src", "forward")):
        return REF_SO if os.path.exists(REF_SO) else None
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), reference_root],
                          stdout=subprocess.DEVNULL)
    return REF_SO


class CaseStruct(C.Structure):
    """struct m3d_case (m3d_case.h)."""
    _fields_ = [
        ("domain", C.c_double * 6), ("min_level", C.c_int), ("max_level", C.c_int),
        ("n_cells", C.c_int), ("level", ip), ("cx", dp), ("cy", dp), ("cz", dp),
        ("cell_type", ip), ("sigma", dp), ("sigma_bg", C.c_double),
        ("n_stations", C.c_int), ("station_xyz", dp), ("n_freqs", C.c_int), ("freqs", dp),
        ("bicgstab_tol", C.c_double), ("bicgstab_maxiter", C.c_int),
        ("scattered_field", C.c_int), ("air_z_threshold", C.c_double),
        ("div_correction", C.c_int), ("div_corr_iters", C.c_int), ("div_corr_tol", C.c_double),
        ("divcorr_outer_max", C.c_int), ("divcorr_iter_per_dc", C.c_int),
        ("obs_Z", dp), ("obs_err", dp),
    ]


class Case:
    """Owns the numpy arrays behind an m3d_case so the pointers stay valid."""

    def __init__(self, *, domain, min_level, max_level, level, cx, cy, cz, cell_type, sigma,
                 sigma_bg, stations, freqs, tol=1e-7, maxiter=5000, scattered_field=1,
                 air_z_threshold=1.0, div_correction=1, div_corr_iters=10, div_corr_tol=2e-3,
                 divcorr_outer_max=20, divcorr_iter_per_dc=500, obs_Z=None, obs_err=None):
        a = lambda x, t: np.ascontiguousarray(np.asarray(x, dtype=t))  # noqa: E731
        self.level = a(level, np.int32); self.cx = a(cx, np.float64); self.cy = a(cy, np.float64)
        self.cz = a(cz, np.float64); self.cell_type = a(cell_type, np.int32)
        self.sigma = a(sigma, np.float64)
        self.stations = a(np.asarray(stations).reshape(-1, 3), np.float64)
        self.freqs = a(np.asarray(freqs).reshape(-1), np.float64)
        self.obs_Z = None if obs_Z is None else a(obs_Z, np.complex128)
        self.obs_err = None if obs_err is None else a(obs_err, np.float64)
        s = CaseStruct()
        for i in range(6):
            s.domain[i] = float(domain[i])
        s.min_level = int(min_level); s.max_level = int(max_level)
        s.n_cells = int(self.level.shape[0])
        s.level = self.level.ctypes.data_as(ip)
        s.cx = self.cx.ctypes.data_as(dp); s.cy = self.cy.ctypes.data_as(dp)
        s.cz = self.cz.ctypes.data_as(dp)
        s.cell_type = self.cell_type.ctypes.data_as(ip)
        s.sigma = self.sigma.ctypes.data_as(dp)
        s.sigma_bg = float(sigma_bg)
        s.n_stations = int(self.stations.shape[0])
        s.station_xyz = self.stations.ctypes.data_as(dp)
        s.n_freqs = int(self.freqs.shape[0])
        s.freqs = self.freqs.ctypes.data_as(dp)
        s.bicgstab_tol = float(tol); s.bicgstab_maxiter = int(maxiter)
        s.scattered_field = int(scattered_field); s.air_z_threshold = float(air_z_threshold)
        s.div_correction = int(div_correction); s.div_corr_iters = int(div_corr_iters)
        s.div_corr_tol = float(div_corr_tol); s.divcorr_outer_max = int(divcorr_outer_max)
        s.divcorr_iter_per_dc = int(divcorr_iter_per_dc)
        s.obs_Z = self.obs_Z.ctypes.data_as(dp) if self.obs_Z is not None else None
        s.obs_err = self.obs_err.ctypes.data_as(dp) if self.obs_err is not None else None
        self.struct = s

    @classmethod
    def from_survey(cls, sv, **kw):
        lv = sv.leaves
        return cls(domain=lv.domain, min_level=lv.min_level, max_level=lv.max_level,
                   level=lv.level, cx=lv.cx, cy=lv.cy, cz=lv.cz, cell_type=lv.cell_type,
                   sigma=sv.sigma, sigma_bg=sv.sigma_bg, stations=sv.stations, freqs=sv.freqs, **kw)

    @classmethod
    def from_arrays(cls, d: dict, **kw):
        keys = ("domain", "min_level", "max_level", "level", "cx", "cy", "cz", "cell_type",
                "sigma", "sigma_bg", "stations", "freqs")
        args = {k: d[k] for k in keys}
        args["min_level"] = int(np.asarray(args["min_level"]))
        args["max_level"] = int(np.asarray(args["max_level"]))
        args["sigma_bg"] = float(np.asarray(args["sigma_bg"]))
        args.update(kw)
        return cls(**args)


# ---------------------------------------------------------------------------
# the compiled reference
# ---------------------------------------------------------------------------

def _read_m3da(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        if f.read(8)[:5] != b"M3DA1":
            raise ValueError("bad M3DA file")
        while True:
            h = f.read(4)
            if not h:
                break
            (n,) = struct.unpack("<I", h)
            name = f.read(n).decode()
            dt = f.read(1).decode()
            (cnt,) = struct.unpack("<Q", f.read(8))
            t = {"f": np.float64, "i": np.int32, "c": np.complex128}[dt]
            out[name] = np.frombuffer(f.read(cnt * np.dtype(t).itemsize), dtype=t).copy()
    return out


def run_ref(case: Case, *, layout=True, forward=True, adjoint=True, regularization=False, log_level=4) -> dict:
    """Run the reference's own ForwardSolverFV on `case` (see ref_driver.cpp)."""
    if not os.path.exists(REF_SO):
        raise RuntimeError("oracle/_ref/libm3d_ref.so not built (reference tree absent?)")
    lib = C.CDLL(REF_SO)
    lib.ref_run.restype = C.c_int
    lib.ref_run.argtypes = [C.POINTER(CaseStruct), C.c_char_p, C.c_int, C.c_int]
    flags = (1 if layout else 0) | (2 if forward else 0) | (4 if adjoint else 0) | (8 if regularization else 0)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "out.m3da")
        rc = lib.ref_run(C.byref(case.struct), path.encode(), flags, int(log_level))
        if rc != 0:
            raise RuntimeError(f"ref_run failed: {rc}")
        return _read_m3da(path)


# ---------------------------------------------------------------------------
# the C restatement
# ---------------------------------------------------------------------------

_oracle_lib = None


def load_oracle():
    global _oracle_lib
    if _oracle_lib is None:
        lib = C.CDLL(build_oracle())
        vp = C.c_void_p
        sig = {
            "m3d_oracle_create": (vp, [C.POINTER(CaseStruct)]),
            "m3d_oracle_destroy": (None, [vp]),
            "m3d_oracle_sizes": (C.c_int, [vp, ip, ip, ip, ip]),
            "m3d_oracle_set_sigma": (C.c_int, [vp, dp]),
            "m3d_oracle_set_tol_override": (C.c_int, [vp, C.c_double]),
            "m3d_oracle_solve_frequency": (C.c_int, [vp, C.c_double, dp]),
            "m3d_oracle_factorize": (C.c_int, [vp, C.c_double]),
            "m3d_oracle_release": (C.c_int, [vp]),
            "m3d_oracle_get_E": (C.c_int, [vp, C.c_int, dp]),
            "m3d_oracle_set_E": (C.c_int, [vp, dp, dp]),
            "m3d_oracle_adjoint_rhs": (C.c_int, [vp, dp, dp, dp]),
            "m3d_oracle_adjoint_solve": (C.c_int, [vp, dp, dp]),
            "m3d_oracle_sensitivity": (C.c_int, [vp, dp, dp, dp]),
            "m3d_oracle_perturbation_rhs": (C.c_int, [vp, C.c_int, dp, dp]),
            "m3d_oracle_delta_impedance": (C.c_int, [vp, dp, C.c_int, dp]),
            "m3d_oracle_last_iters": (C.c_int, [vp, ip, C.c_int]),
            "m3d_oracle_station_cells": (C.c_int, [vp, ip]),
            "m3d_oracle_matrix_nnz": (C.c_int, [vp]),
            "m3d_oracle_get_matrix": (C.c_int, [vp, ip, ip, dp]),
            "m3d_oracle_get_edges": (C.c_int, [vp, dp, dp, ip, dp, ip, ip, ip]),
            "m3d_oracle_gradient": (C.c_int, [vp, dp, C.c_int, dp, dp, dp, dp]),
            "m3d_oracle_time_iterations": (C.c_double, [vp, C.c_double, C.c_int, dp]),
            "m3d_oracle_reg_create": (vp, [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
            "m3d_oracle_reg_destroy": (None, [vp]),
            "m3d_oracle_reg_num_active": (C.c_int, [vp]),
            "m3d_oracle_reg_active_to_global": (None, [vp, ip]),
            "m3d_oracle_reg_apply_wtw": (None, [vp, dp, dp]),
            "m3d_oracle_reg_diagonal": (None, [vp, dp]),
            "m3d_oracle_reg_apply_cmcmt": (None, [vp, dp, dp]),
            "m3d_oracle_reg_evaluate": (C.c_double, [vp, dp, dp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _oracle_lib = lib
    return _oracle_lib


def _p(a, t=dp):
    return a.ctypes.data_as(t)


class Oracle:
    """Python face of the C restatement, shaped like ForwardSolverFV."""

    def __init__(self, case: Case):
        self.lib = load_oracle()
        self.case = case
        self.h = self.lib.m3d_oracle_create(C.byref(case.struct))
        ne, nf, nc, nn = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.lib.m3d_oracle_sizes(self.h, C.byref(ne), C.byref(nf), C.byref(nc), C.byref(nn))
        self.ne, self.nf, self.nc, self.nn = ne.value, nf.value, nc.value, nn.value
        self.ns = case.stations.shape[0]

    def close(self):
        if self.h:
            self.lib.m3d_oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve_frequency(self, freq):
        Z = np.zeros((self.ns, 4), np.complex128)
        self.lib.m3d_oracle_solve_frequency(self.h, float(freq), _p(Z))
        return Z

    def factorize(self, freq):
        self.lib.m3d_oracle_factorize(self.h, float(freq))

    def release(self):
        self.lib.m3d_oracle_release(self.h)

    def E(self, pol):
        out = np.zeros(self.ne, np.complex128)
        self.lib.m3d_oracle_get_E(self.h, int(pol), _p(out))
        return out

    def set_E(self, E1, E2):
        E1 = np.ascontiguousarray(E1, np.complex128); E2 = np.ascontiguousarray(E2, np.complex128)
        self.lib.m3d_oracle_set_E(self.h, _p(E1), _p(E2))

    def adjoint_rhs(self, wr):
        wr = np.ascontiguousarray(np.asarray(wr, np.complex128).reshape(self.ns, 4))
        a1 = np.zeros(self.ne, np.complex128); a2 = np.zeros(self.ne, np.complex128)
        self.lib.m3d_oracle_adjoint_rhs(self.h, _p(wr), _p(a1), _p(a2))
        return a1, a2

    def adjoint_solve(self, rhs):
        rhs = np.ascontiguousarray(rhs, np.complex128)
        lam = np.zeros(self.ne, np.complex128)
        self.lib.m3d_oracle_adjoint_solve(self.h, _p(rhs), _p(lam))
        return lam

    def sensitivity(self, E, lam):
        E = np.ascontiguousarray(E, np.complex128); lam = np.ascontiguousarray(lam, np.complex128)
        g = np.zeros(self.nc)
        self.lib.m3d_oracle_sensitivity(self.h, _p(E), _p(lam), _p(g))
        return g

    def perturbation_rhs(self, pol, dsig):
        dsig = np.ascontiguousarray(dsig, np.float64)
        out = np.zeros(self.ne, np.complex128)
        self.lib.m3d_oracle_perturbation_rhs(self.h, int(pol), _p(dsig), _p(out))
        return out

    def delta_impedance(self, dE, pol):
        dE = np.ascontiguousarray(dE, np.complex128)
        dZ = np.zeros((self.ns, 4), np.complex128)
        self.lib.m3d_oracle_delta_impedance(self.h, _p(dE), int(pol), _p(dZ))
        return dZ

    def set_tol_override(self, tol):
        self.lib.m3d_oracle_set_tol_override(self.h, float(tol))

    def last_iters(self):
        buf = np.zeros(64, np.int32)
        n = self.lib.m3d_oracle_last_iters(self.h, _p(buf, ip), 64)
        return buf[:n].tolist()

    def station_cells(self):
        out = np.zeros(self.ns, np.int32)
        self.lib.m3d_oracle_station_cells(self.h, _p(out, ip))
        return out

    def matrix(self):
        nnz = self.lib.m3d_oracle_matrix_nnz(self.h)
        if nnz < 0:
            raise RuntimeError("no assembled system")
        ptr = np.zeros(self.ne + 1, np.int32); idx = np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.complex128)
        self.lib.m3d_oracle_get_matrix(self.h, _p(ptr, ip), _p(idx, ip), _p(val))
        return ptr, idx, val

    def edges(self):
        xyz = np.zeros((self.ne, 3)); ln = np.zeros(self.ne); d = np.zeros(self.ne, np.int32)
        ad = np.zeros(self.ne); dead = np.zeros(self.ne, np.int32)
        n1 = np.zeros(self.ne, np.int32); n2 = np.zeros(self.ne, np.int32)
        self.lib.m3d_oracle_get_edges(self.h, _p(xyz), _p(ln), _p(d, ip), _p(ad), _p(dead, ip),
                                      _p(n1, ip), _p(n2, ip))
        return dict(xyz=xyz, len=ln, dir=d, adual=ad, dead=dead, node1=n1, node2=n2)

    def time_iterations(self, freq, n_iter):
        """(seconds in n_iter reference BiCGStab+SSOR iterations, setup seconds)."""
        setup = C.c_double()
        t = self.lib.m3d_oracle_time_iterations(self.h, float(freq), int(n_iter), C.byref(setup))
        return t, setup.value

    def gradient(self, freqs, obs_Z, obs_err):
        fr = np.ascontiguousarray(freqs, np.float64)
        oz = np.ascontiguousarray(obs_Z, np.complex128); oe = np.ascontiguousarray(obs_err, np.float64)
        Z = np.zeros((len(fr), self.ns, 4), np.complex128)
        g = np.zeros(self.nc)
        self.lib.m3d_oracle_gradient(self.h, _p(fr), len(fr), _p(oz), _p(oe), _p(Z), _p(g))
        return Z, g


class Regularization:
    """RegularizationOctree (src/inversion/regularization_octree.cpp) restated
    in C on the mesh of an Oracle."""

    def __init__(self, orc: "Oracle", alpha_s=1.0, alpha_x=1.0, alpha_y=1.0, alpha_z=1.0, n_smooth=2):
        self.lib = orc.lib
        self.orc = orc
        self.h = self.lib.m3d_oracle_reg_create(orc.h, float(alpha_s), float(alpha_x), float(alpha_y),
                                                float(alpha_z), int(n_smooth))
        self.na = self.lib.m3d_oracle_reg_num_active(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.m3d_oracle_reg_destroy(self.h)
            self.h = None

    def active_to_global(self):
        out = np.zeros(self.na, np.int32)
        self.lib.m3d_oracle_reg_active_to_global(self.h, _p(out, ip))
        return out

    def apply_wtw(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.na)
        self.lib.m3d_oracle_reg_apply_wtw(self.h, _p(x), _p(y))
        return y

    def diagonal(self):
        d = np.zeros(self.na)
        self.lib.m3d_oracle_reg_diagonal(self.h, _p(d))
        return d

    def apply_cmcmt(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.na)
        self.lib.m3d_oracle_reg_apply_cmcmt(self.h, _p(x), _p(y))
        return y

    def evaluate(self, params, ref=None):
        p = np.ascontiguousarray(params, np.float64)
        r = None if ref is None else np.ascontiguousarray(ref, np.float64)
        g = np.zeros(len(p))
        v = self.lib.m3d_oracle_reg_evaluate(self.h, _p(p), _p(r) if r is not None else None, _p(g))
        return v, g

