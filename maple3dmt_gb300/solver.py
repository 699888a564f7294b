"""Python face of the GB300 solver, shaped like the reference's IForwardSolver.

Method names follow maple3dmt::forward::IForwardSolver
(include/maple3dmt/forward/iforward_solver.h:31-115) and ForwardSolverFV
(include/maple3dmt/forward/forward_solver_fv.h:77-187); each call goes
straight through the C ABI of include/m3d_gb300.h to the CUDA path.  There is
no CPU fallback: without a CUDA device, construction raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _loader, mesh
from ._abi import c_double_p, c_int_p
from ._abi_solver import KERNEL_CLASSES, KernelTimes, Params, RegParams, Stats, TuneEntry

ERRORS = {1: "ARG", 2: "STATE", 3: "CUDA", 4: "OOM", 5: "NO_DEVICE", 6: "TOO_LARGE", 7: "NUMERIC"}


class SolverError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"M3D_ERR_{ERRORS.get(code, code)}: {msg}")
        self.code = code


def default_params(**overrides) -> Params:
    lib = _loader.load()
    p = Params()
    lib.m3d_params_default(C.byref(p))
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _c(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a, a.ctypes.data_as(c_double_p)


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(c_double_p)


class ForwardSolverFV:
    """GPU forward + adjoint octree-FV solver (one CUDA device)."""

    def __init__(self, device: int = 0, lib=None):
        self.lib = lib or _loader.load()
        h = C.c_void_p()
        rc = self.lib.m3d_solver_create(int(device), C.byref(h))
        if rc != 0:
            raise SolverError(rc, "m3d_solver_create failed")
        self.h = h
        self.ne = self.nc = self.nn = self.n_colours = 0
        self.ns = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.m3d_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            raise SolverError(rc, self.lib.m3d_last_error(self.h).decode(errors="replace"))

    # -- setup ------------------------------------------------------------
    def setup(self, leaves: mesh.Leaves, params: Params | None = None, **kw):
        p = params or default_params(**kw)
        self._leaves = leaves
        self._krylov = [p.krylov, p.fgmres_m, p.learned_period]
        st = mesh.leaves_struct(leaves)
        self._ck(self.lib.m3d_solver_setup(self.h, C.byref(st), C.byref(p)))
        ne, nc, nn, ncol = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._ck(self.lib.m3d_solver_sizes(self.h, C.byref(ne), C.byref(nc), C.byref(nn), C.byref(ncol)))
        self.ne, self.nc, self.nn, self.n_colours = ne.value, nc.value, nn.value, ncol.value
        return self

    def set_sigma(self, sigma):
        s, p = _d(sigma)
        self._ck(self.lib.m3d_set_sigma(self.h, p, int(s.shape[0])))

    def set_stations(self, xyz):
        a, p = _d(np.asarray(xyz).reshape(-1, 3))
        self.ns = a.shape[0]
        self._ck(self.lib.m3d_set_stations(self.h, p, self.ns))

    def set_solver_tolerance_override(self, tol):
        self._ck(self.lib.m3d_set_tolerance_override(self.h, float(tol)))

    def current_omega(self) -> float:
        o = C.c_double()
        self._ck(self.lib.m3d_current_omega(self.h, C.byref(o)))
        return o.value

    # -- per frequency ----------------------------------------------------
    def compute_single_frequency(self, freq):
        Z = np.zeros((self.ns, 4), np.complex128)
        self._ck(self.lib.m3d_compute_single_frequency(self.h, float(freq), Z.ctypes.data_as(c_double_p)))
        return Z

    def factorize_frequency(self, freq):
        self._ck(self.lib.m3d_factorize_frequency(self.h, float(freq)))

    def release_factorization(self):
        self._ck(self.lib.m3d_release_factorization(self.h))

    def background_E(self, pol):
        E = np.zeros(self.ne, np.complex128)
        self._ck(self.lib.m3d_background_E(self.h, int(pol), E.ctypes.data_as(c_double_p)))
        return E

    def set_background_fields_complex(self, E1, E2):
        a, pa = _c(E1)
        b, pb = _c(E2)
        self._ck(self.lib.m3d_set_background_fields(self.h, pa, pb))

    def build_adjoint_rhs_from_residual(self, wr):
        w, pw = _c(np.asarray(wr).reshape(self.ns, 4))
        r1 = np.zeros(self.ne, np.complex128)
        r2 = np.zeros(self.ne, np.complex128)
        self._ck(self.lib.m3d_build_adjoint_rhs(self.h, pw, r1.ctypes.data_as(c_double_p),
                                                r2.ctypes.data_as(c_double_p)))
        return r1, r2

    def adjoint_solve_complex(self, rhs):
        r, pr = _c(rhs)
        lam = np.zeros(self.ne, np.complex128)
        self._ck(self.lib.m3d_adjoint_solve(self.h, pr, lam.ctypes.data_as(c_double_p)))
        return lam

    def solve_rhs_complex(self, rhs):
        r, pr = _c(rhs)
        x = np.zeros(self.ne, np.complex128)
        self._ck(self.lib.m3d_solve_rhs(self.h, pr, x.ctypes.data_as(c_double_p)))
        return x

    def solve_rhs_batch(self, rhs):
        """Many right-hand sides [n][n_edges] at the factorised frequency (16 per batched solve)."""
        r, pr = _c(np.atleast_2d(rhs))
        out = np.zeros_like(r)
        self._ck(self.lib.m3d_solve_rhs_batch(self.h, pr, int(r.shape[0]), out.ctypes.data_as(c_double_p)))
        return out

    def station_gradients(self, wr):
        """Gradients of residual sources wr [n_src][n_stations][4] complex at the
        solved single frequency, one per source: g [n_src][n_cells]
        (m3d_station_gradients)."""
        w, pw = _c(np.asarray(wr).reshape(-1, self.ns, 4))
        g = np.zeros((w.shape[0], self.nc))
        self._ck(self.lib.m3d_station_gradients(self.h, pw, int(w.shape[0]), g.ctypes.data_as(c_double_p)))
        return g

    def compute_sensitivity_complex(self, E, lam):
        e, pe = _c(E)
        l, pl = _c(lam)
        g = np.zeros(self.nc)
        self._ck(self.lib.m3d_compute_sensitivity(self.h, pe, pl, g.ctypes.data_as(c_double_p)))
        return g

    def build_perturbation_rhs_complex(self, pol, delta_sigma):
        d, pd = _d(delta_sigma)
        out = np.zeros(self.ne, np.complex128)
        self._ck(self.lib.m3d_build_perturbation_rhs(self.h, int(pol), pd, out.ctypes.data_as(c_double_p)))
        return out

    def extract_delta_impedance_complex(self, dE, pol):
        e, pe = _c(dE)
        dZ = np.zeros((self.ns, 4), np.complex128)
        self._ck(self.lib.m3d_extract_delta_impedance(self.h, pe, int(pol), dZ.ctypes.data_as(c_double_p)))
        return dZ

    # -- batched ----------------------------------------------------------
    def forward_batch(self, freqs, with_fields=False):
        f, pf = _d(freqs)
        Z = np.zeros((f.shape[0], self.ns, 4), np.complex128)
        E = np.zeros((f.shape[0], 2, self.ne), np.complex128) if with_fields else None
        self._ck(self.lib.m3d_forward_batch(self.h, pf, int(f.shape[0]), Z.ctypes.data_as(c_double_p),
                                            E.ctypes.data_as(c_double_p) if with_fields else None))
        return (Z, E) if with_fields else Z

    def gradient_batch(self, freqs, obs_Z, obs_err):
        f, pf = _d(freqs)
        oz, poz = _c(obs_Z)
        oe, poe = _d(obs_err)
        Z = np.zeros((f.shape[0], self.ns, 4), np.complex128)
        g = np.zeros(self.nc)
        self._ck(self.lib.m3d_gradient_batch(self.h, pf, int(f.shape[0]), poz, poe,
                                             Z.ctypes.data_as(c_double_p), g.ctypes.data_as(c_double_p)))
        return Z, g

    def jtjv_batch(self, freqs, dsigma, obs_err, inner_tol=1e-4):
        """J^T W^2 J dsigma summed over freqs (ImplicitJtJOperatorFV::Mult without
        the regularisation term); needs the background fields of the same
        frequencies from forward_batch."""
        f, pf = _d(freqs)
        ds, pds = _d(dsigma)
        oe, poe = _d(obs_err)
        out = np.zeros(self.nc)
        self._ck(self.lib.m3d_jtjv_batch(self.h, pf, int(f.shape[0]), pds, poe, float(inner_tol),
                                         out.ctypes.data_as(c_double_p)))
        return out

    # -- octree regularisation (RegularizationOctree) --------------------
    def reg_setup(self, alpha_s=1.0, alpha_x=1.0, alpha_y=1.0, alpha_z=1.0, n_smooth=2):
        p = RegParams(float(alpha_s), float(alpha_x), float(alpha_y), float(alpha_z), int(n_smooth))
        self._ck(self.lib.m3d_reg_setup(self.h, C.byref(p)))
        n = C.c_int()
        self._ck(self.lib.m3d_reg_num_active(self.h, C.byref(n)))
        self.n_active = n.value
        return self.n_active

    def reg_active_to_global(self):
        out = np.zeros(self.n_active, np.int32)
        self._ck(self.lib.m3d_reg_active_to_global(self.h, out.ctypes.data_as(c_int_p)))
        return out

    def reg_apply_wtw(self, x):
        a, pa = _d(x)
        y = np.zeros(self.n_active)
        self._ck(self.lib.m3d_reg_apply_wtw(self.h, pa, y.ctypes.data_as(c_double_p)))
        return y

    def reg_apply_cmcmt(self, x):
        a, pa = _d(x)
        y = np.zeros(self.n_active)
        self._ck(self.lib.m3d_reg_apply_cmcmt(self.h, pa, y.ctypes.data_as(c_double_p)))
        return y

    def reg_diagonal_wtw(self):
        d = np.zeros(self.n_active)
        self._ck(self.lib.m3d_reg_diagonal_wtw(self.h, d.ctypes.data_as(c_double_p)))
        return d

    def reg_evaluate(self, log_sigma, ref=None):
        p, pp = _d(log_sigma)
        r, pr = _d(ref) if ref is not None else (None, None)
        v = C.c_double()
        g = np.zeros(self.nc)
        self._ck(self.lib.m3d_reg_evaluate(self.h, pp, pr, C.byref(v), g.ctypes.data_as(c_double_p)))
        return v.value, g

    def dot_batched(self, x_ptr: int, y_ptr: int, n: int, K: int, out_ptr: int):
        """Hermitian dots of K interleaved complex128 device vectors ([n][K]);
        writes K complex values at device address out_ptr."""
        self._ck(self.lib.m3d_dot_batched(self.h, x_ptr, y_ptr, int(n), int(K), out_ptr))

    def timer_start(self):
        self._ck(self.lib.m3d_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._ck(self.lib.m3d_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def autotune(self, freq, max_K=16, reps=10, force=False) -> dict:
        """Measure and apply the row-kernel layout and the right-hand-side
        block of the batched FP32 inner solve (include/m3d_gb300.h)."""
        table = (TuneEntry * 8)()
        n, rk, blk, cached = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._ck(self.lib.m3d_autotune(self.h, float(freq), int(max_K), int(reps), 1 if force else 0, table,
                                       C.byref(n), C.byref(rk), C.byref(blk), C.byref(cached)))
        return dict(row_kernels=rk.value, rhs_block=blk.value, cached=bool(cached.value),
                    table=[dict(row_kernels=t.row_kernels, K=t.K, ms_per_iter=t.ms_per_iter,
                                ms_per_rhs_iter=t.ms_per_rhs_iter) for t in table[:n.value]])

    def set_params(self, krylov=None, fgmres_m=None, learned_period=None):
        """Change the inner solve between calls (m3d_set_krylov)."""
        k = self._krylov
        for i, v in enumerate((krylov, fgmres_m, learned_period)):
            if v is not None:
                k[i] = int(v)
        self._ck(self.lib.m3d_set_krylov(self.h, *k))

    # ---- learned preconditioner (include/m3d_gb300.h, m3d_learn_*) ----
    def learn_setup(self, grid_level=5, layers=6, hidden=32, seed=0, max_samples=5000):
        self._ck(self.lib.m3d_learn_setup(self.h, int(grid_level), int(layers), int(hidden), int(seed),
                                          int(max_samples)))

    def learn_collect(self, freqs) -> int:
        f, pf = _d(np.asarray(freqs, np.float64).reshape(-1))
        n = C.c_longlong()
        self._ck(self.lib.m3d_learn_collect(self.h, pf, int(f.shape[0]), C.byref(n)))
        return n.value

    def learn_train(self, epochs=20, lr=1e-3, batch=16, seed=0, val_frac=0.1):
        hist = np.zeros(int(epochs))
        val = C.c_double()
        self._ck(self.lib.m3d_learn_train(self.h, int(epochs), float(lr), int(batch), int(seed), float(val_frac),
                                          hist.ctypes.data_as(c_double_p), C.byref(val)))
        return hist, val.value

    def test_set_consume_no_wait(self, on: bool):
        """Test hook: staged kernels take their copy-wait timeout path."""
        self._ck(self.lib.m3d_test_set_consume_no_wait(self.h, 1 if on else 0))

    def set_kernel_timing(self, on: bool):
        self._ck(self.lib.m3d_set_kernel_timing(self.h, 1 if on else 0))

    def kernel_times(self) -> dict:
        t = KernelTimes()
        self._ck(self.lib.m3d_get_kernel_times(self.h, C.byref(t)))
        kb = ("K2", "K4", "K8", "K16", "other")
        return {name: dict(launches=t.launches[i], ms=t.ms[i], bytes=t.bytes[i],
                           by_k={kb[j]: dict(launches=t.launches_k[i][j], ms=t.ms_k[i][j], bytes=t.bytes_k[i][j])
                                 for j in range(5) if t.launches_k[i][j]})
                for i, name in enumerate(KERNEL_CLASSES)}

    def stats(self) -> dict:
        s = Stats()
        self._ck(self.lib.m3d_get_stats(self.h, C.byref(s)))
        n = min(s.n_rhs, 64)
        return dict(n_rhs=s.n_rhs, iterations=list(s.iterations[:n]), status=list(s.status[:n]),
                    true_residual=list(s.true_residual[:n]), total_iterations=s.total_iterations,
                    refinements=s.refinements, seconds=s.seconds, kernel_launches=s.kernel_launches,
                    divcorr_calls=s.divcorr_calls, divcorr_outer=s.divcorr_outer,
                    divcorr_cg_iterations=s.divcorr_cg_iterations,
                    forward_iterations=s.forward_iterations, adjoint_iterations=s.adjoint_iterations,
                    divcorr_cg_sweeps=s.divcorr_cg_sweeps, divcorr_setup_ms=s.divcorr_setup_ms,
                    replacements=s.replacements, graphs_failed=s.graphs_failed, graph_replays=s.graph_replays)


def solver_for_survey(sv: mesh.Survey, device=0, **params) -> ForwardSolverFV:
    s = ForwardSolverFV(device)
    params.setdefault("sigma_bg", sv.sigma_bg)
    s.setup(sv.leaves, **params)
    s.set_sigma(sv.sigma)
    s.set_stations(sv.stations)
    return s


def solvers_for_surveys(surveys, device=0, workers=8, **params) -> list:
    """One handle per survey (e.g. C3's per-frequency meshes), set up on
    `workers` host threads: each set-up (layout, colouring, segments,
    multigrid aggregation, uploads) is native code on its own handle and
    stream and runs outside the GIL."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=max(1, min(workers, len(surveys)))) as ex:
        return list(ex.map(lambda sv: solver_for_survey(sv, device=device, **params), surveys))


def group_station_gradients(solvers, freqs, wr, max_concurrent=0):
    """Per-frequency meshes run concurrently on one device
    (m3d_group_station_gradients): solvers[m] at freqs[m], residual sources
    wr[m] [n_src][n_stations][4].  Returns (Z [m] [n_stations][4],
    g [m] [n_src][n_cells(m)], status [m])."""
    n = len(solvers)
    if n < 1 or len(freqs) != n or len(wr) != n:
        raise ValueError("one frequency and one source set per solver")
    lib = solvers[0].lib
    hs = (C.c_void_p * n)(*[s.h for s in solvers])
    fr = np.ascontiguousarray(np.asarray(freqs, np.float64))
    ws = [np.ascontiguousarray(np.asarray(w, np.complex128).reshape(-1, s.ns, 4)) for w, s in zip(wr, solvers)]
    ns = (C.c_int * n)(*[w.shape[0] for w in ws])
    Z = [np.zeros((s.ns, 4), np.complex128) for s in solvers]
    g = [np.zeros((w.shape[0], s.nc)) for w, s in zip(ws, solvers)]
    pw = (c_double_p * n)(*[w.ctypes.data_as(c_double_p) for w in ws])
    pz = (c_double_p * n)(*[z.ctypes.data_as(c_double_p) for z in Z])
    pg = (c_double_p * n)(*[a.ctypes.data_as(c_double_p) for a in g])
    st = (C.c_int * n)()
    rc = lib.m3d_group_station_gradients(hs, n, fr.ctypes.data_as(c_double_p), pw, ns, pz, pg, int(max_concurrent), st)
    status = list(st)
    if rc != 0:
        m = next(i for i, v in enumerate(status) if v != 0)
        raise SolverError(rc, f"mesh {m}: " + lib.m3d_last_error(solvers[m].h).decode(errors="replace"))
    return Z, g, status
