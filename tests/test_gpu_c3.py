"""C3 pieces on the GPU, through the C ABI: per-source station gradients at
one frequency (m3d_station_gradients) against the oracle's composition of
the reference's single-source calls, and per-frequency meshes of uneven size
run concurrently (m3d_group_station_gradients) against the same meshes run
one handle at a time.

The reference computes a source's gradient as build_adjoint_rhs_from_residual
(forward_solver_fv.cpp:1804-2013), adjoint_solve_complex of each
polarisation (:914-924) and compute_sensitivity_complex (:989-1059) summed
over the polarisations (inversion_fv.cpp:280-290); both sides solve to 1e-10
and the gradients must agree to 1e-4 relative (the gradient target of the
solver's specification).
"""
import numpy as np
import pytest

from conftest import leaves_from_golden, load_golden, rel

pytestmark = pytest.mark.gpu

G_TOL = 1e-4


def _gpu(g, **params):
    from maple3dmt_gb300.solver import ForwardSolverFV
    s = ForwardSolverFV(0)
    params.setdefault("sigma_bg", float(g["sigma_bg"]))
    params.setdefault("bicgstab_tol", 1e-10)
    params.setdefault("bicgstab_maxiter", 5000)
    s.setup(leaves_from_golden(g), **params)
    s.set_sigma(g["sigma"])
    s.set_stations(g["stations"])
    return s


@pytest.fixture(scope="module")
def g_small(lib):
    return load_golden("small_block")


@pytest.mark.parametrize("precision", [0, 1])
def test_station_gradients_match_oracle(g_small, precision):
    """Ten sources (two batches: eight and two): one per station with the
    residual at that station only, then six with residuals at every station."""
    import oracle
    g = g_small
    s = _gpu(g, precision=precision)
    o = oracle.Oracle(oracle.Case.from_arrays(g, tol=1e-10, maxiter=5000))
    fr = float(g["freqs"][1])
    s.compute_single_frequency(fr)
    o.solve_frequency(fr)
    ns = s.ns
    rng = np.random.default_rng(21)
    wr = np.zeros((10, ns, 4), np.complex128)
    for j in range(ns):
        wr[j, j] = rng.normal(size=4) + 1j * rng.normal(size=4)
    wr[ns:] = rng.normal(size=(10 - ns, ns, 4)) + 1j * rng.normal(size=(10 - ns, ns, 4))
    G = s.station_gradients(wr)
    st = s.stats()
    assert st["n_rhs"] == 20
    assert all(t <= 1e-10 for t in st["true_residual"][:st["n_rhs"]]), st
    for j in range(10):
        a1, a2 = o.adjoint_rhs(wr[j])
        go = o.sensitivity(o.E(0), o.adjoint_solve(a1)) + o.sensitivity(o.E(1), o.adjoint_solve(a2))
        e = rel(G[j], go)
        print(f"source {j}: gradient relative error {e:.2e}")
        assert np.abs(go).max() > 0
        assert e < G_TOL
    # linear in the residual: the sum of the station sources is the source of the summed residual
    Gs = s.station_gradients(wr[:ns].sum(axis=0, keepdims=True))
    assert rel(Gs[0], G[:ns].sum(axis=0)) < 1e-6


def test_station_gradients_need_a_solved_frequency(g_small):
    from maple3dmt_gb300.solver import SolverError
    s = _gpu(g_small)
    with pytest.raises(SolverError) as ex:
        s.station_gradients(np.zeros((1, s.ns, 4), np.complex128))
    assert ex.value.code == 2
    s.compute_single_frequency(float(g_small["freqs"][0]))
    bad = np.zeros((1, s.ns, 4), np.complex128)
    bad[0, 0, 1] = np.nan
    with pytest.raises(SolverError) as ex:
        s.station_gradients(bad)
    assert ex.value.code == 7


def test_station_gradients_of_no_source(g_small):
    """Zero sources is an empty result, not an error (the reference's loop
    over no stations does nothing)."""
    s = _gpu(g_small)
    s.compute_single_frequency(float(g_small["freqs"][0]))
    G = s.station_gradients(np.zeros((0, s.ns, 4), np.complex128))
    assert G.shape == (0, s.nc)


@pytest.fixture(scope="module")
def small_c3(lib):
    from maple3dmt_gb300 import mesh
    return mesh.c3_surveys([0.01, 1.0, 100.0], min_level=3, max_level=5)


def test_group_matches_one_handle_at_a_time(small_c3):
    """Three per-frequency meshes (uneven sizes) run concurrently give the
    impedances and station gradients of the same handles run one at a time
    (the same arithmetic in the same order: agreement to rounding noise)."""
    from maple3dmt_gb300 import workloads
    from maple3dmt_gb300.solver import group_station_gradients, solvers_for_surveys
    svs = small_c3
    # the handles are set up on host threads, as the C3 bench does
    solvers = solvers_for_surveys(svs, workers=3, bicgstab_tol=1e-7, bicgstab_maxiter=5000, precision=1)
    sizes = [s.ne for s in solvers]
    assert len(set(sizes)) > 1, sizes
    rng = np.random.default_rng(3)
    wr = [workloads.station_sources(s.ns, rng)[:12] for s in solvers]
    freqs = [float(sv.freqs[0]) for sv in svs]
    Zg, Gg, status = group_station_gradients(solvers, freqs, wr)
    assert status == [0, 0, 0]
    for m, s in enumerate(solvers):
        Z1 = s.compute_single_frequency(freqs[m])
        G1 = s.station_gradients(wr[m])
        st = s.stats()
        assert all(t <= 1e-7 for t in st["true_residual"][:st["n_rhs"]]), st
        print(f"mesh {m}: {s.ne} edges, {freqs[m]:g} Hz, |g| {np.abs(G1).max():.3e}")
        assert rel(Zg[m], Z1) < 1e-10
        assert rel(Gg[m], G1) < 1e-10
        assert np.abs(G1).max() > 0
    # at most one mesh at a time gives the same results
    Zs, Gs, _ = group_station_gradients(solvers, freqs, wr, max_concurrent=1)
    for m in range(len(solvers)):
        assert rel(Zs[m], Zg[m]) < 1e-10 and rel(Gs[m], Gg[m]) < 1e-10


def test_group_rejects_a_repeated_handle(small_c3):
    from maple3dmt_gb300.solver import SolverError, group_station_gradients, solver_for_survey
    s = solver_for_survey(small_c3[0], bicgstab_tol=1e-7, precision=1)
    w = np.zeros((1, s.ns, 4), np.complex128)
    with pytest.raises(SolverError) as ex:
        group_station_gradients([s, s], [1.0, 1.0], [w, w])
    assert ex.value.code == 1
