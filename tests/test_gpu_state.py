"""Solver state across call sequences (GPU, through the C ABI).

The solver keeps the background field, the station cache and buffers sized by
the station count between calls.  These tests run call sequences that grow
one buffer while another caller still depends on what it held, and check each
result against a solver that only ever ran the final call.
"""
import numpy as np
import pytest

from conftest import leaves_from_golden, load_golden, rel

pytestmark = pytest.mark.gpu

G_TOL = 1e-4


def _gpu(g, stations=None, **params):
    from maple3dmt_gb300.solver import ForwardSolverFV
    s = ForwardSolverFV(0)
    params.setdefault("sigma_bg", float(g["sigma_bg"]))
    params.setdefault("bicgstab_tol", 1e-10)
    params.setdefault("bicgstab_maxiter", 5000)
    params.setdefault("precision", 1)
    s.setup(leaves_from_golden(g), **params)
    s.set_sigma(g["sigma"])
    s.set_stations(g["stations"] if stations is None else stations)
    return s


@pytest.fixture(scope="module")
def g_small(lib):
    return load_golden("small_block")


def _dsig(g, seed=5):
    rng = np.random.default_rng(seed)
    return np.where(g["cell_type"] == 0, g["sigma"] * 0.1 * rng.normal(size=g["sigma"].shape), 0.0)


def test_wide_rhs_batch_keeps_background_field(g_small):
    """forward_batch (4 lanes), then solve_rhs_batch with 20 right-hand sides
    (scratch regrown to 16 lanes), then jtjv_batch on the background field of
    the forward call: equal to jtjv_batch straight after forward_batch."""
    g = g_small
    freqs = g["freqs"]
    err = np.ascontiguousarray(g["obs_err"])
    dsig = _dsig(g)
    a = _gpu(g)
    a.forward_batch(freqs)
    want = a.jtjv_batch(freqs, dsig, err, inner_tol=1e-10)
    E_want = [a.background_E(p) for p in (0, 1)]
    b = _gpu(g)
    b.forward_batch(freqs)
    rng = np.random.default_rng(11)
    B = rng.normal(size=(20, b.ne)) + 1j * rng.normal(size=(20, b.ne))
    X = b.solve_rhs_batch(B)
    assert np.isfinite(X).all()
    for p in (0, 1):
        assert rel(b.background_E(p), E_want[p]) < 1e-12
    got = b.jtjv_batch(freqs, dsig, err, inner_tol=1e-10)
    assert np.linalg.norm(want) > 0
    assert rel(got, want) < G_TOL


def test_more_stations_after_gradient_and_jtjv(g_small):
    """gradient_batch and jtjv_batch, then set_stations with more stations:
    both calls again give what a solver set up with the larger station set
    gives (the station-sized buffers follow the new count)."""
    g = g_small
    freqs = g["freqs"]
    nf = len(freqs)
    st0 = np.asarray(g["stations"], np.float64).reshape(-1, 3)
    s = _gpu(g)
    s.gradient_batch(freqs, g["obs_Z"], g["obs_err"])
    s.forward_batch(freqs)
    s.jtjv_batch(freqs, _dsig(g), np.ascontiguousarray(g["obs_err"]), inner_tol=1e-10)
    # a second, larger station set: the original stations plus shifted copies
    extra = st0.copy()
    extra[:, 0] += 0.37 * (st0[:, 0].max() - st0[:, 0].min() + 1.0)
    st1 = np.concatenate([st0, extra, st0 * 0.5])
    ns1 = st1.shape[0]
    rng = np.random.default_rng(3)
    obs1 = (rng.normal(size=(ns1, nf, 4)) + 1j * rng.normal(size=(ns1, nf, 4))) * np.abs(g["obs_Z"]).max()
    err1 = np.full((ns1, nf, 4), 0.05 * np.abs(g["obs_Z"]).max())
    s.set_stations(st1)
    Z_s, g_s = s.gradient_batch(freqs, obs1, err1)
    s.forward_batch(freqs)
    y_s = s.jtjv_batch(freqs, _dsig(g, 8), err1, inner_tol=1e-10)
    f = _gpu(g, stations=st1)
    Z_f, g_f = f.gradient_batch(freqs, obs1, err1)
    f.forward_batch(freqs)
    y_f = f.jtjv_batch(freqs, _dsig(g, 8), err1, inner_tol=1e-10)
    assert Z_s.shape == (nf, ns1, 4)
    assert rel(Z_s, Z_f) < 1e-8
    assert rel(g_s, g_f) < G_TOL
    assert rel(y_s, y_f) < G_TOL


def test_autotune_applies_and_caches(g_small):
    """The autotuner times both row-kernel layouts at K = 2..16, applies a
    choice that keeps the solve's results, and a second call on the same
    mesh and settings reuses the cached choice without timing."""
    g = g_small
    s = _gpu(g)
    r = s.autotune(g["freqs"][0], max_K=16, reps=5, force=True)
    assert not r["cached"]
    assert len(r["table"]) == 8
    assert {(t["row_kernels"], t["K"]) for t in r["table"]} == {(rk, k) for rk in (0, 1) for k in (2, 4, 8, 16)}
    assert all(t["ms_per_iter"] > 0 for t in r["table"])
    assert r["row_kernels"] in (0, 1) and r["rhs_block"] in (2, 4, 8, 16)
    f = _gpu(g)
    for fr in g["freqs"]:
        assert rel(s.compute_single_frequency(fr), f.compute_single_frequency(fr)) < 1e-6
    rng = np.random.default_rng(12)
    B = rng.normal(size=(5, s.ne)) + 1j * rng.normal(size=(5, s.ne))
    X = s.solve_rhs_batch(B)
    for k in (0, 4):
        assert rel(X[k], f.solve_rhs_complex(B[k])) < 1e-6
    r2 = _gpu(g).autotune(g["freqs"][0], max_K=16, reps=5)
    assert r2["cached"] and r2["row_kernels"] == r["row_kernels"] and r2["rhs_block"] == r["rhs_block"]
