"""Failure detection of the GPU solve (through the C ABI), in forms that
fault, trap or hang no GPU: bad inputs rejected on the host, the reference's
own breakdown and iteration-cap exits reached with ordinary inputs, and the
bounded copy wait of the slice-staged kernels made to give up through a test
hook (the block skips its work and waits, bounded, for its copies in flight).

Reference exits: bicgstab.cpp:53-58 (rho = 0), :80-85, :117-124, :152-157
(iteration cap); the reference has no non-finite input check (it iterates on
NaN to maxiter), the C ABI adds M3D_ERR_NUMERIC for that.
"""
import numpy as np
import pytest

from conftest import leaves_from_golden, load_golden, rel

pytestmark = pytest.mark.gpu

ERR_CUDA, ERR_NUMERIC = 3, 7
CONVERGED, BREAKDOWN, MAXITER = 1, 2, 3


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


def test_nonfinite_inputs_rejected(g_small):
    """A NaN or Inf in a right-hand side, field or data vector fails the call
    with M3D_ERR_NUMERIC before any launch; the solver stays usable."""
    from maple3dmt_gb300.solver import SolverError
    g = g_small
    s = _gpu(g, precision=1)
    s.compute_single_frequency(g["freqs"][0])
    rng = np.random.default_rng(4)
    b = rng.normal(size=s.ne) + 1j * rng.normal(size=s.ne)
    good = s.solve_rhs_complex(b)
    bad = b.copy()
    bad[s.ne // 2] = np.nan
    for call in (s.solve_rhs_complex, s.adjoint_solve_complex):
        with pytest.raises(SolverError) as e:
            call(bad)
        assert e.value.code == ERR_NUMERIC
    B = np.stack([b, bad])
    with pytest.raises(SolverError) as e:
        s.solve_rhs_batch(B)
    assert e.value.code == ERR_NUMERIC
    inf = b.copy()
    inf[0] = np.inf
    with pytest.raises(SolverError) as e:
        s.compute_sensitivity_complex(inf, b)
    assert e.value.code == ERR_NUMERIC
    obs = np.array(g["obs_Z"], copy=True)
    obs[0, 0, 1] = np.nan
    with pytest.raises(SolverError) as e:
        s.gradient_batch(g["freqs"], obs, g["obs_err"])
    assert e.value.code == ERR_NUMERIC
    assert rel(s.solve_rhs_complex(b), good) < 1e-8


@pytest.mark.parametrize("precision", [0, 1])
def test_maxiter_one_reports_status(g_small, precision):
    """bicgstab_maxiter = 1: the call returns, every right-hand side reports
    M3D_SOLVE_MAXITER with its true residual above the tolerance."""
    g = g_small
    s = _gpu(g, precision=precision, bicgstab_maxiter=1, forward_interleaved=0)
    Z = s.compute_single_frequency(g["freqs"][0])
    st = s.stats()
    assert st["n_rhs"] == 2
    assert st["status"][:2] == [MAXITER, MAXITER], st
    assert all(1 <= it <= 2 for it in st["iterations"][:2]), st
    assert all(t > 1e-10 for t in st["true_residual"][:2]), st
    assert np.isfinite(Z).all()


def test_rho_breakdown_matches_reference(g_small):
    """The reference's absolute breakdown test |rho| < 1e-30
    (bicgstab.cpp:53-58) met with an ordinary right-hand side of norm 1e-16:
    rho = |r|^2 = 1e-32 at the first iteration.  The FP64 solve reports
    M3D_SOLVE_BREAKDOWN after one iteration and returns x = 0, as the oracle
    (the reference's algorithm) does."""
    import oracle
    g = g_small
    s = _gpu(g, precision=0, div_correction=0)
    fr = float(g["freqs"][0])
    s.compute_single_frequency(fr)
    rng = np.random.default_rng(8)
    b = rng.normal(size=s.ne) + 1j * rng.normal(size=s.ne)
    b *= 1e-16 / np.linalg.norm(b)
    x = s.solve_rhs_complex(b)
    st = s.stats()
    assert st["status"][0] == BREAKDOWN and st["iterations"][0] == 1, st
    assert np.abs(x).max() == 0.0
    o = oracle.Oracle(oracle.Case.from_arrays(g, tol=1e-10, maxiter=5000, div_correction=0))
    o.solve_frequency(fr)
    xo = o.adjoint_solve(b)
    assert o.last_iters()[-1] == 1
    assert np.abs(xo).max() == 0.0
    # a right-hand side of ordinary size converges
    x2 = s.solve_rhs_complex(b * 1e16)
    assert s.stats()["status"][0] == CONVERGED
    assert rel(x2, o.adjoint_solve(b * 1e16)) < 1e-5


def test_staged_copy_wait_timeout_path(g_small):
    """With the test hook on, every slice-staged kernel gives up its copy
    wait at once: blocks skip their slices, wait (bounded) for their copies
    in flight and set the error flag; the solve fails with M3D_ERR_CUDA.
    With the hook off the same solver solves again and matches a fresh one."""
    from maple3dmt_gb300.solver import SolverError
    g = g_small
    fr = float(g["freqs"][0])
    s = _gpu(g, precision=1, row_kernels=1, bicgstab_maxiter=20)
    s.test_set_consume_no_wait(True)
    with pytest.raises(SolverError) as e:
        s.compute_single_frequency(fr)
    assert e.value.code == ERR_CUDA
    assert "timed out" in str(e.value)
    s.test_set_consume_no_wait(False)
    s.set_solver_tolerance_override(0.0)
    f = _gpu(g, precision=1, row_kernels=1, bicgstab_maxiter=20)
    assert rel(s.compute_single_frequency(fr), f.compute_single_frequency(fr)) < 1e-12
