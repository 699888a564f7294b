"""Parity on the benchmarked configuration C2 (1,687,305 edges) against the
reference's own solve (tests/golden/c2_subset.npz, written by
make_golden_c2.py from the reference's sources compiled unmodified).

The gradient step runs through gradient_batch, the call bench.py times, on
the frequencies the reference converges within its 5000-iteration cap (0.52,
1.9, 7.2, 26.8 and 100 Hz):

* at the bench's settings (mixed precision, tolerance 1e-7) against the
  reference at its own 1e-7, and against it at 1e-10;
* at 1e-10 against the reference at 1e-10: impedances to 1e-6, the gradient
  to 1e-4 (the targets of the solver's specification).

Relative error = max |a - b| / max |b| over all stations, components and
frequencies.  The reference's own solves at 1e-7 and 1e-10 differ by about
1e-6 in Z on this mesh, which bounds what a 1e-7 solve can agree to.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel

pytestmark = pytest.mark.gpu

FIX = os.path.join(GOLDEN, "c2_subset.npz")


@pytest.fixture(scope="module")
def c2(lib):
    if not os.path.exists(FIX):
        pytest.skip("c2_subset.npz not generated")
    from maple3dmt_gb300 import mesh, workloads
    g = dict(np.load(FIX))
    sp = workloads.C2
    sv = mesh.layered_block_survey(min_level=sp.min_level, max_level=sp.max_level, n_side=sp.n_side,
                                   spacing=sp.spacing, freqs=np.asarray(sp.freqs))
    import sys
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import make_golden_c2 as mk
    lv = dict(level=sv.leaves.level, cx=sv.leaves.cx, cy=sv.leaves.cy, cz=sv.leaves.cz,
              cell_type=sv.leaves.cell_type)
    assert mk.leaves_digest(lv) == str(g["leaves_sha256"]), "mesh differs from the one the fixture was made on"
    obs, err = workloads.halfspace_data(sv.stations, sv.freqs, seed=42)
    idx = list(g["freq_index"])
    return sv, g, np.ascontiguousarray(obs[:, idx]), np.ascontiguousarray(err[:, idx])


def _errors(Z, grad, g, tag):
    eZ = rel(Z, g[f"Z_{tag}"])
    eG = rel(grad, g[f"grad_{tag}"].astype(np.float64))
    return eZ, eG


def test_c2_bench_settings_against_reference(c2):
    from maple3dmt_gb300.solver import solver_for_survey
    sv, g, obs, err = c2
    s = solver_for_survey(sv, bicgstab_tol=1e-7, bicgstab_maxiter=5000, precision=1)
    Z, grad = s.gradient_batch(g["freqs"], obs, err)
    st = s.stats()
    assert all(t <= 1e-7 for t in st["true_residual"][:st["n_rhs"]]), st
    e7 = _errors(Z, grad, g, "t7")
    e10 = _errors(Z, grad, g, "t10")
    ref_noise = rel(g["Z_t7"], g["Z_t10"])
    print(f"C2 bench settings (1e-7): Z vs reference 1e-7 {e7[0]:.2e}, vs 1e-10 {e10[0]:.2e}; "
          f"gradient {e7[1]:.2e} / {e10[1]:.2e}; reference 1e-7 vs 1e-10 in Z {ref_noise:.2e}")
    assert e10[0] < 3e-6 and e7[0] < 3e-6
    assert e10[1] < 1e-4 and e7[1] < 1e-4


def test_c2_tight_against_reference(c2):
    from maple3dmt_gb300.solver import solver_for_survey
    sv, g, obs, err = c2
    s = solver_for_survey(sv, bicgstab_tol=1e-10, bicgstab_maxiter=5000, precision=1)
    Z, grad = s.gradient_batch(g["freqs"], obs, err)
    st = s.stats()
    assert all(t <= 1e-10 for t in st["true_residual"][:st["n_rhs"]]), st
    eZ, eG = _errors(Z, grad, g, "t10")
    print(f"C2 at 1e-10: Z vs reference 1e-10 {eZ:.2e}, gradient {eG:.2e}")
    assert eZ < 1e-6
    assert eG < 1e-4
    # fields and adjoint fields at the stored edge ids, last frequency group
    spot = g["spot"]
    Zf, E = s.forward_batch(g["freqs"], with_fields=True)
    for f in range(len(g["freqs"])):
        assert rel(E[f, 0][spot], g["E1_t10"][f]) < 1e-5
        assert rel(E[f, 1][spot], g["E2_t10"][f]) < 1e-5
