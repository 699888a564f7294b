"""C5 at scale on the GPU: the octree of levels 6/8 (about 3.1 M edges), 400
stations, a seeded random layered-plus-blocks model, 100 ohm-m starting
halfspace.  The adjoint gradient of the inversion step is checked against
central finite differences in ln sigma, as the reference's gradient check
does (examples/gradient_check_fv.cpp:192-333: eps = 1e-4, relative error
< 0.1), on four of the 24 frequencies (one per decade band) and cells near
the station array that are not station cells."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c5(lib):
    from maple3dmt_gb300 import mesh
    return mesh.c5_survey()


def test_c5_mesh_size(c5):
    from maple3dmt_gb300 import mesh
    lay = mesh.host_layout(c5.leaves)
    assert 2_000_000 <= lay["n_edges"] <= 6_000_000
    assert len(c5.stations) == 400 and len(c5.freqs) == 24


def test_c5_gradient_against_finite_differences(c5):
    from maple3dmt_gb300 import workloads
    from maple3dmt_gb300.solver import solver_for_survey
    freqs = c5.freqs[[4, 10, 16, 22]]
    s = solver_for_survey(c5, bicgstab_tol=1e-10, bicgstab_maxiter=5000, precision=1)
    s.set_sigma(c5.meta["sigma_true"])
    Zt = s.forward_batch(freqs)
    obs, err = workloads.noisy_data(Zt.transpose(1, 0, 2), seed=42)
    s.set_sigma(c5.sigma)
    Z0, grad = s.gradient_batch(freqs, obs, err)
    st = s.stats()
    assert all(t <= 1e-10 for t in st["true_residual"][:st["n_rhs"]]), st
    w = np.where(err > 0, 1.0 / np.where(err > 0, err, 1.0), 0.0)

    def misfit(sig):
        s.set_sigma(sig)
        Z = s.forward_batch(freqs)
        r = (obs - Z.transpose(1, 0, 2)) * w
        return 0.5 * float(np.sum(np.abs(r) ** 2))

    lv = c5.leaves
    st_xy = c5.stations[:, :2]
    near = ((np.abs(lv.cx) < 6000) & (np.abs(lv.cy) < 6000) & (lv.cz < 0) & (lv.cz > -4000)
            & (lv.cell_type == 0))
    cand = np.where(near)[0]
    # not a station cell (the nearest-cell interpolation makes the adjoint singular there)
    d = np.sqrt(((np.stack([lv.cx[cand], lv.cy[cand]], 1)[:, None, :] - st_xy[None]) ** 2).sum(-1)).min(1)
    h = (lv.domain[1] - lv.domain[0]) / 2.0 ** lv.level[cand]
    cand = cand[d > h]
    cells = cand[np.argsort(-np.abs(grad[cand]))[:3]]
    eps = 1e-4
    sig0 = c5.sigma.copy()
    for c in cells:
        sp = sig0.copy(); sp[c] *= math.exp(eps)
        sm = sig0.copy(); sm[c] *= math.exp(-eps)
        fd = (misfit(sp) - misfit(sm)) / (2 * eps)
        ad = grad[c]
        err_rel = abs(ad - fd) / max(abs(fd), abs(ad))
        print(f"cell {c}: adjoint {ad:.6e} fd {fd:.6e} rel {err_rel:.2e}")
        assert err_rel < 0.1, (c, ad, fd)
