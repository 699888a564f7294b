"""The CPU oracle (C restatement) against the reference's own outputs.

The golden fixtures were produced by the reference's solver sources compiled
unmodified (tests/golden/make_golden.py); the restatement must reproduce them
bit for bit, which pins it before it is used as the checker of the GPU path.
"""
import math

import numpy as np
import pytest

from conftest import rel


def _case(oracle_mod, g, **kw):
    return oracle_mod.Case.from_arrays(g, tol=float(g["tol"]), maxiter=int(g["maxiter"]),
                                       obs_Z=g["obs_Z"], obs_err=g["obs_err"], **kw)


@pytest.mark.parametrize("name", ["small_block", "halfspace_c1"])
def test_oracle_gradient_bit_exact(oracle_mod, name):
    from conftest import load_golden
    g = load_golden(name)
    o = oracle_mod.Oracle(_case(oracle_mod, g))
    Z, grad = o.gradient(g["freqs"], g["obs_Z"], g["obs_err"])
    ns, nf = g["stations"].shape[0], g["freqs"].shape[0]
    assert np.array_equal(Z, g["ref_Z"].reshape(nf, ns, 4))
    assert np.array_equal(grad, g["ref_grad"])


def test_oracle_fields_bit_exact(oracle_mod, golden_small):
    g = golden_small
    o = oracle_mod.Oracle(_case(oracle_mod, g))
    ne = o.ne
    for f, fr in enumerate(g["freqs"]):
        o.solve_frequency(fr)
        assert np.array_equal(o.E(0), g["ref_E1"][f * ne:(f + 1) * ne])
        assert np.array_equal(o.E(1), g["ref_E2"][f * ne:(f + 1) * ne])
        o.release()


def test_oracle_adjoint_pieces_bit_exact(oracle_mod, golden_small):
    g = golden_small
    o = oracle_mod.Oracle(_case(oracle_mod, g))
    ne, ns, nf = o.ne, g["stations"].shape[0], g["freqs"].shape[0]
    Z = o.solve_frequency(g["freqs"][0])
    w = np.where(g["obs_err"][:, 0, :] > 0, 1.0 / np.where(g["obs_err"][:, 0, :] > 0, g["obs_err"][:, 0, :], 1), 0)
    wr = w * w * np.conj(g["obs_Z"][:, 0, :] - Z)
    wr[g["obs_err"][:, 0, :] <= 0] = 0
    a1, a2 = o.adjoint_rhs(wr)
    assert np.array_equal(a1, g["ref_adj_rhs1"][:ne])
    assert np.array_equal(a2, g["ref_adj_rhs2"][:ne])
    l1 = o.adjoint_solve(a1)
    assert np.array_equal(l1, g["ref_lambda1"][:ne])
    assert nf == 2


def test_oracle_layout_matches_reference(oracle_mod, golden_small):
    g = golden_small
    o = oracle_mod.Oracle(_case(oracle_mod, g))
    ed = o.edges()
    assert np.array_equal(ed["xyz"].ravel(), g["ref_edge_xyz"])
    assert np.array_equal(ed["len"], g["ref_edge_len"])
    assert np.array_equal(ed["dir"], g["ref_edge_dir"])
    assert np.array_equal(ed["adual"], g["ref_edge_dual_area"])
    assert np.array_equal(ed["dead"], g["ref_dead_edge"])


def test_halfspace_known_answer(oracle_mod, golden_c1):
    """Analytic 1-D halfspace impedance (examples/halfspace_1d_test.cpp:123-187):
    apparent resistivity within 25 % of 100 ohm-m and phase within 15 degrees
    of the halfspace value (45 deg for Zxy with this code's sign convention)."""
    g = golden_c1
    f = float(g["freqs"][0])
    Z = g["ref_Z"].reshape(-1, 4)
    om = 2 * math.pi * f
    mu0 = 4e-7 * math.pi
    for comp, ph_ref in ((1, 45.0), (2, -135.0)):
        rho = np.abs(Z[:, comp]) ** 2 / (om * mu0)
        ph = np.angle(Z[:, comp], deg=True)
        assert np.all((rho > 75) & (rho < 125)), rho
        assert np.all(np.abs(ph - ph_ref) < 15), ph


def test_oracle_converges_to_tolerance(oracle_mod, golden_small):
    """Both polarisations of both frequencies reach the 1e-10 tolerance in the oracle."""
    g = golden_small
    o = oracle_mod.Oracle(_case(oracle_mod, g))
    o.solve_frequency(g["freqs"][1])
    its = o.last_iters()
    assert len(its) == 2 and all(0 < i < int(g["maxiter"]) for i in its)


def test_oracle_fd_gradient(oracle_mod, golden_small):
    """Adjoint gradient against central finite differences in ln sigma
    (examples/gradient_check_fv.cpp:192-333: eps 1e-4, rel < 0.1 or abs tiny)."""
    g = golden_small
    freqs = g["freqs"][:1]
    obs, err = g["obs_Z"][:, :1], g["obs_err"][:, :1]
    base = oracle_mod.Case.from_arrays(g, tol=1e-12, maxiter=5000)
    o = oracle_mod.Oracle(base)
    _, grad = o.gradient(freqs, obs, err)
    sigma0 = np.array(g["sigma"])

    def misfit(sig):
        c = oracle_mod.Case.from_arrays({**g, "sigma": sig}, tol=1e-12, maxiter=5000)
        oo = oracle_mod.Oracle(c)
        Z, _ = oo.gradient(freqs, obs, err)
        w = np.where(err > 0, 1.0 / np.where(err > 0, err, 1.0), 0.0)
        r = (obs - Z.transpose(1, 0, 2)) * w
        return 0.5 * float(np.sum(np.abs(r) ** 2))

    earth = np.where(g["cell_type"] == 0)[0]
    # cells near the station array, below the surface
    cand = [c for c in earth if abs(g["cx"][c]) < 4000 and abs(g["cy"][c]) < 4000 and -3000 < g["cz"][c] < 0]
    eps = 1e-4
    checked = 0
    for c in cand[:3]:
        sp = sigma0.copy(); sp[c] *= math.exp(eps)
        sm = sigma0.copy(); sm[c] *= math.exp(-eps)
        fd = (misfit(sp) - misfit(sm)) / (2 * eps)
        # the reference's gradient is d(0.5 * sum |W r|^2)/d ln sigma with the
        # sign convention of compute_gradient_ (inversion_fv.cpp:258-288)
        ad = grad[c]
        ok = abs(ad - fd) <= 0.1 * max(abs(fd), 1e-12) or abs(ad - fd) < 1e-4 * max(1.0, abs(fd))
        assert ok, (c, ad, fd)
        checked += 1
    assert checked > 0
