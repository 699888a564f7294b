"""The C restatement of RegularizationOctree (oracle/m3d_oracle.c) against
the reference's own outputs (tests/golden/regularization_*.npz, made by
tests/golden/make_golden.py from the reference sources): active cells,
W^T W x, diag(W^T W), CmCm^T x, objective and gradient, bit for bit."""
import numpy as np
import pytest

from conftest import load_golden

# the fixed parameters of oracle/ref_driver.cpp
ALPHA = dict(alpha_s=1.5, alpha_x=1.0, alpha_y=0.8, alpha_z=0.5, n_smooth=2)


@pytest.mark.parametrize("name", ["regularization_small", "regularization_layered"])
def test_regularization_oracle_matches_reference(oracle_mod, name):
    g = load_golden(name)
    orc = oracle_mod.Oracle(oracle_mod.Case.from_arrays(g))
    reg = oracle_mod.Regularization(orc, **ALPHA)
    a2g = reg.active_to_global()
    assert np.array_equal(a2g, g["ref_reg_a2g"])
    x = g["ref_reg_x"]
    assert np.array_equal(reg.apply_wtw(x), g["ref_reg_wtw_x"])
    assert np.array_equal(reg.diagonal(), g["ref_reg_diag"])
    assert np.array_equal(reg.apply_cmcmt(x), g["ref_reg_cmcm_x"])
    v, grad = reg.evaluate(np.log(g["sigma"]), np.full(len(a2g), np.log(0.01)))
    assert v == g["ref_reg_eval"][0]
    assert np.array_equal(grad, g["ref_reg_grad"])
