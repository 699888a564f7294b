"""The learned preconditioner in the solve (GPU, through the C ABI).

Training pairs come from the plain FP64 SSOR-BiCGStab forward solves of
seeded random layered-plus-blocks models (block resistivities log-uniform in
0.1-1000 ohm-m, sizes 0.5-5 km) on one mesh; the network is trained on the
GPU; then held-out models are solved with flexible GMRES, once with every
direction a two-level step with the network as its coarse solve and once
with the SSOR / gradient-space preconditioner alone.  Both runs stop at the
same 1e-7 FP64 true residual and must give the same impedances; the test
reports what the trained network gains in inner iterations (and the device
time of both runs) and requires fewer iterations with it.
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(lib):
    from maple3dmt_gb300 import mesh, workloads
    from maple3dmt_gb300.solver import solver_for_survey
    sv = mesh.layered_block_survey(min_level=5, max_level=6)
    lv = sv.leaves
    s = solver_for_survey(sv, bicgstab_tol=1e-7, bicgstab_maxiter=3000, precision=1, krylov=1, fgmres_m=24)
    s.learn_setup(grid_level=5, layers=6, hidden=32, seed=1, max_samples=4000)
    n = 0
    for seed in range(100, 130):
        sig = workloads.cell_sigma(lv.cell_type, lv.cx, lv.cy, lv.cz, workloads.random_layered_blocks(seed))
        s.set_sigma(sig)
        n = s.learn_collect(sv.freqs)
        if n >= 4000:
            break
    hist, val = s.learn_train(epochs=20, lr=1e-3, batch=16, seed=3, val_frac=0.1)
    print(f"pairs {n}, loss {hist[0]:.3f} -> {hist[-1]:.3f}, held-out pairs {val:.3f}")
    return sv, s, n, hist, val


def test_training_from_plain_solver(trained):
    sv, s, n, hist, val = trained
    assert n >= 500
    assert np.isfinite(hist).all()
    assert hist[-1] < 0.8 * hist[0]
    # the target has unit RMS per channel, so a zero prediction has loss
    # 0.5 x 6 channels = 3.0; the held-out pairs must be predicted well below it
    assert val < 1.5


def test_learned_fgmres_gains_on_held_out_models(trained):
    from maple3dmt_gb300 import workloads
    sv, s, *_ = trained
    lv = sv.leaves
    its = {0: 0, 1: 0}
    t_ms = {0: 0.0, 1: 0.0}
    for seed in (900, 901, 902):
        sig = workloads.cell_sigma(lv.cell_type, lv.cx, lv.cy, lv.cz, workloads.random_layered_blocks(seed))
        s.set_sigma(sig)
        Z = {}
        for period in (0, 1):
            s.set_params(learned_period=period)
            s.timer_start()
            Z[period] = s.forward_batch(sv.freqs)
            t_ms[period] += s.timer_stop()
            st = s.stats()
            tr = st["true_residual"][:st["n_rhs"]]
            assert all(t <= 1e-7 for t in tr), (period, st)
            its[period] += st["forward_iterations"]
        assert rel(Z[1], Z[0]) < 1e-5
    gain = its[0] / max(its[1], 1)
    print(f"held-out models: FGMRES inner iterations without the network {its[0]}, with it {its[1]} "
          f"({gain:.3f}x); device time {t_ms[0]:.0f} ms vs {t_ms[1]:.0f} ms")
    assert its[1] < its[0]
