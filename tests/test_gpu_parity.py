"""GPU path (sm_103a, through the C ABI) against the CPU oracle and the
reference's golden outputs.

Tolerances: the GPU colours the SSOR sweeps and sums in a different order, so
iterates differ; converged results are compared.  With the solves run to
1e-10, impedances must agree to 1e-6 relative and the gradient to 1e-4
relative (the targets of the solver's specification), fields and adjoint
solutions to 1e-6.
"""
import numpy as np
import pytest

from conftest import leaves_from_golden, load_golden, rel

pytestmark = pytest.mark.gpu

Z_TOL = 1e-6
G_TOL = 1e-4
F_TOL = 1e-6


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


def _oracle(g, tol=1e-10):
    import oracle
    return oracle.Oracle(oracle.Case.from_arrays(g, tol=tol, maxiter=5000))


@pytest.fixture(scope="module")
def g_small(lib):
    return load_golden("small_block")


@pytest.mark.parametrize("gradcorr", [0, 1])
@pytest.mark.parametrize("row_kernels", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("interleaved", [0, 1])
def test_forward_matches_oracle(g_small, precision, interleaved, row_kernels, gradcorr):
    if precision == 0 and gradcorr == 1:
        pytest.skip("the gradient-space term is part of the mixed-precision solve only")
    g = g_small
    s = _gpu(g, precision=precision, forward_interleaved=interleaved, row_kernels=row_kernels, gradcorr=gradcorr)
    o = _oracle(g)
    for fr in g["freqs"]:
        Zg = s.compute_single_frequency(fr)
        st = s.stats()
        assert all(t <= 1e-8 for t in st["true_residual"][:2]), st
        Zo = o.solve_frequency(fr)
        assert rel(Zg, Zo) < Z_TOL
        for p in (0, 1):
            assert rel(s.background_E(p), o.E(p)) < F_TOL
        o.release()


@pytest.mark.parametrize("presmooth,overlap", [(0, 1), (1, 1), (0, 0)])
def test_gradient_correction_cycles_match_oracle(g_small, presmooth, overlap):
    """Both V-cycles of the gradient-space term (V(1,1), V(0,1)), on the side
    stream or on the solver's stream, give the oracle's impedances and fields
    at the 1e-10 solve."""
    g = g_small
    s = _gpu(g, precision=1, gradcorr=1, gradcorr_presmooth=presmooth, gradcorr_overlap=overlap)
    o = _oracle(g)
    for fr in g["freqs"]:
        Zg = s.compute_single_frequency(fr)
        st = s.stats()
        assert all(t <= 1e-8 for t in st["true_residual"][:2]), st
        assert rel(Zg, o.solve_frequency(fr)) < Z_TOL
        for p in (0, 1):
            assert rel(s.background_E(p), o.E(p)) < F_TOL
        o.release()


@pytest.mark.parametrize("mixed", [0, 1])
def test_divcorr_mixed_matches_reference(g_small, mixed):
    """The divergence-correction Poisson solve as FP64 PCG and as FP32 PCG
    inside FP64 refinement (both stopped at the FP64 residual 1e-10 |divJ|)
    give the reference's impedances and gradient."""
    g = g_small
    s = _gpu(g, precision=1, forward_interleaved=1, divcorr_precond=1, divcorr_mixed=mixed)
    Z, grad = s.gradient_batch(g["freqs"], g["obs_Z"], g["obs_err"])
    ns, nf = g["stations"].shape[0], g["freqs"].shape[0]
    assert rel(Z, g["ref_Z"].reshape(nf, ns, 4)) < Z_TOL
    assert rel(grad, g["ref_grad"]) < G_TOL
    assert s.stats()["divcorr_calls"] > 0


@pytest.mark.parametrize("replacement", [0, 1])
def test_residual_replacement_matches_reference(g_small, replacement):
    """The FP32 inner solve restarted per FP64 refinement and run through with
    FP64 residual replacement reach the same 1e-10 true residual and the
    reference's impedances and gradient."""
    g = g_small
    s = _gpu(g, precision=1, forward_interleaved=1, residual_replacement=replacement)
    Z, grad = s.gradient_batch(g["freqs"], g["obs_Z"], g["obs_err"])
    ns, nf = g["stations"].shape[0], g["freqs"].shape[0]
    assert rel(Z, g["ref_Z"].reshape(nf, ns, 4)) < Z_TOL
    assert rel(grad, g["ref_grad"]) < G_TOL
    st = s.stats()
    assert all(t <= 1e-10 for t in st["true_residual"][:st["n_rhs"]]), st
    if replacement:
        assert st["replacements"] > 0


def test_cuda_graph_chunks_match_direct_launches(lib):
    """The mixed-precision inner solve's 10-iteration chunks replayed from
    CUDA graphs (both streams captured; a batch shape is captured at its third
    chunk) run the same kernels in the same order as the launches issued one
    by one: bit-identical impedances and fields, the same iteration counts,
    and the replays are counted."""
    from maple3dmt_gb300 import mesh
    from maple3dmt_gb300.solver import solver_for_survey
    sv = mesh.layered_block_survey(min_level=5, max_level=6, freqs=np.array([0.1, 10.0]))
    out = {}
    for graphs in (0, 1):
        s = solver_for_survey(sv, bicgstab_tol=1e-9, bicgstab_maxiter=5000, precision=1, cuda_graphs=graphs)
        Z, E = s.forward_batch(sv.freqs, with_fields=True)
        out[graphs] = (Z, E, s.stats())
    assert out[1][2]["graphs_failed"] == 0
    assert out[1][2]["graph_replays"] > 0 and out[0][2]["graph_replays"] == 0
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2]["total_iterations"] == out[1][2]["total_iterations"]
    assert all(t <= 1e-9 for t in out[1][2]["true_residual"][:out[1][2]["n_rhs"]])


@pytest.mark.parametrize("sweep_rows,coop", [(0, 1), (16384, 0), (16384, 1)])
def test_sweep_groups_match_default_order(lib, sweep_rows, coop):
    """SSOR sweep groups (super-blocks of about sweep_rows edges, colours
    inside) and whole sweeps as one cooperative launch with grid barriers
    are other orderings of the same multicolour SSOR: at the 1e-10 solve the
    impedances match the default ordering's."""
    from maple3dmt_gb300 import mesh
    from maple3dmt_gb300.solver import solver_for_survey
    sv = mesh.layered_block_survey(min_level=5, max_level=6, freqs=np.array([0.1, 10.0]))
    base = solver_for_survey(sv, bicgstab_tol=1e-10, bicgstab_maxiter=5000, precision=1)
    assert base.ne > 4 * 16384
    Z0 = base.forward_batch(sv.freqs)
    s = solver_for_survey(sv, bicgstab_tol=1e-10, bicgstab_maxiter=5000, precision=1, sweep_rows=sweep_rows,
                          coop_sweep=coop)
    if sweep_rows:
        assert s.n_colours > base.n_colours
    Z = s.forward_batch(sv.freqs)
    st = s.stats()
    assert all(t <= 1e-10 for t in st["true_residual"][:st["n_rhs"]]), st
    assert rel(Z, Z0) < 1e-7


@pytest.mark.parametrize("relax", [0.8, 1.3])
def test_ssor_relaxation_matches_reference(g_small, relax):
    """Over- and under-relaxed SSOR in the FP32 inner solve is another
    preconditioner of the same system: the FP64 true residual still decides,
    and impedances and gradient match the reference's."""
    g = g_small
    s = _gpu(g, precision=1, forward_interleaved=1, ssor_relax=relax)
    Z, grad = s.gradient_batch(g["freqs"], g["obs_Z"], g["obs_err"])
    st = s.stats()
    assert all(t <= 1e-10 for t in st["true_residual"][:st["n_rhs"]]), st
    ns, nf = g["stations"].shape[0], g["freqs"].shape[0]
    assert rel(Z, g["ref_Z"].reshape(nf, ns, 4)) < Z_TOL
    assert rel(grad, g["ref_grad"]) < G_TOL


def test_forward_matches_reference_golden(g_small):
    g = g_small
    s = _gpu(g)
    ns, nf = g["stations"].shape[0], g["freqs"].shape[0]
    Zref = g["ref_Z"].reshape(nf, ns, 4)
    ne = s.ne
    for f, fr in enumerate(g["freqs"]):
        assert rel(s.compute_single_frequency(fr), Zref[f]) < Z_TOL
        assert rel(s.background_E(0), g["ref_E1"][f * ne:(f + 1) * ne]) < F_TOL
        assert rel(s.background_E(1), g["ref_E2"][f * ne:(f + 1) * ne]) < F_TOL


def test_halfspace_c1_against_reference(lib):
    """The CPU-runnable configuration (reference tolerance 1e-7): impedances of
    the GPU solve to the reference's within the solver-noise floor."""
    g = load_golden("halfspace_c1")
    s = _gpu(g, bicgstab_tol=1e-7)
    Zg = s.compute_single_frequency(float(g["freqs"][0]))
    Zref = g["ref_Z"].reshape(-1, 4)
    assert rel(Zg[:, 1:3], Zref[:, 1:3]) < 1e-5


def test_halfspace_c1_tight_against_reference(lib):
    """C1 with both solves at 1e-10: all four impedance components of the GPU
    solve agree with the reference's to 1e-6 relative (max |dZ| / max |Z|),
    in FP64 and in mixed precision."""
    g = load_golden("halfspace_c1_t10")
    Zref = g["ref_Z"].reshape(-1, 4)
    for precision in (0, 1):
        s = _gpu(g, bicgstab_tol=1e-10, precision=precision)
        Zg = s.compute_single_frequency(float(g["freqs"][0]))
        st = s.stats()
        assert all(t <= 1e-10 for t in st["true_residual"][:2]), st
        e = rel(Zg, Zref)
        print(f"C1 at 1e-10, precision {precision}: Z relative error {e:.2e}")
        assert e < 1e-6


def test_adjoint_pieces_match_oracle(g_small):
    g = g_small
    s = _gpu(g)
    o = _oracle(g)
    fr = g["freqs"][0]
    s.compute_single_frequency(fr)
    o.solve_frequency(fr)
    rng = np.random.default_rng(5)
    wr = rng.normal(size=(s.ns, 4)) + 1j * rng.normal(size=(s.ns, 4))
    a1g, a2g = s.build_adjoint_rhs_from_residual(wr)
    a1o, a2o = o.adjoint_rhs(wr)
    assert rel(a1g, a1o) < F_TOL and rel(a2g, a2o) < F_TOL
    lg = s.adjoint_solve_complex(a1o)
    lo = o.adjoint_solve(a1o)
    assert rel(lg, lo) < 1e-5
    E0 = o.E(0)
    assert rel(s.compute_sensitivity_complex(E0, lo), o.sensitivity(E0, lo)) < 1e-12


def test_jv_pieces_match_oracle(g_small):
    """J.v pieces: perturbation source, solve_rhs and delta impedances."""
    g = g_small
    s = _gpu(g)
    o = _oracle(g)
    fr = g["freqs"][1]
    s.compute_single_frequency(fr)
    o.solve_frequency(fr)
    rng = np.random.default_rng(9)
    dsig = np.where(g["cell_type"] == 0, rng.normal(size=g["sigma"].shape) * 1e-3, 0.0)
    for pol in (1, 2):
        pg = s.build_perturbation_rhs_complex(pol, dsig)
        po = o.perturbation_rhs(pol, dsig)
        assert rel(pg, po) < 1e-8   # the background fields differ at the 1e-10 solve tolerance
    xg = s.solve_rhs_complex(po)
    xo = o.adjoint_solve(po)
    assert rel(xg, xo) < 1e-5
    for pol in (1, 2):
        assert rel(s.extract_delta_impedance_complex(xo, pol), o.delta_impedance(xo, pol)) < 1e-8


@pytest.mark.parametrize("gradcorr", [0, 1])
@pytest.mark.parametrize("ssor_form", [0, 1])
@pytest.mark.parametrize("divcorr_precond", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_gradient_batch_matches_reference(g_small, precision, divcorr_precond, ssor_form, gradcorr):
    """Against the reference's own outputs; both PCG preconditioners of the
    divergence correction (Jacobi as the reference, aggregation multigrid)
    stop at the same 1e-10 relative residual, and both forms of the FP32
    SSOR-BiCGStab (right-preconditioned as the reference, Eisenstat split),
    with and without the gradient-space term of the preconditioner, are
    driven to the same FP64 true residual."""
    if precision == 0 and (ssor_form == 1 or gradcorr == 1):
        pytest.skip("the split form and the gradient-space term belong to the mixed-precision solve")
    if gradcorr == 1 and ssor_form == 1:
        pytest.skip("batches with the gradient-space term run the right-preconditioned form")
    g = g_small
    s = _gpu(g, precision=precision, forward_interleaved=1, divcorr_precond=divcorr_precond, ssor_form=ssor_form,
             gradcorr=gradcorr)
    Z, grad = s.gradient_batch(g["freqs"], g["obs_Z"], g["obs_err"])
    ns, nf = g["stations"].shape[0], g["freqs"].shape[0]
    assert rel(Z, g["ref_Z"].reshape(nf, ns, 4)) < Z_TOL
    assert rel(grad, g["ref_grad"]) < G_TOL


def test_jtjv_batch_matches_oracle(g_small):
    """Batched GN-CG product J^T W^2 J dsigma against the reference's
    ImplicitJtJOperatorFV::Mult composed from the oracle's single-frequency
    pieces (perturbation RHS, solve, delta Z, w^2 weighting, adjoint source of
    the same polarisation, adjoint solve, sensitivity), both at 1e-10."""
    g = g_small
    s = _gpu(g, precision=1)
    freqs = g["freqs"]
    s.forward_batch(freqs)
    rng = np.random.default_rng(5)
    earth = g["cell_type"] == 0
    dsig = np.where(earth, g["sigma"] * 0.1 * rng.normal(size=g["sigma"].shape), 0.0)
    err = np.ascontiguousarray(g["obs_err"])
    y = s.jtjv_batch(freqs, dsig, err, inner_tol=1e-10)
    o = _oracle(g)
    yo = np.zeros_like(y)
    for f, fr in enumerate(freqs):
        o.solve_frequency(fr)
        e = err[:, f, :]
        w2 = np.where(e > 0, 1.0 / np.where(e > 0, e, 1.0) ** 2, 0.0)
        for p in (0, 1):
            dE = o.adjoint_solve(o.perturbation_rhs(p + 1, dsig))
            a1, a2 = o.adjoint_rhs(w2 * o.delta_impedance(dE, p + 1))
            lam = o.adjoint_solve(a1 if p == 0 else a2)
            yo += o.sensitivity(o.E(p), lam)
        o.release()
    assert np.linalg.norm(yo) > 0
    assert rel(y, yo) < G_TOL
    # linear in dsigma
    y2 = s.jtjv_batch(freqs, 2.0 * dsig, err, inner_tol=1e-10)
    assert rel(y2, 2.0 * y) < 1e-6
    # needs the background fields of the same frequencies
    from maple3dmt_gb300.solver import SolverError
    with pytest.raises(SolverError) as ex:
        s.jtjv_batch(freqs[:1], dsig, np.ascontiguousarray(err[:, :1, :]))
    assert ex.value.code == 2


def test_sigma_update_matches_fresh_solver(g_small):
    """Line-search trial steps (inversion_fv.cpp:427-436): a conductivity
    update keeps the layout, colouring, segments and multigrid aggregates and
    re-assembles only the values; its impedances match a solver set up from
    scratch for the new conductivity, and the original conductivity set
    again reproduces the first result."""
    g = g_small
    s = _gpu(g, precision=1)
    Z1 = s.forward_batch(g["freqs"])
    earth = g["cell_type"] == 0
    sig2 = np.where(earth, g["sigma"] * np.exp(0.3 * np.random.default_rng(7).normal(size=g["sigma"].shape)),
                    g["sigma"])
    s.set_sigma(sig2)
    Z2 = s.forward_batch(g["freqs"])
    f = _gpu(g, precision=1)
    f.set_sigma(sig2)
    assert rel(Z2, f.forward_batch(g["freqs"])) < Z_TOL
    assert rel(Z2, Z1) > 10 * Z_TOL
    s.set_sigma(g["sigma"])
    assert rel(s.forward_batch(g["freqs"]), Z1) < Z_TOL


def test_batch_equals_single_frequency(g_small):
    g = g_small
    s = _gpu(g)
    Zb, Eb = s.forward_batch(g["freqs"], with_fields=True)
    for f, fr in enumerate(g["freqs"]):
        assert rel(s.compute_single_frequency(fr), Zb[f]) < 1e-8
        assert rel(s.background_E(1), Eb[f, 1]) < 1e-8


def test_error_codes(g_small):
    from maple3dmt_gb300.solver import SolverError
    g = g_small
    s = _gpu(g)
    with pytest.raises(SolverError) as e:
        s.set_sigma(g["sigma"][:-1])
    assert e.value.code == 1
    with pytest.raises(SolverError) as e:
        s.build_adjoint_rhs_from_residual(np.zeros((s.ns, 4)))
    assert e.value.code == 2
    bad = g["sigma"].copy()
    bad[0] = -1.0
    with pytest.raises(SolverError):
        s.set_sigma(bad)
    with pytest.raises(SolverError) as e:
        s.compute_single_frequency(-1.0)
    assert e.value.code == 1


def test_solve_rhs_batch_equals_single_solves(g_small):
    """Twenty right-hand sides at one frequency (two launch groups of up to 16)
    give the single solve_rhs results."""
    g = g_small
    s = _gpu(g)
    s.compute_single_frequency(g["freqs"][0])
    rng = np.random.default_rng(11)
    B = rng.normal(size=(20, s.ne)) + 1j * rng.normal(size=(20, s.ne))
    X = s.solve_rhs_batch(B)
    for k in (0, 7, 15, 16, 19):
        assert rel(X[k], s.solve_rhs_complex(B[k])) < 1e-8


def test_solution_linear_in_rhs(g_small):
    """Size-independent property: x(b1 + 2 b2) = x(b1) + 2 x(b2) to solver tolerance."""
    g = g_small
    s = _gpu(g)
    s.compute_single_frequency(g["freqs"][0])
    rng = np.random.default_rng(2)
    b1 = rng.normal(size=s.ne) + 1j * rng.normal(size=s.ne)
    b2 = rng.normal(size=s.ne) + 1j * rng.normal(size=s.ne)
    x1, x2, x3 = (s.solve_rhs_complex(b) for b in (b1, b2, b1 + 2 * b2))
    assert rel(x3, x1 + 2 * x2) < 1e-6


def test_c2_scale_true_residual(lib):
    """Full-size mesh (1.69 M edges): the two highest frequencies, mixed
    precision, both polarisations reach the 1e-7 true relative residual."""
    from maple3dmt_gb300 import mesh
    from maple3dmt_gb300.solver import solver_for_survey
    sv = mesh.layered_block_survey(min_level=6)     # the mesh depends on the full frequency set
    s = solver_for_survey(sv, bicgstab_tol=1e-7, bicgstab_maxiter=5000, precision=1, forward_interleaved=1)
    Z = s.forward_batch(sv.freqs[-2:])
    st = s.stats()
    assert s.ne == 1687305
    assert np.isfinite(Z).all()
    assert all(t <= 1e-7 for t in st["true_residual"][:4]), st


def test_c2_scale_divcorr_preconditioners_agree(lib):
    """Full-size mesh, the two highest frequencies, the reference's forward
    strategy (BiCGStab to 1e-7, then the divergence correction): impedances
    with the multigrid-preconditioned PCG agree with the Jacobi PCG (the
    reference's) to 1e-5 relative -- both solves stop at the 1e-7 true
    residual and both PCGs at 1e-10, so Z differs at the solve tolerance, not
    more.  (At 0.01 Hz this strategy does not converge on this mesh without
    the interleaved divergence correction; the interleaved strategy is the
    one the gradient runs.)"""
    from maple3dmt_gb300 import mesh
    from maple3dmt_gb300.solver import solver_for_survey
    sv = mesh.layered_block_survey(min_level=6)
    Zs = []
    for pc in (0, 1):
        s = solver_for_survey(sv, bicgstab_tol=1e-7, bicgstab_maxiter=5000, precision=1, forward_interleaved=0,
                              divcorr_precond=pc)
        Zs.append(s.forward_batch(sv.freqs[-2:]))
        st = s.stats()
        assert all(t <= 1e-7 for t in st["true_residual"][:4]), st
        s.close()
    assert rel(Zs[1], Zs[0]) < 1e-5


def test_c2_scale_gradient_correction_low_frequency(lib):
    """Full-size mesh at 0.01 Hz, both polarisations: with the gradient-space
    term the reference's forward strategy (BiCGStab to 1e-7, then the
    divergence correction) converges in a small fraction of the iterations
    that SSOR alone needs with interleaved corrections, and the impedances of
    the two agree to 1e-5 relative (both solves stop at the 1e-7 FP64 true
    residual)."""
    from maple3dmt_gb300 import mesh
    from maple3dmt_gb300.solver import solver_for_survey
    sv = mesh.layered_block_survey(min_level=6)
    runs = []
    for gc, inter in ((0, 1), (1, 0)):
        s = solver_for_survey(sv, bicgstab_tol=1e-7, bicgstab_maxiter=5000, precision=1, forward_interleaved=inter,
                              gradcorr=gc)
        Z = s.forward_batch(sv.freqs[:1])
        st = s.stats()
        assert all(t <= 1e-7 for t in st["true_residual"][:2]), st
        runs.append((Z, st["iterations"][:2]))
        s.close()
    (Z0, it0), (Z1, it1) = runs
    assert max(it1) * 4 < min(it0), (it0, it1)
    assert rel(Z1, Z0) < 1e-5


@pytest.mark.parametrize("K", [1, 2, 4, 8, 16])
def test_dot_batched_matches_numpy(g_small, K):
    """Batched Hermitian dot of device vectors (the BiCGStab dot for K
    systems): FP64 sums in a different order, so 1e-12 relative."""
    import torch
    from maple3dmt_gb300.solver import SolverError
    s = _gpu(g_small)
    rng = np.random.default_rng(K)
    for n in (0, 1, 1000, 300001):
        x = rng.normal(size=(n, K)) + 1j * rng.normal(size=(n, K))
        y = rng.normal(size=(n, K)) + 1j * rng.normal(size=(n, K))
        dx = torch.from_numpy(x).to("cuda:0")
        dy = torch.from_numpy(y).to("cuda:0")
        out = torch.full((K,), complex(7.0, 7.0), dtype=torch.complex128, device="cuda:0")
        torch.cuda.synchronize()
        s.dot_batched(dx.data_ptr(), dy.data_ptr(), n, K, out.data_ptr())
        want = (np.conj(x) * y).sum(axis=0)
        got = out.cpu().numpy()
        assert np.abs(got - want).max() <= 1e-12 * max(np.abs(want).max(), 1.0), (n, K)
    with pytest.raises(SolverError) as e:
        s.dot_batched(dx.data_ptr(), dy.data_ptr(), 10, 3, out.data_ptr())
    assert e.value.code == 1


@pytest.mark.parametrize("name", ["regularization_small", "regularization_layered"])
def test_regularization_matches_reference(lib, name):
    """RegularizationOctree on the GPU against the reference's own outputs
    (tests/golden/regularization_*.npz): active cells, W^T W x, diag(W^T W)
    and CmCm^T x and the gradient bit for bit (rounded operation by operation in
    the reference's order), the objective to 1e-13 (block-reduced dot)."""
    g = load_golden(name)
    s = _gpu(g)
    na = s.reg_setup(alpha_s=1.5, alpha_x=1.0, alpha_y=0.8, alpha_z=0.5, n_smooth=2)
    assert na == len(g["ref_reg_a2g"])
    assert np.array_equal(s.reg_active_to_global(), g["ref_reg_a2g"])
    x = g["ref_reg_x"]
    assert np.array_equal(s.reg_apply_wtw(x), g["ref_reg_wtw_x"])
    assert np.array_equal(s.reg_diagonal_wtw(), g["ref_reg_diag"])
    assert np.array_equal(s.reg_apply_cmcmt(x), g["ref_reg_cmcm_x"])
    v, grad = s.reg_evaluate(np.log(g["sigma"]), np.full(na, np.log(0.01)))
    assert abs(v - g["ref_reg_eval"][0]) <= 1e-13 * abs(g["ref_reg_eval"][0])
    assert np.array_equal(grad, g["ref_reg_grad"])
