"""Generates the golden fixtures of tests/golden from the reference's OWN
solver sources (compiled unmodified into oracle/_ref by oracle/build_ref.sh).

Run in a checkout where the reference tree is available:
    python tests/golden/make_golden.py
Each fixture stores the inputs of a case (leaf list, conductivity, stations,
frequencies, observed data) and the reference's outputs for it: staggered-grid
edge geometry, the stiffness pattern and values, the hanging pairs, E1/E2,
impedances, adjoint sources, adjoint fields and the gradient.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from maple3dmt_gb300 import mesh  # noqa: E402


def observed(sv, seed):
    rng = np.random.default_rng(seed)
    ns, nf = len(sv.stations), len(sv.freqs)
    om = 2 * np.pi * sv.freqs
    z1 = np.sqrt(1j * om * mesh.MU0 / 0.01)
    obs = np.zeros((ns, nf, 4), np.complex128)
    obs[:, :, 1] = z1[None, :]
    obs[:, :, 2] = -z1[None, :]
    obs += 0.05 * np.abs(z1)[None, :, None] * (rng.normal(size=(ns, nf, 4)) + 1j * rng.normal(size=(ns, nf, 4)))
    err = np.full((ns, nf, 4), 0.05) * np.abs(z1)[None, :, None]
    err[:, :, 0] = 0.0   # Zxx carries no weight, as unset components in the reference
    return obs, err


def make(name, sv, tol, maxiter, seed, layout=True):
    obs, err = observed(sv, seed)
    case = oracle.Case.from_survey(sv, tol=tol, maxiter=maxiter, obs_Z=obs, obs_err=err)
    r = oracle.run_ref(case, layout=layout, forward=True, adjoint=True)
    lv = sv.leaves
    out = dict(domain=np.array(lv.domain), min_level=lv.min_level, max_level=lv.max_level, level=lv.level,
               cx=lv.cx, cy=lv.cy, cz=lv.cz, cell_type=lv.cell_type, sigma=sv.sigma, sigma_bg=sv.sigma_bg,
               stations=sv.stations, freqs=sv.freqs, obs_Z=obs, obs_err=err, tol=tol, maxiter=maxiter)
    keys = ["E1", "E2", "Z", "adj_rhs1", "adj_rhs2", "lambda1", "lambda2", "grad"]
    if layout:
        keys += ["edge_xyz", "edge_len", "edge_dir", "edge_dual_area", "dead_edge", "hanging_edges",
                 "A_rowptr", "A_colidx", "A_values", "num_nodes"]
    for k in keys:
        out["ref_" + k] = r[k]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(name, os.path.getsize(path), "bytes")


def make_regularization(name, sv):
    """RegularizationOctree outputs of the reference (fixed parameters in
    oracle/ref_driver.cpp): active cells, W^T W x, CmCm^T x, diag(W^T W),
    the objective and its gradient."""
    case = oracle.Case.from_survey(sv)
    r = oracle.run_ref(case, layout=False, forward=False, adjoint=False, regularization=True)
    lv = sv.leaves
    out = dict(domain=np.array(lv.domain), min_level=lv.min_level, max_level=lv.max_level, level=lv.level,
               cx=lv.cx, cy=lv.cy, cz=lv.cz, cell_type=lv.cell_type, sigma=sv.sigma, sigma_bg=sv.sigma_bg,
               stations=sv.stations, freqs=sv.freqs)
    for k in ("reg_a2g", "reg_x", "reg_wtw_x", "reg_cmcm_x", "reg_diag", "reg_eval", "reg_grad"):
        out["ref_" + k] = r[k]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(name, os.path.getsize(path), "bytes")


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference tree not available: cannot regenerate golden fixtures")
    # a small mesh with hanging faces and a conductive block, 2 frequencies
    make("small_block", mesh.small_survey(freqs=(0.5, 4.0)), tol=1e-10, maxiter=5000, seed=1)
    # the CPU-runnable halfspace configuration (5x5 stations, 1 Hz), at the
    # reference's own tolerance 1e-7
    make("halfspace_c1", mesh.halfspace_survey(), tol=1e-7, maxiter=5000, seed=2, layout=False)
    # the same at 1e-10, below the solver-noise floor of the 1e-7 solve
    make("halfspace_c1_t10", mesh.halfspace_survey(), tol=1e-10, maxiter=5000, seed=2, layout=False)
    # octree regularisation on the small mesh and on a 4/6-level layered mesh
    make_regularization("regularization_small", mesh.small_survey(freqs=(0.5, 4.0)))
    make_regularization("regularization_layered", mesh.layered_block_survey(min_level=4, max_level=6))


if __name__ == "__main__":
    main()
