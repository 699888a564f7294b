"""Generates tests/golden/c2_subset.npz: the reference's OWN solve (its sources
compiled unmodified into oracle/_ref by oracle/build_ref.sh) on the C2
benchmark system of bench.py, for the gradient step's frequencies that the
reference converges within its iteration cap.

C2: 0.5 ohm-m block in a 10/100/1000 ohm-m layered earth, octree levels 6/7
(1,687,305 edges, 542,144 cells; the mesh depends on all 8 frequencies),
121 stations on an 11x11 grid at 1 km, observed data = bench.py's (seeded 5 %
noise on the 100 ohm-m halfspace impedance).  The frequency subset is the
upper five of logspace(-2, 2, 8) (0.52, 1.9, 7.2, 26.8 and 100 Hz); at 0.01
and 0.037 Hz the reference's SSOR-BiCGStab does not reach 1e-7 within 5000
iterations on this mesh and 0.14 Hz takes hours of CPU.

For every frequency of the subset, one process runs the reference's
compute_single_frequency, weighted residual, adjoint sources, the two adjoint
solves and sensitivities (the per-frequency body of
InversionFV::compute_gradient_, src/inversion/inversion_fv.cpp:250-291), at
the reference's own tolerance 1e-7 and at 1e-10.  Stored: the impedances of
each frequency, the gradient summed over the subset (float32: the parity
bound is 1e-4), E1, E2, lambda1 and lambda2 at 2048 seeded edge ids, and
the digest of the leaf list the solve ran on.

    python tests/golden/make_golden_c2.py [--procs N]     (CPU hours; run where the reference tree is)
"""
from __future__ import annotations

import argparse
import hashlib
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SUBSET = (3, 4, 5, 6, 7)
TOLS = (1e-7, 1e-10)
N_SPOT = 2048


def leaves_digest(lv) -> str:
    h = hashlib.sha256()
    for a in (lv["level"], lv["cx"], lv["cy"], lv["cz"], lv["cell_type"]):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def inputs():
    from maple3dmt_gb300 import workloads
    from oracle import leaflist
    sp = workloads.C2
    lv = leaflist.load("c2")
    sigma = workloads.cell_sigma(lv["cell_type"], lv["cx"], lv["cy"], lv["cz"], workloads.layered_block_sigma)
    st = workloads.station_grid(sp.n_side, sp.spacing)
    fr = np.asarray(sp.freqs, np.float64)
    obs, err = workloads.halfspace_data(st, fr, seed=42)
    return lv, sigma, st, fr, obs, err


def one(job):
    fi, tol = job
    import oracle
    from maple3dmt_gb300 import workloads
    lv, sigma, st, fr, obs, err = inputs()
    case = oracle.Case(domain=lv["domain"], min_level=lv["min_level"], max_level=lv["max_level"],
                       level=lv["level"], cx=lv["cx"], cy=lv["cy"], cz=lv["cz"], cell_type=lv["cell_type"],
                       sigma=sigma, sigma_bg=workloads.SIGMA_BG, stations=st, freqs=fr[fi:fi + 1], tol=tol,
                       maxiter=5000, obs_Z=np.ascontiguousarray(obs[:, fi:fi + 1]),
                       obs_err=np.ascontiguousarray(err[:, fi:fi + 1]))
    t0 = time.time()
    r = oracle.run_ref(case, layout=False, forward=True, adjoint=True, log_level=2)
    dt = time.time() - t0
    spot = np.random.default_rng(1234).choice(len(r["E1"]), N_SPOT, replace=False)
    print(f"f={fr[fi]:.4g} Hz tol={tol:g}: {dt:.0f} s", flush=True)
    return dict(fi=fi, tol=tol, Z=r["Z"].reshape(-1, 4), grad=r["grad"], E1=r["E1"][spot], E2=r["E2"][spot],
                lambda1=r["lambda1"][spot], lambda2=r["lambda2"][spot], spot=spot, seconds=dt)


def main():
    import oracle
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=min(8, os.cpu_count() or 1))
    a = ap.parse_args()
    if oracle.build_ref() is None:
        raise SystemExit("reference tree not available: cannot generate the C2 fixture")
    oracle.build_oracle()
    jobs = [(fi, tol) for tol in TOLS for fi in SUBSET]
    with mp.get_context("spawn").Pool(a.procs) as pool:
        res = pool.map(one, jobs, chunksize=1)
    lv, sigma, st, fr, obs, err = inputs()
    out = dict(freq_index=np.array(SUBSET), freqs=fr[list(SUBSET)], all_freqs=fr, leaves_sha256=leaves_digest(lv),
               n_spot=N_SPOT)
    for tol in TOLS:
        tag = f"t{int(round(-np.log10(tol)))}"
        rs = sorted((r for r in res if r["tol"] == tol), key=lambda r: r["fi"])
        out[f"Z_{tag}"] = np.stack([r["Z"] for r in rs])                     # [nf_sub, ns, 4]
        out[f"grad_{tag}"] = np.sum([r["grad"] for r in rs], axis=0).astype(np.float32)
        out[f"seconds_{tag}"] = np.array([r["seconds"] for r in rs])
        for k in ("E1", "E2", "lambda1", "lambda2"):
            out[f"{k}_{tag}"] = np.stack([r[k] for r in rs])
        out["spot"] = rs[0]["spot"]
    path = os.path.join(HERE, "c2_subset.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
