"""The committed leaf list of the benchmark mesh (what the CPU reference arm
of bench.py loads instead of calling the GPU library's leaf builder) expands
to exactly the builder's leaves: levels, centres and earth/air types bit for
bit, and the conductivity of the workload model on them."""
import numpy as np

from maple3dmt_gb300 import mesh, workloads
from oracle import leaflist


def test_c2_leaf_list_matches_builder(lib):
    spec = workloads.C2
    sv = mesh.layered_block_survey(min_level=spec.min_level, max_level=spec.max_level, n_side=spec.n_side,
                                   spacing=spec.spacing, freqs=np.asarray(spec.freqs))
    d = leaflist.load("c2")
    lv = sv.leaves
    assert d["domain"] == lv.domain
    assert (d["min_level"], d["max_level"]) == (lv.min_level, lv.max_level)
    assert np.array_equal(d["level"], lv.level)
    for k in ("cx", "cy", "cz"):
        assert np.array_equal(d[k], getattr(lv, k)), k
    assert np.array_equal(d["cell_type"], lv.cell_type)
    sig = workloads.cell_sigma(d["cell_type"], d["cx"], d["cy"], d["cz"], workloads.layered_block_sigma)
    assert np.array_equal(sig, sv.sigma)
