"""Writes the committed leaf lists of oracle/leaves/ from the octree leaf
builder (run where the GPU library is built; the leaf builder is host code):

    python oracle/make_leaves.py            # every benchmark mesh

c2: the C2 mesh of bench.py (layered earth + block, levels 6/7, 11x11
stations at 1 km, 8 frequencies 0.01-100 Hz).
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from maple3dmt_gb300 import mesh, workloads  # noqa: E402
from oracle import leaflist  # noqa: E402


def survey(name):
    spec = {"c2": workloads.C2}[name]
    import numpy as np
    return mesh.layered_block_survey(min_level=spec.min_level, max_level=spec.max_level, n_side=spec.n_side,
                                     spacing=spec.spacing, freqs=np.asarray(spec.freqs))


def main(names):
    for name in names:
        lv = survey(name).leaves
        p = leaflist.save(name, lv.domain, lv.min_level, lv.max_level, lv.level, lv.qxyz)
        print(name, lv.n_cells, "cells", os.path.getsize(p), "bytes")


if __name__ == "__main__":
    main(sys.argv[1:] or ["c2"])
