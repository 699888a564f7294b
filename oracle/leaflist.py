"""Committed leaf lists of the benchmark meshes.  TEST INFRASTRUCTURE ONLY.

The CPU reference arm of bench.py must build its mesh without the GPU
library, as the reference receives its mesh from p4est on the host.  A leaf
list (level and integer lower corner of every leaf, in leaf order) is stored
here once, written by ``make_leaves.py`` from the octree leaf builder, and
re-expanded to cell centres and earth/air types by the same arithmetic the
builder uses (p4est-style root length 2**19, centre = corner + half a cell,
flat-terrain classification of src/octree/octree_mesh.cpp:667-694 with
terrain at z = 0).  tests/test_leaflist.py checks the expansion against the
builder bit for bit.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LEAF_DIR = os.path.join(HERE, "leaves")
ROOT_LEN = 1 << 19


def path_of(name: str) -> str:
    return os.path.join(LEAF_DIR, name + ".npz")


def save(name: str, domain, min_level: int, max_level: int, level, qxyz) -> str:
    level = np.asarray(level)
    q = np.asarray(qxyz, np.int64)
    shift = 19 - int(max_level)
    if np.any(q & ((1 << shift) - 1)):
        raise ValueError("leaf corners are not on the finest grid")
    os.makedirs(LEAF_DIR, exist_ok=True)
    p = path_of(name)
    np.savez_compressed(p, domain=np.asarray(domain, np.float64), min_level=int(min_level),
                        max_level=int(max_level), level=level.astype(np.uint8),
                        q=(q >> shift).astype(np.uint16))
    return p


def load(name: str) -> dict:
    """Leaf arrays: domain, min_level, max_level, level (int32), cx, cy, cz
    (float64 centres) and cell_type (int32, 0 earth / 1 air)."""
    d = np.load(path_of(name))
    max_level = int(d["max_level"])
    level = d["level"].astype(np.int32)
    q = d["q"].astype(np.int64) << (19 - max_level)
    dom = d["domain"]
    L = (dom[1] - dom[0], dom[3] - dom[2], dom[5] - dom[4])
    ql = (ROOT_LEN >> level.astype(np.int64)).astype(np.float64)
    c = []
    for a in range(3):
        u = (q[:, a].astype(np.float64) + ql / 2.0) / float(ROOT_LEN)
        c.append(dom[2 * a] + u * L[a])
    cx, cy, cz = c
    h = (1.0 / (1 << level).astype(np.float64)) * L[2]
    below = cz + h / 2.0 < 0.0
    above = cz - h / 2.0 > 0.0
    ef = np.clip((0.0 - (cz - h / 2.0)) / h, 0.0, 1.0)
    ctype = np.where(below, 0, np.where(above, 1, np.where(ef > 0.5, 0, 1))).astype(np.int32)
    return dict(domain=tuple(float(v) for v in dom), min_level=int(d["min_level"]), max_level=max_level,
                level=level, cx=np.ascontiguousarray(cx), cy=np.ascontiguousarray(cy),
                cz=np.ascontiguousarray(cz), cell_type=ctype)
