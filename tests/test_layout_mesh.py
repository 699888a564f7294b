"""Host-side pieces of the product: octree leaf builder, layout producer, ABI."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, leaves_from_golden


def test_layout_bit_exact_with_reference(lib, golden_small):
    """StaggeredGrid + DiscreteOperators restated on the host reproduce the
    reference's edge numbering, geometry, hanging pairs and stiffness bit for bit."""
    from maple3dmt_gb300 import mesh
    g = golden_small
    L = mesh.host_layout(leaves_from_golden(g), lib=lib)
    assert np.array_equal(L["xyz"].ravel(), g["ref_edge_xyz"])
    assert np.array_equal(L["length"], g["ref_edge_len"])
    assert np.array_equal(L["direction"], g["ref_edge_dir"])
    assert np.array_equal(L["dual_area"], g["ref_edge_dual_area"])
    assert np.array_equal(L["dead"], g["ref_dead_edge"])
    assert np.array_equal(L["hanging"].ravel(), g["ref_hanging_edges"])
    assert L["n_nodes"] == int(g["ref_num_nodes"][0])
    # the reference assembles A = S + i omega Me on this pattern: the real part is S
    assert np.array_equal(L["s_ptr"], g["ref_A_rowptr"])
    assert np.array_equal(L["s_idx"], g["ref_A_colidx"])
    assert np.array_equal(L["s_val"], g["ref_A_values"].real)


def test_octree_balanced_and_morton(lib):
    from maple3dmt_gb300 import mesh
    sv = mesh.halfspace_survey(lib=lib)
    lv = sv.leaves
    assert lv.n_cells == 680
    q = lv.qxyz.astype(np.int64)

    def morton(x, y, z):
        k = 0
        for b in range(19):
            k |= ((x >> b) & 1) << (3 * b) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b + 2)
        return k
    keys = [morton(*r) for r in q]
    assert keys == sorted(keys)
    # leaves tile the root cube exactly
    vol = np.sum((2.0 ** (19 - lv.level.astype(np.float64))) ** 3)
    assert vol == float(2 ** 57)
    # earth / air split at z = 0
    assert np.all((lv.cz < 0) == (lv.cell_type == 0))


def test_octree_refines_around_stations(lib):
    from maple3dmt_gb300 import mesh
    sv = mesh.layered_block_survey(min_level=4, max_level=6, lib=lib)
    lv = sv.leaves
    near = (np.abs(lv.cx) < 3000) & (np.abs(lv.cy) < 3000) & (np.abs(lv.cz) < 2000)
    assert lv.level[near].min() == 6


def test_c2_mesh_size(lib):
    """The benchmark mesh (levels 6/7) lands in the 1-2 M edge range."""
    from maple3dmt_gb300 import mesh
    sv = mesh.layered_block_survey(min_level=6, lib=lib)
    L = mesh.host_layout(sv.leaves, lib=lib)
    assert 1_000_000 <= L["n_edges"] <= 2_000_000
    assert L["n_edges"] == 1687305


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(m3d_[a-z0-9_]+)\s*\(", txt)))


@pytest.mark.parametrize("header", ["m3d_gb300.h", "m3d_mesh.h"])
def test_library_exports_every_declared_symbol(lib, header):
    names = _declared(header)
    assert len(names) > 3
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_solver_create_without_gpu_fails_cleanly(lib):
    """Without a device the product refuses to run (no CPU fallback)."""
    import ctypes as C
    n = C.c_int(0)
    try:
        cudart = C.CDLL("libcudart.so")
        has = cudart.cudaGetDeviceCount(C.byref(n)) == 0 and n.value > 0
    except OSError:
        has = None
    h = C.c_void_p()
    rc = lib.m3d_solver_create(0, C.byref(h))
    if rc == 0:
        lib.m3d_solver_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == 5  # M3D_ERR_NO_DEVICE
    assert has in (None, False)


def test_layout_rejects_bad_leaves(lib):
    import ctypes as C
    from maple3dmt_gb300 import _abi
    s = _abi.Leaves()
    s.n_cells = 0
    h = C.c_void_p()
    assert lib.m3d_layout_build(C.byref(s), C.byref(h)) == 1
