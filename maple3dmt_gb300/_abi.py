"""ctypes declarations of the C ABI in include/m3d_mesh.h and include/m3d_gb300.h."""
from __future__ import annotations

import ctypes as C

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)


class MeshParams(C.Structure):
    """struct m3d_mesh_params (include/m3d_mesh.h)."""
    _fields_ = [
        ("domain", C.c_double * 6),
        ("min_level", C.c_int),
        ("max_level", C.c_int),
        ("station_refine_radius", C.c_double),
        ("station_refine_level", C.c_int),
        ("sigma_bg", C.c_double),
        ("max_interest_depth", C.c_double),
        ("air_surface_thickness", C.c_double),
        ("air_mid_thickness", C.c_double),
        ("air_upper_thickness", C.c_double),
        ("transition_padding", C.c_double),
        ("station_bbox", C.c_double * 4),
        ("n_regions", C.c_int),
        ("regions", c_double_p),
    ]


class Leaves(C.Structure):
    """struct m3d_leaves (include/m3d_gb300.h)."""
    _fields_ = [
        ("domain", C.c_double * 6),
        ("min_level", C.c_int),
        ("max_level", C.c_int),
        ("n_cells", C.c_int),
        ("level", c_int_p),
        ("cx", c_double_p),
        ("cy", c_double_p),
        ("cz", c_double_p),
        ("cell_type", c_int_p),
    ]


def _fn(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


def declare(lib) -> None:
    """Attach argtypes/restypes for every exported entry point present."""
    vp = C.c_void_p
    _fn(lib, "m3d_octree_build", C.c_int,
        [C.POINTER(MeshParams), c_double_p, C.c_int, c_double_p, C.c_int, C.POINTER(vp)])
    _fn(lib, "m3d_octree_num_cells", C.c_int, [vp])
    _fn(lib, "m3d_octree_get", C.c_int,
        [vp, c_int_p, c_int_p, c_double_p, c_double_p, c_double_p, c_int_p])
    _fn(lib, "m3d_octree_is_balanced", C.c_int, [vp])
    _fn(lib, "m3d_octree_destroy", None, [vp])
    _fn(lib, "m3d_layout_build", C.c_int, [C.POINTER(Leaves), C.POINTER(vp)])
    _fn(lib, "m3d_layout_destroy", None, [vp])
    _fn(lib, "m3d_layout_sizes", C.c_int, [vp, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p])
    _fn(lib, "m3d_layout_edges", C.c_int,
        [vp, c_double_p, c_double_p, c_int_p, c_double_p, c_int_p, c_int_p, c_int_p])
    _fn(lib, "m3d_layout_stiffness", C.c_int, [vp, c_int_p, c_int_p, c_double_p])
    _fn(lib, "m3d_layout_hanging", C.c_int, [vp, c_int_p])
    if hasattr(lib, "m3d_solver_create"):
        from . import _abi_solver
        _abi_solver.declare(lib)
