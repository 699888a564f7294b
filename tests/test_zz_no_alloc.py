"""m3d_dot_batched_noalloc (no solver handle, no device allocation, fixed
scratch in a static device array) against the solver-bound m3d_dot_batched
on the same device vectors, called twice in a row each time.  Both use the
same kernel and grid, so the results agree to the last bit; the test allows
1e-12 relative.  Collected last so that it also runs after every other
GPU test."""
import ctypes as C

import numpy as np
import pytest

from conftest import leaves_from_golden, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(lib):
    fn = lib.m3d_dot_batched_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p, C.c_void_p]
    return fn


def test_noalloc_dot_matches_solver_dot(lib):
    import torch
    from maple3dmt_gb300.solver import ForwardSolverFV
    g = load_golden("small_block")
    s = ForwardSolverFV(0)
    s.setup(leaves_from_golden(g), sigma_bg=float(g["sigma_bg"]))
    fn = _noalloc(lib)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    for K in (1, 2, 4, 8, 16):
        for n in (0, 1, 1000, 300001):
            x = rng.normal(size=(n, K)) + 1j * rng.normal(size=(n, K))
            y = rng.normal(size=(n, K)) + 1j * rng.normal(size=(n, K))
            dx = torch.from_numpy(x).to("cuda:0")
            dy = torch.from_numpy(y).to("cuda:0")
            ref = torch.full((K,), complex(7.0, 7.0), dtype=torch.complex128, device="cuda:0")
            torch.cuda.synchronize()
            s.dot_batched(dx.data_ptr(), dy.data_ptr(), n, K, ref.data_ptr())
            want = ref.cpu().numpy()
            scale = max(np.abs(want).max(), 1.0)
            for _ in range(2):
                got = torch.full((K,), complex(-3.0, 5.0), dtype=torch.complex128, device="cuda:0")
                torch.cuda.synchronize()
                assert fn(dx.data_ptr(), dy.data_ptr(), n, K, got.data_ptr(), stream) == 0
                torch.cuda.synchronize()
                assert np.abs(got.cpu().numpy() - want).max() <= TOL * scale, (n, K)


def test_noalloc_dot_rejects_sizes_beyond_limit(lib):
    import torch
    fn = _noalloc(lib)
    buf = torch.zeros(64, dtype=torch.complex128, device="cuda:0")
    p = buf.data_ptr()
    assert fn(p, p, 1, 32, p, None) == 6     # M3D_ERR_TOO_LARGE: K beyond 16
    assert fn(p, p, 1, 3, p, None) == 1      # M3D_ERR_ARG: K not a power of two
    assert fn(p, p, -1, 2, p, None) == 1
    assert fn(None, p, 4, 2, p, None) == 1
