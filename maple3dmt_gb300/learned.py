"""Python face of the learned preconditioner's network (include/m3d_gb300.h,
"Learned preconditioner network"): a 3-D CNN run and trained by the
library's BF16 tcgen05 kernels.  Arrays are numpy, channels last."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _loader
from .solver import SolverError


def _f(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


class Cnn:
    def __init__(self, layers=6, c_in=8, hidden=32, c_out=6, seed=0, device=0):
        self.lib = _loader.load()
        self.h = C.c_void_p()
        rc = self.lib.m3d_cnn_create(int(device), int(layers), int(c_in), int(hidden), int(c_out), int(seed),
                                     C.byref(self.h))
        if rc != 0:
            raise SolverError(rc, "m3d_cnn_create failed")
        self.layers, self.c_in, self.c_out = layers, c_in, c_out

    def close(self):
        if self.h:
            self.lib.m3d_cnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            raise SolverError(rc, (self.lib.m3d_cnn_last_error(self.h) or b"").decode())

    def weights(self):
        w = np.zeros((self.layers, 27, 32, 32), np.float32)
        b = np.zeros((self.layers, 32), np.float32)
        self._ck(self.lib.m3d_cnn_get_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)),
                                              b.ctypes.data_as(C.POINTER(C.c_float))))
        return w, b

    def set_weights(self, w, b):
        w, pw = _f(w)
        b, pb = _f(b)
        self._ck(self.lib.m3d_cnn_set_weights(self.h, pw, pb))

    def forward(self, x):
        x, px = _f(x)
        n, D, H, W = x.shape[:4]
        y = np.zeros((n, D, H, W, self.c_out), np.float32)
        self._ck(self.lib.m3d_cnn_forward(self.h, px, n, D, H, W, y.ctypes.data_as(C.POINTER(C.c_float))))
        return y

    def backward(self, x, dy, with_dx=True):
        x, px = _f(x)
        dy, pdy = _f(dy)
        n, D, H, W = x.shape[:4]
        dw = np.zeros((self.layers, 27, 32, 32), np.float32)
        db = np.zeros((self.layers, 32), np.float32)
        dx = np.zeros_like(x) if with_dx else None
        self._ck(self.lib.m3d_cnn_backward(self.h, px, pdy, n, D, H, W, dw.ctypes.data_as(C.POINTER(C.c_float)),
                                           db.ctypes.data_as(C.POINTER(C.c_float)),
                                           dx.ctypes.data_as(C.POINTER(C.c_float)) if with_dx else None))
        return dw, db, dx

    def train_step(self, x, target, lr=1e-3):
        x, px = _f(x)
        t, pt = _f(target)
        n, D, H, W = x.shape[:4]
        loss = C.c_double()
        self._ck(self.lib.m3d_cnn_train_step(self.h, px, pt, n, D, H, W, float(lr), C.byref(loss)))
        return loss.value


def _main(argv=None):
    """Runs the default network (6 layers, 32 channels, 8 -> 6 channels) on a
    batch of 16 grids of 32^3 cells: forward passes and Adam steps through the
    C ABI, wall-clock per call (host copies included).  The tensor-core
    kernels' own times come from the profiler."""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--grid", type=int, default=32)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    net = Cnn(layers=6, c_in=8, hidden=32, c_out=6, seed=1)
    rng = np.random.default_rng(0)
    g = a.grid
    x = rng.normal(size=(a.n, g, g, g, 8)).astype(np.float32)
    t = rng.normal(size=(a.n, g, g, g, 6)).astype(np.float32)
    net.forward(x)
    t0 = time.perf_counter()
    for _ in range(a.reps):
        net.forward(x)
    tf = (time.perf_counter() - t0) / a.reps
    net.train_step(x, t)
    t0 = time.perf_counter()
    for _ in range(a.reps):
        loss = net.train_step(x, t)
    tt = (time.perf_counter() - t0) / a.reps
    flop = 2.0 * a.n * g ** 3 * 32 * 27 * 32 * 6
    print(f"forward {tf * 1e3:.2f} ms, train step {tt * 1e3:.2f} ms per call (host copies included); "
          f"{flop / 1e9:.1f} GFLOP per forward; loss {loss:.3f}")


if __name__ == "__main__":
    _main()
