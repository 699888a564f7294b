"""The learned preconditioner's network on the tensor cores (BF16 tcgen05
implicit-GEMM convolutions, FP32 accumulation) against the CPU FP64
restatement in oracle/cnn.py: forward values, and the weight, bias and
input gradients of the backward pass (the gradient check), then training.

The GPU rounds inputs and weights to BF16 (both sides use the same rounded
values) and every intermediate activation to BF16, which the FP64
restatement does not; the tolerances are relative norms per tensor:
1e-2 for one rounded activation layer, 3e-2 through six layers, and for the
gradients 2.5e-2 through two layers, 1.2e-1 through six.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round to BF16 (nearest, ties to even) and back to float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def nrel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _net(lib, layers, c_in, hidden, c_out, seed):
    from maple3dmt_gb300.learned import Cnn
    return Cnn(layers=layers, c_in=c_in, hidden=hidden, c_out=c_out, seed=seed)


def _cpu_params(net, layers, c_in, hidden, c_out):
    w, b = net.weights()
    ci = [c_in] + [hidden] * (layers - 1)
    co = [hidden] * (layers - 1) + [c_out]
    ws = [bf16(w[l][:, :co[l], :ci[l]]) for l in range(layers)]
    bs = [b[l][:co[l]].astype(np.float64) for l in range(layers)]
    return ws, bs


@pytest.mark.parametrize("layers,grid", [(2, (1, 2, 4, 32)), (6, (2, 4, 8, 32)), (6, (1, 2, 2, 64))])
def test_forward_matches_cpu(lib, layers, grid):
    from oracle import cnn
    c_in, hidden, c_out = 8, 32, 6
    net = _net(lib, layers, c_in, hidden, c_out, seed=3)
    rng = np.random.default_rng(1)
    w, b = net.weights()
    b[:] = rng.normal(size=b.shape).astype(np.float32) * 0.1
    net.set_weights(w, b)
    x = rng.normal(size=grid + (c_in,)).astype(np.float32)
    y = net.forward(x)
    ws, bs = _cpu_params(net, layers, c_in, hidden, c_out)
    xb = bf16(x)
    want = np.stack([cnn.forward(xb[i], ws, bs)[-1] for i in range(x.shape[0])])
    e = nrel(y, want)
    print(f"layers {layers} grid {grid}: forward relative error {e:.2e}")
    assert e < (1e-2 if layers == 2 else 3e-2)


@pytest.mark.parametrize("layers,tol", [(2, 2.5e-2), (6, 1.2e-1)])
def test_backward_matches_cpu_gradients(lib, layers, tol):
    """Gradient check: dW, db and d/dx of sum(dy * net(x)) against the FP64
    restatement at the same (BF16-rounded) weights and inputs.  The GPU keeps
    activations and back-propagated gradients in BF16 (and takes the ReLU
    mask from the BF16 activation), so the error grows with depth: 2.5e-2
    through two layers, 1.2e-1 for the first layer of six."""
    from oracle import cnn
    c_in, hidden, c_out = 8, 32, 6
    net = _net(lib, layers, c_in, hidden, c_out, seed=5)
    rng = np.random.default_rng(2)
    w, b = net.weights()
    b[:] = rng.normal(size=b.shape).astype(np.float32) * 0.1
    net.set_weights(w, b)
    x = rng.normal(size=(2, 4, 8, 32, c_in)).astype(np.float32)
    dy = rng.normal(size=(2, 4, 8, 32, c_out)).astype(np.float32)
    dw, db, dx = net.backward(x, dy)
    ws, bs = _cpu_params(net, layers, c_in, hidden, c_out)
    xb = bf16(x)
    cdw = [np.zeros_like(ws[l]) for l in range(layers)]
    cdb = [np.zeros_like(bs[l]) for l in range(layers)]
    cdx = np.zeros(x.shape)
    for i in range(x.shape[0]):
        acts = cnn.forward(xb[i], ws, bs)
        gw, gb, gx = cnn.backward(acts, ws, dy[i].astype(np.float64))
        for l in range(layers):
            cdw[l] += gw[l]
            cdb[l] += gb[l]
        cdx[i] = gx
    ci = [c_in] + [hidden] * (layers - 1)
    co = [hidden] * (layers - 1) + [c_out]
    errs = []
    for l in range(layers):
        ew = nrel(dw[l][:, :co[l], :ci[l]], cdw[l])
        eb = nrel(db[l][:co[l]], cdb[l])
        print(f"layers {layers}, layer {l}: dW {ew:.2e} db {eb:.2e}")
        errs.append((l, ew, eb))
        pad_o, pad_i = dw[l][:, co[l]:, :], dw[l][:, :, ci[l]:]
        assert (pad_o.size == 0 or np.abs(pad_o).max() == 0) and (pad_i.size == 0 or np.abs(pad_i).max() == 0)
    ex = nrel(dx, cdx)
    print(f"layers {layers}: dx {ex:.2e}")
    for l, ew, eb in errs:
        assert ew < tol and eb < tol, (l, ew, eb)
    assert ex < tol


def test_training_reduces_loss(lib):
    """Adam on the tensor-core forward and backward passes fits a fixed
    teacher network's outputs on random inputs."""
    teacher = _net(lib, 3, 8, 16, 6, seed=11)
    student = _net(lib, 3, 8, 16, 6, seed=12)
    rng = np.random.default_rng(4)
    x = rng.normal(size=(4, 4, 8, 32, 8)).astype(np.float32)
    t = teacher.forward(x)
    losses = [student.train_step(x, t, lr=3e-3) for _ in range(300)]
    print(f"loss {losses[0]:.3e} -> {losses[-1]:.3e}")
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.25 * losses[0]
