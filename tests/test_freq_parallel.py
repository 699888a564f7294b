"""Frequency-parallel gradient: ranks take frequencies round-robin and sum
their gradients (the reference's FreqParallelManager, src/utils/freq_parallel.cpp:99-142),
here as two gloo ranks on CPU with the oracle as the per-rank solver."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, load_golden


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out_path):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist
    import oracle
    from conftest import load_golden
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = load_golden("small_block")
    nf = g["freqs"].shape[0]
    mine = [f for f in range(nf) if f % world == rank]
    o = oracle.Oracle(oracle.Case.from_arrays(g, tol=float(g["tol"]), maxiter=int(g["maxiter"])))
    grad = np.zeros(g["level"].shape[0])
    for f in mine:
        _, gf = o.gradient(g["freqs"][f:f + 1], g["obs_Z"][:, f:f + 1], g["obs_err"][:, f:f + 1])
        grad += gf
    t = torch.from_numpy(grad)
    dist.all_reduce(t)
    if rank == 0:
        np.save(out_path, t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gradient_equals_serial(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    oracle.build_oracle()
    out = str(tmp_path / "g.npy")
    mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    g = load_golden("small_block")
    got = np.load(out)
    # serial sum over frequencies in rank order differs only by summation order
    ref = g["ref_grad"]
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
    assert torch is not None
