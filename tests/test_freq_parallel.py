"""Frequency-parallel gradient: ranks take frequencies round-robin and sum
their gradients (the reference's FreqParallelManager, src/utils/freq_parallel.cpp:99-142).
The product's partition and reduction logic (maple3dmt_gb300.freq_parallel,
what bench.py runs under torchrun) runs here as two and three gloo ranks on
CPU, with the oracle standing in for the per-rank GPU solver."""
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
    from maple3dmt_gb300 import freq_parallel
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = load_golden("small_block")
    o = oracle.Oracle(oracle.Case.from_arrays(g, tol=float(g["tol"]), maxiter=int(g["maxiter"])))

    class OracleSolver:            # the GPU solver's gradient_batch face
        nc = o.nc

        @staticmethod
        def gradient_batch(freqs, obs, err):
            return o.gradient(freqs, obs, err)

    def allreduce(v):
        t = torch.from_numpy(v)
        dist.all_reduce(t)
        return t.numpy()

    idx, Z, grad, solves = freq_parallel.gradient_step(OracleSolver, g["freqs"], g["obs_Z"], g["obs_err"],
                                                       rank, world, allreduce)
    assert idx == freq_parallel.my_frequencies(len(g["freqs"]), rank, world)
    assert Z.shape[0] == len(idx) and solves == 4 * len(idx)
    if rank == 0:
        np.save(out_path, grad)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_multi_rank_gradient_equals_serial(tmp_path, world):
    """Two ranks (one frequency each) and three ranks (one rank without a
    frequency) both give the reference's full gradient."""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    oracle.build_oracle()
    out = str(tmp_path / "g.npy")
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    g = load_golden("small_block")
    got = np.load(out)
    # serial sum over frequencies in rank order differs only by summation order
    ref = g["ref_grad"]
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
    assert torch is not None


def test_round_robin_groups():
    from maple3dmt_gb300.freq_parallel import my_frequencies
    groups = [my_frequencies(81, g, 8) for g in range(8)]
    assert groups[0] == list(range(0, 81, 8)) and len(groups[0]) == 11 and len(groups[7]) == 10
    assert sorted(i for gr in groups for i in gr) == list(range(81))
    with pytest.raises(ValueError):
        my_frequencies(8, 2, 2)
