"""Frequency groups across processes (one GPU each), after the reference's
FreqParallelManager (src/utils/freq_parallel.cpp:99-195).

Frequencies are independent until the gradient sum, so a rank solves only
the frequencies of its group and the gradient (and the misfit) are summed
over ranks: the data path has no collective, one host-side SUM per call
(freq_parallel.cpp:129, :150).  Pure Python: the solver object and the
all-reduce are passed in, so the same logic runs with the GPU solver under
torchrun and with a CPU stand-in under gloo in the tests.
"""
from __future__ import annotations

import numpy as np


def my_frequencies(n_freqs: int, group: int, n_groups: int) -> list[int]:
    """Round-robin indices of frequency group `group` (freq_parallel.cpp:117):
    group g takes g, g + G, g + 2G, ... so every group gets low (expensive)
    and high (cheap) frequencies."""
    if not (0 <= group < n_groups):
        raise ValueError("group out of range")
    return list(range(group, n_freqs, n_groups))


def gradient_step(solver, freqs, obs, err, group: int, n_groups: int, allreduce=None):
    """One inversion gradient (InversionFV::compute_gradient_,
    src/inversion/inversion_fv.cpp:230-312) over this group's frequencies.

    solver.gradient_batch(freqs, obs[:, f], err[:, f]) -> (Z [nf_g, ns, 4], g)
    allreduce(ndarray) -> ndarray sums a float64 vector over all groups (None:
    a single group).  Returns (indices of this group's frequencies, their Z,
    the gradient summed over all groups, the number of solves this group ran).
    """
    freqs = np.asarray(freqs, np.float64)
    idx = my_frequencies(len(freqs), group, n_groups)
    if idx:
        Z, g = solver.gradient_batch(freqs[idx], np.ascontiguousarray(obs[:, idx]),
                                     np.ascontiguousarray(err[:, idx]))
    else:
        Z, g = np.zeros((0, obs.shape[0], 4), np.complex128), None
    if g is None:
        g = np.zeros(solver.nc)
    if allreduce is not None and n_groups > 1:
        g = allreduce(np.ascontiguousarray(g, np.float64))
    return idx, Z, g, 4 * len(idx)
