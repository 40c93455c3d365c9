"""Allocation-free entry point vs the regular one, through the C-ABI on the GPU.

pq_amplitudes_noalloc serves callers that cannot allocate device memory at call time (for
example code running inside CUDA graph capture, or under an outer allocator's fixed budget):
it keeps its per-call state in a fixed static device array instead of allocating.  Two calls
in a row must each reproduce pq_amplitudes, which shows the shared scratch is reset between
calls.  This file is collected last so a failure here comes after every other test ran.
"""
import ctypes as ct

import numpy as np
import pytest

from polyq_gb300 import Simulator
from polyq_gb300 import _native as N
from polyq_gb300.rng import random_outputs, workload_many_boundaries, workload_small
from polyq_gb300.sim import pack_bits

pytestmark = pytest.mark.gpu


def _noalloc(sim, xs, ys, torch):
    n = len(ys)
    dx = torch.from_numpy(pack_bits(xs, sim.num_qubits).view(np.int64)).cuda()
    dy = torch.from_numpy(pack_bits(ys, sim.num_qubits).view(np.int64)).cuda()
    out = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = N.lib().pq_amplitudes_noalloc(sim.handle, n, ct.c_void_p(dx.data_ptr()), ct.c_void_p(dy.data_ptr()),
                                       ct.c_void_p(out.data_ptr()), None)
    N.check(st)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.complex128)


def test_noalloc_matches_regular_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    # many-boundaries workload: 16 branch engines, 64 boundaries -> 1024 jobs
    c = workload_many_boundaries(0)
    sim = Simulator(c)
    # (the entry point walks units of at most 4 chunks: results move by the grouping of chunks
    # into units, combined in FP32 pairs, far inside the stated bounds)
    for seed in (5, 6):  # two calls in a row, different boundaries
        ys = random_outputs(50, 64, seed)
        want, err = sim.amplitudes([0] * 64, ys, with_error=True)
        got = _noalloc(sim, [0] * 64, ys, torch)
        assert np.all(np.isfinite(got))
        assert np.all(np.abs(got - want) <= 1e-3 * err + 1e-15 * np.max(np.abs(want)))
    # a small circuit with vanishing boundaries in the mix
    c = workload_small(1)
    sim = Simulator(c)
    ys = [0] + random_outputs(c.num_qubits, 31, 3)
    for _ in range(2):
        want, err = sim.amplitudes([0] * 32, ys, with_error=True)
        got = _noalloc(sim, [0] * 32, ys, torch)
        assert np.all(np.abs(got - want) <= 1e-3 * err + 1e-15 * max(1e-300, np.max(np.abs(want))))


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu):
    torch = pytest.importorskip("torch")
    sim = Simulator(workload_many_boundaries(0))  # 16 branch engines: at most 256 boundaries
    with pytest.raises(N.PqError) as e:
        _noalloc(sim, [0] * 300, random_outputs(50, 300, 1), torch)
    assert e.value.status == 1
    assert "4096" in str(e.value)
