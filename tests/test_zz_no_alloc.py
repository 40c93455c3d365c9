"""Allocation-free entry point vs the regular one, through the C-ABI on the GPU.

pq_amplitudes_noalloc serves callers that cannot allocate device memory when they need
amplitudes -- a process whose device memory belongs to an outer allocator with a fixed budget,
or plugin and callback code where an allocation would block or fail.  It keeps its per-call
state in a fixed static device array instead of allocating, and runs on the structures the
simulator uploaded when it was created.  Each job gets the same work shape as in the
simulator's own launch plans, so its results (and error bounds) are the same numbers as
pq_amplitudes_device's.  Two calls in a row must each reproduce them, which shows the shared
scratch is reset between calls.  This file is collected last so a failure here comes after
every other test ran.
"""
import ctypes as ct

import numpy as np
import pytest

from polyq_gb300 import Simulator
from polyq_gb300 import _native as N
from polyq_gb300.rng import random_outputs, workload_many_boundaries, workload_small
from polyq_gb300.sim import pack_bits

pytestmark = pytest.mark.gpu


def _device_call(fn, sim, xs, ys, torch, with_err=True):
    n = len(ys)
    dx = torch.from_numpy(pack_bits(xs, sim.num_qubits).view(np.int64)).cuda()
    dy = torch.from_numpy(pack_bits(ys, sim.num_qubits).view(np.int64)).cuda()
    out = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
    err = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    args = [sim.handle, n, ct.c_void_p(dx.data_ptr()), ct.c_void_p(dy.data_ptr()), ct.c_void_p(out.data_ptr()),
            ct.c_void_p(err.data_ptr()) if with_err else None, None]
    N.check(fn(*args))
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.complex128), err.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    L = N.lib()
    # many-boundaries workload: 16 branch engines, 64 boundaries -> 1024 jobs
    c = workload_many_boundaries(0)
    sim = Simulator(c)
    for seed in (5, 6):  # two calls in a row, different boundaries
        ys = random_outputs(50, 64, seed)
        want, werr = _device_call(L.pq_amplitudes_device, sim, [0] * 64, ys, torch)
        got, gerr = _device_call(L.pq_amplitudes_noalloc, sim, [0] * 64, ys, torch)
        assert np.all(np.isfinite(got)) and np.all(np.isfinite(gerr))
        # same per-job work decomposition and summation order: the same numbers
        assert np.array_equal(got, want) and np.array_equal(gerr, werr)
        host, herr = sim.amplitudes([0] * 64, ys, with_error=True)
        assert np.array_equal(got, host) and np.array_equal(gerr, herr)
    # a small circuit with vanishing boundaries in the mix, no error bound requested
    c = workload_small(1)
    sim = Simulator(c)
    ys = [0] + random_outputs(c.num_qubits, 31, 3)
    want = sim.amplitudes([0] * 32, ys)
    for _ in range(2):
        got, _ = _device_call(L.pq_amplitudes_noalloc, sim, [0] * 32, ys, torch, with_err=False)
        assert np.array_equal(got, want)


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu):
    torch = pytest.importorskip("torch")
    sim = Simulator(workload_many_boundaries(0))  # 16 branch engines: at most 256 boundaries
    with pytest.raises(N.PqError) as e:
        _device_call(N.lib().pq_amplitudes_noalloc, sim, [0] * 300, random_outputs(50, 300, 1), torch)
    assert e.value.status == 1
    assert "4096" in str(e.value)
