"""Engine::prepare on the device, bit-exact against the oracle at full size.

prepare (src/engine.rs:569-610, with Elim::solve_into :188-201) turns a boundary into integers:
whether the (boundary, branch engine) sum vanishes, the constant phase in the u32 ring, the Z8
index k0 at the start shift (src/normal_form.rs:479-493), the particular solution's pivot bits
and the Z4 increment of every kernel coordinate.  Everything the enumeration does afterwards
depends only on these, so comparing them exactly for every job is the full-size anchor of the
amplitude path: a boundary-map or radical-solution slip on a rare bit pattern shows up here
even where an amplitude comparison on a sample would miss it.
"""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300.rng import random_outputs, workload_batch, workload_many_boundaries

pytestmark = pytest.mark.gpu


def _compare(got, want):
    assert got.shape == want.shape
    bad = np.any(got != want, axis=2)
    if bad.any():
        i, b = map(int, np.argwhere(bad)[0])
        raise AssertionError("%d of %d jobs differ; first: boundary %d engine %d\n device %s\n oracle %s"
                             % (int(bad.sum()), bad.size, i, b, got[i, b], want[i, b]))


def test_prepare_bit_exact_many_boundaries_full_size(gpu):
    # n=50, 2000 gates, 32 T (seed 0), all 4096 boundaries x 16 branch engines = 65536 jobs
    c = workload_many_boundaries(0)
    s, r = Simulator(c), O.OracleSim(c)
    ys = random_outputs(50, 4096, 1)
    got = s.prepare_info([0] * 4096, ys)
    want = r.prepare_info([0] * 4096, ys)
    assert got.shape == (4096, 16, O.PREP_WORDS)
    live = want[:, :, 0] == 0
    assert live.sum() > 10000 and (~live).sum() > 10000  # both kinds of job are exercised
    # the closed form has only even Z8 increments (odd ones are marked 0xFF by the oracle)
    lp = want[:, :, 4:].view(np.uint8)
    assert not np.any(lp == 0xFF)
    _compare(got, want)


def test_prepare_bit_exact_uneven_batch_members(gpu):
    # members of the uneven batch (n ~ U[16,64], 40n gates, T ~ U[8,36]) with their boundaries,
    # including nonzero inputs x
    circs = workload_batch(24, seed=3)
    jobs = 0
    for i, (c, _) in enumerate(circs):
        s, r = Simulator(c), O.OracleSim(c)
        ys = random_outputs(c.num_qubits, 64, 1000 + i)
        xs = [0] * 32 + random_outputs(c.num_qubits, 32, 77 + i)
        got = s.prepare_info(xs, ys)
        _compare(got, r.prepare_info(xs, ys))
        jobs += got.shape[0] * got.shape[1]
    assert jobs >= 24 * 64
