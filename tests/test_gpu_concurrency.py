"""The reference's Simulator is Sync and amplitude is callable from many threads at once
(src/sim.rs, src/pybind.rs).  Calls from several host threads on one simulator, and on
different simulators, give the same bits as one thread does."""
import threading

import numpy as np
import pytest

from polyq_gb300 import Simulator
from polyq_gb300.rng import Rng, random_clifford_t, random_outputs, workload_small

pytestmark = pytest.mark.gpu


def test_threads_share_a_simulator(gpu):
    c = workload_small(2)
    sim = Simulator(c)
    others = [Simulator(random_clifford_t(10, 80, 10, False, Rng(s))) for s in (1, 2)]
    work = [(sim, random_outputs(20, 16 + i, 40 + i)) for i in range(4)]
    work += [(o, random_outputs(10, 8, 50 + k)) for k, o in enumerate(others)]
    want = [s.amplitudes([0] * len(ys), ys) for s, ys in work]
    got = [None] * len(work)
    errors = []

    def run(i):
        try:
            s, ys = work[i]
            for _ in range(20):
                a = s.amplitudes([0] * len(ys), ys)
                if got[i] is None:
                    got[i] = a
                elif not np.array_equal(a, got[i]):
                    errors.append(i)
        except Exception as e:  # pragma: no cover - reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(work))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(120)
    assert not errors
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
