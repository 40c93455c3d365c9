"""Resident single-amplitude mode (pq_sim_set_resident): bit-identical to the regular one-launch
path, across the kernel's idle return and relaunch, and after the mode is turned off; within
the oracle's tolerance; refused for simulators whose single amplitude is not small."""
import time

import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300 import _native as N
from polyq_gb300.rng import random_outputs, workload_many_boundaries, workload_small

pytestmark = pytest.mark.gpu


def _one_by_one(sim, xs, ys):
    vals, errs = [], []
    for x, y in zip(xs, ys):
        a, e = sim.amplitudes([x], [y], with_error=True)
        vals.append(a[0])
        errs.append(e[0])
    return np.array(vals), np.array(errs)


def test_resident_matches_regular_path(gpu):
    c = workload_small(2)
    ys = [0] + random_outputs(c.num_qubits, 23, 11)
    xs = [0] * len(ys)
    sim = Simulator(c)
    want, want_err = _one_by_one(sim, xs, ys)
    ref = O.OracleSim(c).amplitudes(xs, ys)
    assert np.all(np.abs(want - ref) <= want_err + 1e-13)

    sim.set_resident(0.05)
    got, err = _one_by_one(sim, xs, ys)
    assert np.array_equal(got, want) and np.array_equal(err, want_err)
    # the kernel returns after 50 ms without a request; the next call launches it again
    time.sleep(0.3)
    got2, err2 = _one_by_one(sim, xs[::-1], ys[::-1])
    assert np.array_equal(got2, want[::-1]) and np.array_equal(err2, want_err[::-1])
    # requests while it runs, from the Python single-amplitude call as well
    for x, y, w in zip(xs, ys, want):
        re, im = sim.amplitude(x, y)
        assert complex(re, im) == w
    # many-boundary calls keep taking the regular path while the mode is on
    many, many_err = sim.amplitudes(xs, ys, with_error=True)
    assert np.array_equal(many, want) and np.array_equal(many_err, want_err)
    sim.set_resident(0)
    got3, err3 = _one_by_one(sim, xs, ys)
    assert np.array_equal(got3, want) and np.array_equal(err3, want_err)


def test_resident_on_off_and_destroy(gpu):
    c = workload_small(2)
    sim = Simulator(c)
    want = sim.amplitudes([0], [0])[0]
    for idle in (0.02, 1.0, 0.02):
        sim.set_resident(idle)
        assert sim.amplitudes([0], [0])[0] == want
    # destroyed while the kernel is resident: the destructor stops it first
    del sim
    sim = Simulator(c)
    assert sim.amplitudes([0], [0])[0] == want


def test_resident_refused_for_large_amplitudes(gpu):
    sim = Simulator(workload_many_boundaries(0))
    with pytest.raises(N.PqError) as e:
        sim.set_resident(0.05)
    assert N.STATUS_NAMES[e.value.status] == "UNSUPPORTED"
    # the simulator keeps working on the regular path
    a, err = sim.amplitudes([0], [0], with_error=True)
    assert np.isfinite(a[0]) and err[0] >= 0
