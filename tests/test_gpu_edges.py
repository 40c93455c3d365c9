"""Edge cases through the C-ABI on the device: empty circuits, no qubits, identity boundaries
that contradict (exact zeros), Clifford circuits (d = 0), qubits beyond one 64-bit word,
plans of several boundary counts, and batches with empty members."""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Batch, Simulator
from polyq_gb300.circuit import Circuit
from polyq_gb300.rng import Rng, random_clifford_t

pytestmark = pytest.mark.gpu


def test_zero_qubits_and_no_gates(gpu):
    assert Simulator(Circuit(0)).amplitudes([0], [0])[0] == 1.0
    c = Circuit(3)
    got = Simulator(c).amplitudes([0, 5, 5], [0, 5, 4])
    assert list(got) == [1.0, 1.0, 0.0]  # contradictory boundary: an exact zero, not an error


def test_clifford_circuit_has_no_branches(gpu):
    c = Circuit(4)
    c.h(0).cx(0, 1).s(1).h(2).cz(2, 3).h(3).x(0)
    sim = Simulator(c)
    assert sim.stats_full()["branch_dim"] == 0
    ys = list(range(16))
    got = sim.amplitudes([0] * 16, ys)
    want = O.dense_statevector(c, 0)
    assert np.max(np.abs(got - want)) < 1e-14


def test_qubits_beyond_one_word(gpu):
    c = Circuit(70)
    c.h(66).t(66).cx(66, 3).h(69).cz(69, 66).t(3).h(3).h(1).t(1).cx(1, 67).h(67)
    sim = Simulator(c)
    xs = [0, 1 << 66, (1 << 69) | 2]
    ys = [0, (1 << 66) | 8, (1 << 69) | (1 << 67) | 2]
    got = sim.amplitudes(xs, ys)
    want = O.OracleSim(c).amplitudes(xs, ys)
    assert np.max(np.abs(got - want)) < 1e-12
    with pytest.raises(ValueError):
        sim.amplitudes([1 << 70], [0])


def test_plans_of_several_sizes(gpu):
    c = random_clifford_t(6, 40, 6, False, Rng(3))
    sim = Simulator(c)
    ref = O.OracleSim(c)
    for n in (1, 7, 64, 3):
        ys = [(7 * i + 1) % 64 for i in range(n)]
        got = sim.amplitudes([0] * n, ys)
        assert np.max(np.abs(got - ref.amplitudes([0] * n, ys))) < 1e-12


def test_batch_with_empty_member(gpu):
    cs = [random_clifford_t(5, 30, 4, False, Rng(s)) for s in (1, 2, 3)]
    sims = [Simulator(c) for c in cs]
    b = Batch(sims, [2, 0, 3])
    xs, ys = b.pack([[0, 0], [], [0, 0, 0]], [[1, 2], [], [3, 4, 5]])
    got = b.run(xs, ys)
    assert got.shape == (5,)
    assert np.max(np.abs(got[:2] - sims[0].amplitudes([0, 0], [1, 2]))) < 1e-15
    assert np.max(np.abs(got[2:] - sims[2].amplitudes([0, 0, 0], [3, 4, 5]))) < 1e-15


def test_plan_cache_is_bounded(gpu):
    # 20 distinct boundary counts: older launch plans are evicted, results stay the same
    c = random_clifford_t(6, 40, 6, False, Rng(5))
    sim = Simulator(c)
    ref = O.OracleSim(c)
    ys = [(5 * i + 3) % 64 for i in range(40)]
    for n in list(range(1, 21)) + [3, 1]:
        got = sim.amplitudes([0] * n, ys[:n])
        assert np.max(np.abs(got - ref.amplitudes([0] * n, ys[:n]))) < 1e-12
