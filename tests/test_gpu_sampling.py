"""Simulator::sample_many on the device (src/sim.rs:253-284): same seed, same samples as the
oracle's restatement, and the reference's distribution test (src/sim.rs:382-399)."""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300.circuit import Circuit
from polyq_gb300.rng import Rng, random_clifford_t

pytestmark = pytest.mark.gpu


def _three_qubit():
    c = Circuit(3)
    c.h(0).t(0).h(0).cx(0, 1).h(2).t(2).h(2).cz(1, 2).h(1).t(1).h(1)
    return c


def test_sampling_follows_the_distribution(gpu):
    c = _three_qubit()
    sv = O.dense_statevector(c, 0)
    shots = 40000
    hist = np.bincount(Simulator(c).sample_many(0, shots, 1234), minlength=8)
    for y in range(8):
        assert abs(abs(sv[y]) ** 2 - hist[y] / shots) < 0.012


@pytest.mark.parametrize("seed", [1, 7])
def test_samples_equal_the_oracle(gpu, seed):
    c = random_clifford_t(7, 40, 6, False, Rng(seed))
    got = Simulator(c).sample_many(5, 300, 99 + seed)
    want = O.OracleSim(c).sample_many(5, 300, 99 + seed)
    assert got == want


def test_samples_equal_the_oracle_three_qubits(gpu):
    c = _three_qubit()
    assert Simulator(c).sample_many(0, 2000, 42) == O.OracleSim(c).sample_many(0, 2000, 42)
