"""Host producer (C++ in the product library) vs the oracle, bit for bit, without a GPU.

pq_analyze builds every branch engine on the host.  Its canonical dump -- the F2 normal
form basis (pairs_a, pairs_b, odd, even with the MinWeight pivot order), the Z4 diagonal
masks and sigma, the kernel columns and vectors, the term and boundary columns and the
RREF of the radical constraint -- must equal the oracle's word for word
(src/normal_form.rs:240-391, src/engine.rs:119-184, :289-390).
"""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300.circuit import Circuit
from polyq_gb300.rng import (Rng, random_clifford_t, random_layered, workload_batch, workload_many_boundaries,
                             workload_rotations, workload_small)


def _same_engines(circ, strategy="auto", pairs=None):
    prod = Simulator(circ, strategy, pairs, host_only=True)
    ref = O.OracleSim(circ, "pairs" if pairs is not None else strategy, pairs or 0)
    rs = ref.stats()
    ps = prod.stats_full()
    assert ps["num_branches"] == rs["branches"]
    assert ps["pairs"] == rs["pairs"]
    assert prod.stats() == (rs["free_vars"], rs["planes"], rs["lines"], rs["radical"], rs["terms"],
                            rs["branch_dim"], rs["pairs"])
    for b in range(rs["branches"]):
        a = prod.engine_dump(b)
        r = ref.engine_dump(b)
        assert a.shape == r.shape and np.array_equal(a, r), "branch %d differs" % b
    return rs


def test_random_clifford_t_engines_bit_exact():
    rng = Rng(21)
    for trial in range(120):
        n = 1 + rng.below(4)
        c = random_clifford_t(n, 8 + rng.below(14), rng.below(6), trial % 3 == 0, rng)
        _same_engines(c, "cached")
        _same_engines(c, "auto")


def test_pair_decomposed_engines_bit_exact():
    rng = Rng(5)
    for trial in range(40):
        n = 2 + rng.below(3)
        c = random_clifford_t(n, 20, 4 + rng.below(5), trial % 4 == 0, rng) if trial % 2 == 0 else random_layered(n, 3, rng)
        for p in (1, 2, 3, 6):
            _same_engines(c, pairs=p)


def test_workload_engines_bit_exact():
    st = _same_engines(workload_small(1))
    assert st["branch_dim"] == 8
    st = _same_engines(workload_many_boundaries(0), "cached")
    assert st["branch_dim"] == 29 and st["free_vars"] == 1734
    st = _same_engines(workload_many_boundaries(0), "auto")
    assert st["pairs"] == 4 and st["branches"] == 16
    for c, _ in workload_batch(6, seed=3):
        _same_engines(c, "auto")
    _same_engines(workload_rotations(n=16, ngates=300, n_rz=6, ccz_layers=1, ccz_per_layer=2), "cached")


def test_generic_angle_engines_bit_exact():
    rng = Rng(123)
    from polyq_gb300.circuit import phase_from_pi_fraction
    for _ in range(20):
        n = 3
        c = Circuit(n)
        th = phase_from_pi_fraction(1 + 2 * rng.below(3), 3)
        for _ in range(2):
            for q in range(n):
                c.h(q)
            for q in range(n):
                if rng.next_f64() < 0.8:
                    c.p(q, th if rng.next_f64() < 0.5 else (-th) % (1 << 32))
            c.cz(0, 1)
            c.cz(1, 2)
        _same_engines(c, pairs=3)
        _same_engines(c, "auto")


def test_invalid_circuits_are_rejected_without_device():
    from polyq_gb300 import _native as N
    c = Circuit(2)
    c.ops.append((99, 0, 0, 0))
    with pytest.raises(N.PqError) as e:
        Simulator(c, host_only=True)
    assert e.value.status == 1
    c = Circuit(2)
    c.ops.append((9, 1, 1, 0))  # CZ on one wire
    with pytest.raises(N.PqError):
        Simulator(c, host_only=True)
    c = Circuit(2)
    c.ops.append((0, 5, 0, 0))  # qubit out of range
    with pytest.raises(N.PqError):
        Simulator(c, host_only=True)
    with pytest.raises(ValueError):
        Simulator(Circuit(1), strategy="fastest", host_only=True)


def test_host_only_simulator_refuses_evaluation():
    from polyq_gb300 import _native as N
    c = Circuit(2)
    c.h(0).cx(0, 1).t(1)
    s = Simulator(c, host_only=True)
    with pytest.raises(N.PqError) as e:
        s.amplitudes([0], [3])
    assert e.value.status == 7


def test_large_engines_bit_exact():
    # thousands of free variables (the elimination's row spans and pivot heaps at scale)
    from polyq_gb300.rng import workload_circuit
    st = _same_engines(workload_circuit(100, 6000, 30, 1), "cached")
    assert st["free_vars"] > 5000
    _same_engines(workload_circuit(100, 10000, 40, 1), "cached")
    _same_engines(workload_circuit(80, 4000, 24, 2), pairs=2)
