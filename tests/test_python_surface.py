"""The Python front-end keeps the reference binding's surface (src/pybind.rs): Circuit builders
and op lists, Simulator(circuit, strategy, pairs) with amplitude / amplitude_estimate /
probability / statevector / sample_many / marginal / stats.  Host-only: no device needed."""
import math

import pytest

from polyq_gb300 import Simulator
from polyq_gb300.circuit import Circuit, phase_from_radians


def test_extend_takes_named_ops():
    a = Circuit(3)
    a.extend([("H", [0]), ("CX", [0, 1]), ("T", [1]), ("SWAP", [1, 2]), ("SDG", [2])])
    b = Circuit(3)
    b.h(0).cx(0, 1).t(1).swap(1, 2).sdg(2)
    assert a.ops == b.ops
    with pytest.raises(ValueError):
        Circuit(2).extend([("CX", [0])])
    with pytest.raises(ValueError):
        Circuit(2).extend([("FOO", [0])])


def test_p_takes_radians_as_float_and_ring_phase_as_int():
    a = Circuit(1).p(0, math.pi / 4)
    b = Circuit(1).p(0, 1 << 29)
    assert a.ops == b.ops
    assert Circuit(1).p(0, 0.3).ops[0][3] == phase_from_radians(0.3)


def test_simulator_surface():
    for name in ("amplitude", "amplitude_estimate", "probability", "statevector", "sample_many", "marginal",
                 "stats", "pairs"):
        assert hasattr(Simulator, name), name
    c = Circuit(2).h(0).cx(0, 1).t(1)
    st = Simulator(c, "cached", host_only=True).stats()
    assert len(st) == 7  # (free_vars, planes, lines, radical, terms, branch_dim, pairs)
    with pytest.raises(ValueError):
        Simulator(c, "fastest", host_only=True)
