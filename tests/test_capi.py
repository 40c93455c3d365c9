"""The C-ABI library loads without a GPU and exports every entry point the header declares."""
import ctypes as ct
import os
import re

import pytest

from polyq_gb300 import _native as N

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "polyq_gb300.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"PQ_API\s+[\w\s\*]+?\b(pq_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(native):
    names = declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(native, n), n


def test_every_declared_symbol_has_a_binding():
    for n in declared():
        assert n in N.SIGNATURES, n


def test_no_device_is_reported_as_a_status(native):
    if native.pq_init(0) == 0:
        pytest.skip("a CUDA device is visible")
    from polyq_gb300 import Circuit, Simulator
    c = Circuit(2)
    c.h(0).cx(0, 1)
    with pytest.raises(N.PqError) as e:
        Simulator(c)
    assert e.value.status == 7
    assert native.pq_version().decode().startswith("polyq-gb300")


def test_tuning_validation(native):
    from polyq_gb300 import get_tuning, set_tuning
    old = get_tuning()
    with pytest.raises(N.PqError):
        set_tuning(inner_dims=20)
    with pytest.raises(N.PqError):
        set_tuning(block_warps=9)
    with pytest.raises(N.PqError):
        set_tuning(blocks_per_sm=5)
    assert get_tuning() == old
