"""The C-ABI library loads without a GPU and exports every entry point the header declares."""
import ctypes as ct
import os
import re

import pytest

from polyq_gb300 import _native as N

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "polyq_gb300.h")


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


def test_struct_layouts_match_header(tmp_path):
    # the ctypes mirrors have the C layout of include/polyq_gb300.h (sizes and field offsets,
    # printed by a C program compiled against the header)
    import subprocess
    structs = {"pq_circuit_desc": N.CircuitDesc, "pq_stats": N.Stats, "pq_tuning": N.Tuning,
               "pq_request": N.Request, "pq_result": N.Result}
    src = ["#include <stddef.h>", "#include <stdio.h>", '#include "polyq_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        src.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in py._fields_:
            src.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f[0], cname, f[0]))
    src.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = str(tmp_path / "layout")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), str(c), "-o", exe], check=True)
    out = dict(ln.split() for ln in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(out[cname]) == ct.sizeof(py), cname
        for f in py._fields_:
            assert int(out[cname + "." + f[0]]) == getattr(py, f[0]).offset, (cname, f[0])
