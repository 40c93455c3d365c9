"""A plain C program linked against the library through include/polyq_gb300.h alone (no
Python, no torch) evaluates amplitudes that match the oracle's dense statevector."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from polyq_gb300.build import LIB_PATH
from polyq_gb300.circuit import Circuit

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def test_c_client(gpu, tmp_path):
    exe = str(tmp_path / "amplitude_client")
    libdir = os.path.dirname(LIB_PATH)
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", os.path.join(REPO, "include"),
                    os.path.join(HERE, "c_client", "amplitude_client.c"), "-L", libdir, "-lpolyq_gb300",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = np.array([complex(*map(float, ln.split())) for ln in r.stdout.strip().splitlines()])
    c = Circuit(3)
    c.h(0).cx(0, 1).t(1).h(1).cz(1, 2).s(2)
    want = O.dense_statevector(c, 0)
    assert np.max(np.abs(got - want)) < 1e-12
