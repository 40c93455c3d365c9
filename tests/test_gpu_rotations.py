"""Arbitrary-angle rotations and CCZ layers through the exact amplitude path, on the GPU.

The rotation workload places rz(theta) gates (theta uniform in [0, 2 pi); src/circuit.rs:136-139
expands each into a phase gate and a global phase) and layers of CCZ on disjoint random triples
(src/circuit.rs:163-186: the 7-T Toffoli decomposition between Hadamards) into a random
Clifford circuit.  As written (n=40, 1500 gates, 24 rz, 4 layers of 8 CCZ) its cached engine has
a 239-dimensional branch subspace, beyond any exact evaluation; these tests run the scaled
variants the same generator makes with fewer CCZ per layer:

  * n=20, 400 gates, 24 rz, 2 layers of 1 CCZ (32 branch engines): every one of the 2^20
    amplitudes against the oracle's dense statevector (src/dense.rs:12-27);
  * n=20, 400 gates, 24 rz, 4 layers of 1 CCZ (2048 branch engines): the 4096 largest and 4096
    uniformly drawn amplitudes against the dense statevector;
  * n=40, 1500 gates, 24 rz, 2 layers of 1 CCZ (128 branch engines): 8 boundaries against the
    oracle's FP64 engine (the 4-layer n=40 variant's 16384 engines take the single-threaded
    oracle minutes to build, so that size is checked against the device FP64 mode and its
    prepare integers alone).

Every amplitude must lie within the error bound the library reports for it, and within 1e-6
relative of the FP64 value unless it cancels below 1e-3 of the largest amplitude compared; the
per-amplitude relative errors are recorded as test properties.
"""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300.rng import random_outputs, workload_rotations

pytestmark = pytest.mark.gpu

REL = 1e-6


def _check(got, err, want, record, name):
    diff = np.abs(got - want)
    scale = float(np.max(np.abs(want)))
    # FP64 rounding of the reference value itself (a few ulp of the sum of |terms| <= 1)
    ref_err = 1e-13 * max(scale, 1e-300)
    assert np.all(diff <= err + ref_err), "%s: error bound violated by %.3e" % (name, float(np.max(diff - err)))
    big = np.abs(want) >= 1e-3 * scale
    rel = diff[big] / np.abs(want[big])
    assert np.all(rel <= REL), "%s: max relative error %.3e" % (name, float(np.max(rel)))
    record(name + "_amplitudes", int(want.size))
    record(name + "_max_rel_err", float(np.max(rel)))
    record(name + "_median_rel_err", float(np.median(rel)))
    record(name + "_p99_rel_err", float(np.quantile(rel, 0.99)))
    record(name + "_max_bound_rel", float(np.max(err[big] / np.abs(want[big]))))


def test_rotations_n20_every_amplitude_vs_dense(gpu, record_property):
    c = workload_rotations(n=20, ngates=400, n_rz=24, ccz_layers=2, ccz_per_layer=1, seed=4)
    sv = O.dense_statevector(c, 0)
    s = Simulator(c)
    assert s.stats_full()["num_branches"] == 32
    n = 1 << 20
    got = np.zeros(n, dtype=np.complex128)
    err = np.zeros(n)
    step = 1 << 15
    for k in range(0, n, step):
        got[k:k + step], err[k:k + step] = s.amplitudes([0] * step, list(range(k, k + step)), with_error=True)
    _check(got, err, sv, record_property, "n20_2x1ccz")
    # probabilities to 1e-12 absolute on the largest amplitudes
    top = [int(i) for i in np.argsort(-np.abs(sv))[:2048]]
    p = s.probabilities([0] * len(top), top)
    assert np.max(np.abs(p - np.abs(sv[top]) ** 2)) <= 1e-12
    assert abs(float(np.sum(np.abs(got) ** 2)) - 1.0) < 1e-9


def test_rotations_n20_four_ccz_layers_vs_dense(gpu, record_property):
    c = workload_rotations(n=20, ngates=400, n_rz=24, ccz_layers=4, ccz_per_layer=1, seed=4)
    sv = O.dense_statevector(c, 0)
    s = Simulator(c)
    assert s.stats_full()["num_branches"] == 2048
    idx = [int(i) for i in np.argsort(-np.abs(sv))[:4096]] + random_outputs(20, 4096, 8)
    got, err = s.amplitudes([0] * len(idx), idx, with_error=True)
    _check(got, err, sv[idx], record_property, "n20_4x1ccz")


def test_rotations_n40_vs_oracle(gpu, record_property):
    c = workload_rotations(n=40, ngates=1500, n_rz=24, ccz_layers=2, ccz_per_layer=1, seed=4)
    s, r = Simulator(c), O.OracleSim(c)
    assert s.stats_full()["num_branches"] == 128
    ys = random_outputs(40, 8, 4)
    got, err = s.amplitudes([0] * 8, ys, with_error=True)
    want = r.amplitudes([0] * 8, ys)
    _check(got, err, want, record_property, "n40_2x1ccz")
    # the prepare integers of every (boundary, branch engine) job, bit-exact
    assert np.array_equal(s.prepare_info([0] * 8, ys), r.prepare_info([0] * 8, ys))


def test_rotations_n40_16384_engines_vs_device_fp64(gpu, record_property):
    # the scaled workload of the benchmark: 4 layers of 1 CCZ, 14 T-pairs, 16384 branch engines
    c = workload_rotations(n=40, ngates=1500, n_rz=24, ccz_layers=4, ccz_per_layer=1, seed=4)
    s = Simulator(c)
    assert s.stats_full()["num_branches"] == 16384
    ys = random_outputs(40, 8, 4)
    got, err = s.amplitudes([0] * 8, ys, with_error=True)
    ref = s.amplitudes_fp64([0] * 8, ys)
    _check(got, err, ref, record_property, "n40_4x1ccz_vs_fp64")
