"""Serving loop on the GPU: mixed request kinds, continuous batching, memory admission.

Each served result must equal the simulator's own answer for that request evaluated alone
(the same work decomposition: bit-identical), whatever else shares its wave.
"""
import time

import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300.rng import random_outputs, workload_batch
from polyq_gb300.serve import AMPLITUDE, MARGINAL, PROBABILITY, Server

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pool(gpu):
    circs = [c for c, _ in workload_batch(6, seed=11, t_max=14)]
    return circs, [Simulator(c) for c in circs]


def _requests(circs, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        k = int(rng.integers(len(circs)))
        n = circs[k].num_qubits
        kind = int(rng.integers(3))
        y = random_outputs(n, 1, int(rng.integers(1 << 30)))[0]
        reqs.append({"sim": k, "kind": kind, "x": 0, "y": y, "qubit": int(rng.integers(n)),
                     "outcome": int(rng.integers(2)), "tag": i})
    return reqs


def _expected(sims, r):
    s = sims[r["sim"]]
    if r["kind"] == AMPLITUDE:
        return complex(s.amplitudes([0], [r["y"]])[0])
    if r["kind"] == PROBABILITY:  # same re-evaluation rule as the server (1e-12 certification)
        return float(s.probabilities([0], [r["y"]])[0])
    return s.marginal(0, [(r["qubit"], r["outcome"])])


def _value(res):
    return complex(res["re"], res["im"]) if res["kind"] == AMPLITUDE else res["re"]


def test_mixed_requests_match_direct_evaluation(pool):
    circs, sims = pool
    srv = Server(sims, max_slots=32, mem_budget_bytes=1 << 28, max_branch_dim=40)
    reqs = _requests(circs, 200, 1)
    srv.submit(reqs)
    got = {r["tag"]: r for r in srv.collect(len(reqs), 120)}
    assert len(got) == len(reqs)
    for r in reqs:
        res = got[r["tag"]]
        assert res["status"] == 0, res
        want = _expected(sims, r)
        if r["kind"] == MARGINAL:
            assert abs(_value(res) - want) <= 1e-12
        elif r["kind"] == PROBABILITY:  # |a|^2 formed on the host (a fused multiply-add may differ by an ulp)
            assert abs(_value(res) - want) <= 1e-15 * abs(want)
        else:
            assert _value(res) == want  # same decomposition -> bit-identical
        assert res["done_s"] >= res["submit_s"]
    srv.close()


def test_alone_equals_in_the_mix(pool):
    circs, sims = pool
    srv = Server(sims, max_slots=64, mem_budget_bytes=1 << 28)
    probe = {"sim": 2, "kind": AMPLITUDE, "x": 0, "y": random_outputs(circs[2].num_qubits, 1, 99)[0], "tag": -1}
    srv.submit([probe])
    alone = srv.collect(1, 60)[0]
    mix = _requests(circs, 150, 2)
    srv.submit(mix[:75] + [dict(probe, tag=-2)] + mix[75:])
    res = {r["tag"]: r for r in srv.collect(151, 120)}
    assert _value(res[-2]) == _value(alone)
    srv.close()


def test_marginals_match_oracle(pool):
    circs, sims = pool
    srv = Server(sims, max_slots=16, mem_budget_bytes=1 << 28)
    c = circs[0]
    ref = O.OracleSim(c)
    reqs = [{"sim": 0, "kind": MARGINAL, "x": 0, "qubit": q, "outcome": b, "tag": 2 * q + b}
            for q in range(min(4, c.num_qubits)) for b in (0, 1)]
    srv.submit(reqs)
    res = {r["tag"]: r for r in srv.collect(len(reqs), 120)}
    for r in reqs:
        want = ref.marginal(0, [(r["qubit"], r["outcome"])])
        assert abs(res[r["tag"]]["re"] - want) <= 1e-9
    # P(q=0) + P(q=1) = 1
    for q in range(min(4, c.num_qubits)):
        assert abs(res[2 * q]["re"] + res[2 * q + 1]["re"] - 1.0) <= 1e-9
    srv.close()


def test_admission_by_dimension_cap_and_memory(pool):
    circs, sims = pool
    dims = [s.stats_full()["branch_dim"] for s in sims]
    k = int(np.argmax(dims))
    srv = Server(sims, max_slots=8, mem_budget_bytes=1 << 28, max_branch_dim=max(1, dims[k] - 1))
    srv.submit([{"sim": k, "kind": AMPLITUDE, "x": 0, "y": 0, "tag": 1}])
    r = srv.collect(1, 30)[0]
    assert r["status"] == 3  # refused, not run
    srv.close()
    # a budget too small for any single request: refused immediately
    srv = Server(sims, max_slots=8, mem_budget_bytes=64, max_branch_dim=40)
    srv.submit([{"sim": 0, "kind": AMPLITUDE, "x": 0, "y": 0, "tag": 1}])
    assert srv.collect(1, 30)[0]["status"] == 3
    srv.close()
    # a budget that fits only a few requests at a time: everything completes, in waves
    one = sims[0]
    srv = Server(sims, max_slots=64, mem_budget_bytes=20000, max_branch_dim=40)
    reqs = [{"sim": 0, "kind": AMPLITUDE, "x": 0, "y": y, "tag": i}
            for i, y in enumerate(random_outputs(circs[0].num_qubits, 40, 5))]
    srv.submit(reqs)
    res = {r["tag"]: r for r in srv.collect(40, 120)}
    assert all(res[i]["status"] == 0 for i in range(40))
    want = one.amplitudes([0] * 40, [r["y"] for r in reqs])
    assert np.array_equal(np.array([_value(res[i]) for i in range(40)]), want)
    srv.close()


def test_invalid_requests_complete_with_status(pool):
    circs, sims = pool
    srv = Server(sims, max_slots=8, mem_budget_bytes=1 << 24)
    srv.submit([{"sim": 99, "kind": 0, "tag": 1}, {"sim": 0, "kind": MARGINAL, "qubit": 999, "tag": 2},
                {"sim": 0, "kind": AMPLITUDE, "y": 1 << 127, "tag": 3}])
    res = {r["tag"]: r for r in srv.collect(3, 10)}
    assert res[1]["status"] == 1 and res[2]["status"] == 1 and res[3]["status"] == 1
    srv.drain(10)
    srv.close()


def test_overlapping_arrivals_are_admitted_while_waves_run(pool):
    circs, sims = pool
    srv = Server(sims, max_slots=4, mem_budget_bytes=1 << 28)
    t0 = time.monotonic()
    tags = 0
    for burst in range(10):
        srv.submit(_requests(circs, 8, 100 + burst))
        tags += 8
        time.sleep(0.001)
    res = srv.collect(tags, 120)
    assert len(res) == tags and all(r["status"] == 0 for r in res)
    lat = sorted(r["done_s"] - r["submit_s"] for r in res)
    assert lat[len(lat) // 2] < 10.0
    srv.close()


def test_served_probabilities_within_1e12_absolute(gpu):
    # 8 qubits, 40 T, one cached engine of d = 20-22: amplitudes of order 2^-4, where the FP32
    # bound cannot show 1e-12 on |a|^2; the server re-evaluates those requests (chunk-sum
    # tables, then the FP64 walk) in later waves, mixed with amplitude requests of the same
    # circuit that stay at the FP32 level
    from polyq_gb300.rng import workload_circuit
    c = workload_circuit(8, 240, 40, 5)
    s = Simulator(c, "cached")
    want = np.abs(O.dense_statevector(c, 0)) ** 2
    srv = Server([s], max_slots=32, mem_budget_bytes=1 << 28, max_branch_dim=40)
    reqs = []
    for y in range(256):
        reqs.append({"sim": 0, "kind": PROBABILITY, "x": 0, "y": y, "tag": y})
        if y % 8 == 0:
            reqs.append({"sim": 0, "kind": AMPLITUDE, "x": 0, "y": y, "tag": 1000 + y})
    srv.submit(reqs)
    res = {r["tag"]: r for r in srv.collect(len(reqs), 300)}
    srv.close()
    p = np.array([res[y]["re"] for y in range(256)])
    assert all(res[y]["status"] == 0 for y in range(256))
    assert np.max(np.abs(p - want)) <= 1e-12
    bound = np.array([res[y]["errbound"] for y in range(256)])
    assert np.all(np.abs(p - want) <= bound + 1e-15)  # each stated bound holds
    levels = [res[y]["level"] for y in range(256)]
    assert max(levels) >= 1  # these needed re-evaluation
    assert all(res[1000 + y]["level"] == 0 for y in range(0, 256, 8))  # amplitudes never do
    amps = s.amplitudes([0] * 32, list(range(0, 256, 8)))
    assert np.array_equal(np.array([complex(res[1000 + y]["re"], res[1000 + y]["im"]) for y in range(0, 256, 8)]), amps)


def test_requests_above_the_piece_size_are_split_not_refused(gpu):
    # the cached engine of the many-boundaries circuit has 2^29 branches per amplitude; with the
    # split threshold and piece size at 2^26 the server evaluates it over work-item ranges in
    # eight background waves and sums the pieces; the result agrees with the direct (one launch)
    # evaluation within the two error bounds, and the probability is certified to 1e-12
    from polyq_gb300.rng import workload_many_boundaries
    c = workload_many_boundaries(0)
    sim = Simulator(c, "cached")
    assert sim.stats_full()["branches_per_amplitude"] > 2 ** 26
    ys = random_outputs(50, 3, 17)
    srv = Server([sim], max_slots=8, mem_budget_bytes=1 << 28, max_branch_dim=40)
    srv.set_pieces(26, 26)
    srv.submit([{"sim": 0, "kind": AMPLITUDE, "x": 0, "y": y, "tag": i} for i, y in enumerate(ys)] +
               [{"sim": 0, "kind": PROBABILITY, "x": 0, "y": ys[0], "tag": 10}])
    res = {r["tag"]: r for r in srv.collect(4, 300)}
    srv.close()
    assert len(res) == 4 and all(r["status"] == 0 for r in res.values())
    direct, derr = sim.amplitudes([0] * 3, ys, with_error=True)
    ref = sim.amplitudes_fp64([0] * 3, ys)
    for i in range(3):
        got = complex(res[i]["re"], res[i]["im"])
        assert abs(got - direct[i]) <= res[i]["errbound"] + derr[i]
        assert abs(got - ref[i]) <= res[i]["errbound"] + 1e-13 * abs(ref[i])
        assert abs(got - ref[i]) <= 1e-6 * abs(ref[i])
    assert abs(res[10]["re"] - abs(ref[0]) ** 2) <= 1e-12


def test_marginal_engine_builds_do_not_hold_up_other_requests(pool):
    # the first marginal on a qubit builds that qubit's sandwich engines on the server's builder
    # thread; amplitude requests submitted with it are served meanwhile
    circs, sims = pool
    k = int(np.argmax([c.num_qubits for c in circs]))
    fresh = Simulator(circs[k])  # no marginal engines built yet
    srv = Server([fresh], max_slots=16, mem_budget_bytes=1 << 28, max_branch_dim=40)
    n = circs[k].num_qubits
    reqs = [{"sim": 0, "kind": MARGINAL, "x": 0, "qubit": q, "outcome": 0, "tag": 1000 + q} for q in range(n)]
    reqs += [{"sim": 0, "kind": AMPLITUDE, "x": 0, "y": y, "tag": i}
             for i, y in enumerate(random_outputs(n, 64, 5))]
    srv.submit(reqs)
    res = {r["tag"]: r for r in srv.collect(len(reqs), 300)}
    srv.close()
    assert len(res) == len(reqs) and all(r["status"] == 0 for r in res.values())
    last_amp = max(res[i]["done_s"] for i in range(64))
    last_marg = max(res[1000 + q]["done_s"] for q in range(n))
    assert last_amp < last_marg  # the amplitudes did not wait for the n marginal builds
    for q in range(n):
        assert abs(res[1000 + q]["re"] - fresh.marginal(0, [(q, 0)])) <= 1e-12
