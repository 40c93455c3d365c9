"""GPU parity: the sm_103a path through the C-ABI against the CPU oracle.

Bit-exact: normal forms (engine dumps) and the Z8 index of every branch.
Numerical: amplitudes within 1e-6 relative of the FP64 oracle and within the per-result
error bound the library reports; probabilities within 1e-12 absolute.
"""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Batch, Simulator, set_tuning, get_tuning
from polyq_gb300 import _native as N
from polyq_gb300.circuit import Circuit
from polyq_gb300.rng import (Rng, random_clifford_t, random_layered, random_outputs, workload_batch,
                             workload_many_boundaries, workload_small)

pytestmark = pytest.mark.gpu

REL = 1e-6  # amplitude tolerance relative to the FP64 oracle
PROB_ABS = 1e-12


def assert_amps(got, want, err=None, rel=REL):
    """Every result within its reported bound; amplitudes within `rel` of the FP64 value,
    except ones that cancel (|want| < 1e-3 of the batch scale), which must be within 1e-7 of
    the scale -- a relative error of an (almost) exactly cancelled sum is not defined."""
    got = np.asarray(got)
    want = np.asarray(want)
    diff = np.abs(got - want)
    scale = float(np.max(np.abs(want))) if want.size else 0.0
    floor = 1e-300 + 1e-7 * scale
    ok = diff <= rel * np.abs(want) + floor
    big = np.abs(want) >= 1e-3 * scale
    assert np.all(diff[big] <= rel * np.abs(want[big]) + 1e-300), "relative error above %g" % rel
    if err is not None:
        # the FP64 reference carries its own rounding (~1e-16 per term): allow 1e-13 of scale
        ref_err = 1e-13 * max(1.0, float(np.max(np.abs(want)))) if want.size else 0.0
        assert np.all(diff <= err + ref_err), "error bound violated: %s" % (diff - err).max()
    assert np.all(ok), "max rel err %.3e" % float(np.max(diff / np.maximum(np.abs(want), 1e-300)))


def test_known_answers(gpu):
    import json, os
    with open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")) as f:
        ka = json.load(f)
    for case in ka["amplitudes"]:
        c = Circuit(case["num_qubits"])
        for op in case["ops"]:
            c.push(*op)
        s = Simulator(c)
        xs = [v[0] for v in case["values"]]
        ys = [v[1] for v in case["values"]]
        want = np.array([complex(v[2], v[3]) for v in case["values"]])
        got, err = s.amplitudes(xs, ys, with_error=True)
        assert np.all(np.abs(got - want) <= np.maximum(REL * np.abs(want), err) + 1e-15), case["source"]
        p = s.probabilities(xs, ys)
        assert np.all(np.abs(p - np.abs(want) ** 2) <= PROB_ABS), case["source"]


def test_branch_phases_bit_exact(gpu):
    # every branch engine b of every strategy: the 2^p T-pair engines (src/rank.rs:88-103,
    # src/pathsum.rs:360-394) as well as the cached engine, Z8 index of every branch
    # (src/normal_form.rs:479-493) bit-exact against the oracle
    rng = Rng(21)
    checked = checked_pairs = 0
    for trial in range(60):
        n = 1 + rng.below(4)
        c = random_clifford_t(n, 8 + rng.below(14), rng.below(6), trial % 3 == 0, rng)
        for strat, p in (("cached", None), ("auto", None), ("pairs", 2)):
            s = Simulator(c, strat, p)
            r = O.OracleSim(c, strat, p or 0)
            nb = s.stats_full()["num_branches"]
            assert nb == r.stats()["branches"]
            for b in range(nb):
                assert s.engine_shape(b)["d"] == r.branch_dim(b)
                for x, y in ((0, 0), (1 % (1 << n), (1 << n) - 1)):
                    want = r.branch_phases(x, y, b)
                    got = s.branch_phases(x, y, b)
                    assert (want is None) == (got is None), (trial, strat, b)
                    if want is None:
                        continue
                    assert np.array_equal(got, want), (trial, strat, b)
                    checked += 1
                    checked_pairs += b > 0
    # layered circuits (src/rng.rs random_layered) keep their T gates apart, so they have pair
    # candidates: up to 8 branch engines of d = 0..9 each
    rng = Rng(77)
    for trial in range(30):
        n = 3 + rng.below(3)
        c = random_layered(n, 2 + rng.below(3), rng)
        for strat, p in (("auto", None), ("pairs", 3)):
            s = Simulator(c, strat, p)
            r = O.OracleSim(c, strat, p or 0)
            nb = s.stats_full()["num_branches"]
            assert nb == r.stats()["branches"]
            for b in range(nb):
                assert s.engine_shape(b)["d"] == r.branch_dim(b)
                for x, y in ((0, 0), (1, (1 << n) - 1), (2, 5 % (1 << n))):
                    want = r.branch_phases(x, y, b)
                    got = s.branch_phases(x, y, b)
                    assert (want is None) == (got is None), (trial, strat, b)
                    if want is None:
                        continue
                    assert np.array_equal(got, want), (trial, strat, b)
                    checked += 1
                    checked_pairs += b > 0
    assert checked > 400 and checked_pairs > 200


def test_branch_phases_bit_exact_workloads(gpu):
    c = workload_small(1)
    s, r = Simulator(c, "cached"), O.OracleSim(c, "cached")
    ys = [0] + random_outputs(c.num_qubits, 40, 5)
    seen = 0
    for y in ys:
        want = r.branch_phases(0, y)
        got = s.branch_phases(0, y)
        assert (want is None) == (got is None)
        if want is not None:
            assert np.array_equal(got, want)
            seen += 1
    # the many-boundaries workload, strategy auto: all 16 branch engines (d = 20..22)
    c = workload_many_boundaries(0)
    s, r = Simulator(c, "auto"), O.OracleSim(c, "auto")
    nb = s.stats_full()["num_branches"]
    assert nb == 16
    live = 0
    for y in random_outputs(50, 2, 9):
        for b in range(nb):
            want = r.branch_phases(0, y, b)
            got = s.branch_phases(0, y, b)
            assert (want is None) == (got is None), b
            if want is not None:
                assert got.shape == want.shape and np.array_equal(got, want), b
                live += 1
    assert live >= 4


def test_engine_dumps_match_oracle(gpu):
    for c in (workload_small(1), workload_many_boundaries(0)):
        s, r = Simulator(c), O.OracleSim(c)
        for b in range(r.stats()["branches"]):
            assert np.array_equal(s.engine_dump(b), r.engine_dump(b))


def test_engine_matches_brute_force(gpu):
    # src/engine.rs:746-774 on the GPU path
    rng = Rng(21)
    for trial in range(120):
        n = 1 + rng.below(4)
        c = random_clifford_t(n, 8 + rng.below(14), rng.below(6), trial % 3 == 0, rng)
        s = Simulator(c, "cached")
        r = O.OracleSim(c, "cached")
        xs = [x for x in range(1 << n) for _ in range(1 << n)]
        ys = [y for _ in range(1 << n) for y in range(1 << n)]
        got, err = s.amplitudes(xs, ys, with_error=True)
        want = np.array([r.brute_force(x, y) for x, y in zip(xs, ys)])
        assert_amps(got, want, err)


def test_statevector_matches_dense_all_strategies(gpu):
    # src/sim.rs:330-342 on the GPU path
    rng = Rng(99)
    for trial in range(50):
        n = 1 + rng.below(5)
        if trial % 2 == 0:
            c = random_clifford_t(n, 25, rng.below(8), trial % 4 == 0, rng)
        else:
            c = random_layered(n, 2 + rng.below(2), rng)
        inp = sum(1 << q for q in range(n) if rng.next_f64() < 0.5)
        want = O.dense_statevector(c, inp)
        for strat, p in (("cached", None), ("auto", None), ("auto", 2), ("auto", 100)):
            s = Simulator(c, strat, p)
            got, err = s.amplitudes([inp] * (1 << n), list(range(1 << n)), with_error=True)
            assert_amps(got, want, err)
            probs = s.probabilities([inp] * (1 << n), list(range(1 << n)))
            assert np.max(np.abs(probs - np.abs(want) ** 2)) <= PROB_ABS


def test_marginals_match_dense(gpu):
    rng = Rng(3)
    for _ in range(12):
        n = 2 + rng.below(3)
        c = random_layered(n, 2, rng)
        sv = O.dense_statevector(c, 0)
        s = Simulator(c)
        for _ in range(4):
            k = 1 + rng.below(n)
            qs = list(range(n))
            for i in range(n - 1, 0, -1):
                j = rng.below(i + 1)
                qs[i], qs[j] = qs[j], qs[i]
            meas = [(q, rng.next_f64() < 0.5) for q in qs[:k]]
            want = sum(abs(a) ** 2 for i, a in enumerate(sv) if all(((i >> q) & 1) == b for q, b in meas))
            assert abs(s.marginal(0, meas) - want) < 1e-6


def test_small_workload_vs_oracle_and_dense(gpu):
    c = workload_small(1)
    s = Simulator(c)
    r = O.OracleSim(c)
    sv = O.dense_statevector(c, 0)
    ys = [0] + [int(i) for i in np.nonzero(np.abs(sv) > 1e-9)[0][:200]]
    got, err = s.amplitudes([0] * len(ys), ys, with_error=True)
    assert_amps(got, r.amplitudes([0] * len(ys), ys), err)
    assert_amps(got, sv[ys], None, rel=1e-6)
    p = s.probabilities([0] * len(ys), ys)
    assert np.max(np.abs(p - np.abs(sv[ys]) ** 2)) <= PROB_ABS


def test_many_boundaries_sample_vs_oracle(gpu):
    c = workload_many_boundaries(0)
    s = Simulator(c)
    r = O.OracleSim(c)
    ys = random_outputs(50, 24, 2024)
    got, err = s.amplitudes([0] * len(ys), ys, with_error=True)
    want = r.amplitudes([0] * len(ys), ys)
    assert_amps(got, want, err)


def test_many_boundaries_full_fp32_vs_device_fp64(gpu):
    # full size: all 4096 boundaries, FP32-compensated against the device FP64 mode
    c = workload_many_boundaries(0)
    s = Simulator(c)
    ys = random_outputs(50, 4096, 1)
    got, err = s.amplitudes([0] * 4096, ys, with_error=True)
    ref = s.amplitudes_fp64([0] * 4096, ys)
    diff = np.abs(got - ref)
    assert np.all(diff <= err + 1e-300)
    rel = diff / np.abs(ref)
    assert np.max(rel) <= REL
    assert np.median(rel) < 1e-8


def test_batch_equals_individual_and_plain(gpu):
    circs = workload_batch(8, seed=3, t_max=14)
    sims = [Simulator(c) for c, _ in circs]
    outs = [random_outputs(c.num_qubits, 5, i) for i, (c, _) in enumerate(circs)]
    b = Batch(sims, [5] * len(sims))
    xs, ys = b.pack([[0] * 5] * len(sims), outs)
    got = b.run(xs, ys)
    for i, s in enumerate(sims):
        alone = s.amplitudes([0] * 5, outs[i])
        assert np.array_equal(got[5 * i:5 * i + 5], alone)  # same work decomposition: bit-identical
        plain = s.amplitudes_plain([0] * 5, outs[i])
        assert np.array_equal(plain, alone)
        r = O.OracleSim(circs[i][0])
        assert_amps(alone, r.amplitudes([0] * 5, outs[i]))


def test_admission_and_invalid_arguments(gpu):
    c = workload_many_boundaries(0)
    old = get_tuning()
    try:
        set_tuning(max_branch_dim=10)
        s = Simulator(c, "cached")
        with pytest.raises(N.PqError) as e:
            s.amplitudes([0], [1])
        assert e.value.status == 3
    finally:
        set_tuning(max_branch_dim=old["max_branch_dim"])
    s = Simulator(workload_small(1))
    with pytest.raises(ValueError):
        s.amplitudes([0], [1 << 40])
    with pytest.raises(N.PqError) as e:
        s.marginal(0, [(99, 1)])
    assert e.value.status == 1


def test_device_resident_path_matches_host_path(gpu):
    torch = pytest.importorskip("torch")
    import ctypes as ct
    c = workload_many_boundaries(0)
    s = Simulator(c)
    ys = random_outputs(50, 64, 77)
    host = s.amplitudes([0] * 64, ys)
    from polyq_gb300.sim import pack_bits
    dx = torch.from_numpy(pack_bits([0] * 64, 50).view(np.int64)).cuda()
    dy = torch.from_numpy(pack_bits(ys, 50).view(np.int64)).cuda()
    out = torch.zeros(128, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    N.check(N.lib().pq_amplitudes_device(s.handle, 64, ct.c_void_p(dx.data_ptr()), ct.c_void_p(dy.data_ptr()),
                                         ct.c_void_p(out.data_ptr()), None, ct.c_void_p(st)))
    torch.cuda.synchronize()
    dev = out.cpu().numpy().view(np.complex128)
    assert np.array_equal(dev, host)
    # the prepare kernel's self-check of that launch (a failure would also make it NaN)
    failed = ct.c_int32(-1)
    N.check(N.lib().pq_sim_device_check(s.handle, 64, ct.byref(failed)))
    assert failed.value == 0 and np.all(np.isfinite(dev))


def test_autotune_keeps_results(gpu):
    # the autotuner may change every launch-shape field; amplitudes move by the FP64 summation
    # order and the grouping of chunks into units (combined in FP32 pairs, ~1e-14 of the summed
    # magnitudes), far inside their bounds, and stay within those bounds of the FP64 oracle
    c = workload_many_boundaries(0)
    s = Simulator(c)
    ys = random_outputs(50, 128, 5)
    before = s.amplitudes([0] * 128, ys)
    tuning, ms = s.autotune([0] * 128, ys, reps=1)
    assert ms > 0.0
    assert s.tuning() == tuning
    assert tuning["blocks_per_sm"] in (2, 3, 4) and 8 <= tuning["inner_dims"] <= 10
    after, err = s.amplitudes([0] * 128, ys, with_error=True)
    scale = float(np.max(np.abs(before)))
    assert np.all(np.abs(after - before) <= err + 1e-12 * scale)
    want = O.OracleSim(c).amplitudes([0] * 24, ys[:24])
    assert_amps(after[:24], want, err[:24])
    for bps in (2, 3, 4):
        set_old = get_tuning()
        try:
            set_tuning(blocks_per_sm=bps)
            s2 = Simulator(c)
            assert s2.tuning()["blocks_per_sm"] == bps
            a2, e2 = s2.amplitudes([0] * 128, ys, with_error=True)
            assert np.all(np.abs(a2 - before) <= 1e-3 * e2 + 1e-13 * scale)
        finally:
            set_tuning(blocks_per_sm=set_old["blocks_per_sm"])


def test_batch_autotune_keeps_results(gpu):
    circs = workload_batch(8, seed=3, t_max=14)
    sims = [Simulator(c) for c, _ in circs]
    outs = [random_outputs(c.num_qubits, 5, i) for i, (c, _) in enumerate(circs)]
    b = Batch(sims, [5] * len(sims))
    xs, ys = b.pack([[0] * 5] * len(sims), outs)
    before, err = b.run(xs, ys, with_error=True)
    tuning, ms = b.autotune(xs, ys, reps=1)
    assert ms > 0.0 and tuning["blocks_per_sm"] in (2, 3, 4) and tuning["unit_chunks"] in (2, 4, 8)
    after = b.run(xs, ys)
    # only the FP64 summation order of work-item partials may change
    assert np.all(np.abs(after - before) <= err + 1e-13 * np.abs(before))
    for i, s in enumerate(sims[:3]):
        r = O.OracleSim(circs[i][0])
        assert_amps(after[5 * i:5 * i + 5], r.amplitudes([0] * 5, outs[i]))


def test_batched_workload_full_fp32_vs_device_fp64(gpu):
    # the uneven batch at full size (256 circuits, 64 boundaries each) through one launch, each
    # amplitude against the device FP64 mode: within its bound, <= 1e-6 relative
    circs = workload_batch(256, seed=3)
    sims = [Simulator(c) for c, _ in circs]
    outs = [random_outputs(c.num_qubits, 64, 1000 + i) for i, (c, _) in enumerate(circs)]
    b = Batch(sims, [64] * len(sims))
    xs, ys = b.pack([[0] * 64] * len(sims), outs)
    got, err = b.run(xs, ys, with_error=True)
    ref = np.concatenate([s.amplitudes_fp64([0] * 64, o) for s, o in zip(sims, outs)])
    diff = np.abs(got - ref)
    assert np.all(diff <= err + 1e-300)
    for i in range(len(sims)):
        assert_amps(got[64 * i:64 * i + 64], ref[64 * i:64 * i + 64], err[64 * i:64 * i + 64])


def test_probabilities_within_1e12_absolute(gpu):
    # probabilities are certified to 1e-12 absolute (FP64 re-evaluation when the FP32 bound
    # cannot show it): many-boundaries workload against the device FP64 mode and the oracle
    c = workload_many_boundaries(0)
    s = Simulator(c)
    ys = random_outputs(50, 512, 31)
    p = s.probabilities([0] * 512, ys)
    ref = np.abs(s.amplitudes_fp64([0] * 512, ys)) ** 2
    assert np.max(np.abs(p - ref)) <= 1e-12
    want = np.abs(O.OracleSim(c).amplitudes([0] * 16, ys[:16])) ** 2
    assert np.max(np.abs(p[:16] - want)) <= 1e-12


def test_chunk_tables_match_fp64(gpu):
    # opt-in chunk-sum tables (one FP64 lookup per chunk): the FP64 enumeration's amplitudes to
    # FP64 rounding (relative to the summed magnitudes), on the many-boundaries workload and an
    # uneven batch
    old = get_tuning()
    try:
        set_tuning(chunk_tables=1)
        c = workload_many_boundaries(0)
        s = Simulator(c)
        ys = random_outputs(50, 512, 3)
        got = s.amplitudes([0] * 512, ys)
        ref = s.amplitudes_fp64([0] * 512, ys)
        scale = float(np.max(np.abs(ref)))
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale
        want = O.OracleSim(c).amplitudes([0] * 12, ys[:12])
        assert_amps(got[:12], want)
        circs = workload_batch(24, seed=3, t_max=20)
        sims = [Simulator(cc) for cc, _ in circs]
        for sm, (cc, _) in zip(sims, circs):
            ys2 = random_outputs(cc.num_qubits, 6, 9)
            a, err = sm.amplitudes([0] * 6, ys2, with_error=True)
            r = sm.amplitudes_fp64([0] * 6, ys2)
            assert_amps(a, r, err)  # within the reported bound; FP64 rounding of cancelling sums
    finally:
        set_tuning(chunk_tables=2)


def test_probabilities_of_large_amplitudes(gpu):
    # 8 qubits, 40 T, one cached engine of d = 20-22: amplitudes of order 2^-4, where the FP32
    # bound cannot certify 1e-12 on |a|^2 and the probability is re-evaluated (chunk-sum
    # tables, then FP64 if needed); all 256 probabilities against the dense statevector
    from polyq_gb300.rng import workload_circuit
    for seed in (5, 7):
        c = workload_circuit(8, 240, 40, seed)
        s = Simulator(c, "cached")
        p = s.probabilities([0] * 256, list(range(256)))
        want = np.abs(O.dense_statevector(c, 0)) ** 2
        assert np.max(np.abs(p - want)) <= 1e-12
        assert abs(np.sum(p) - 1.0) < 1e-9


def test_unit_sizes_agree_within_bounds(gpu):
    # units of 1, 2, 4 and 8 chunks (the pair coordinates a unit does not vary come from its
    # first chunk's bits): every unit size within its bound of the device FP64 walk, on the
    # many-boundaries workload (branch engines with 0..3 pair coordinates)
    c = workload_many_boundaries(0)
    ys = random_outputs(50, 64, 77)
    ref = None
    old = get_tuning()
    try:
        for uc, bps in ((1, 3), (2, 3), (4, 3), (8, 2)):
            set_tuning(unit_chunks=uc, blocks_per_sm=bps)
            s = Simulator(c)
            got, err = s.amplitudes([0] * 64, ys, with_error=True)
            if ref is None:
                ref = s.amplitudes_fp64([0] * 64, ys)
            assert_amps(got, ref, err)
    finally:
        set_tuning(unit_chunks=old["unit_chunks"], blocks_per_sm=old["blocks_per_sm"])


def _many_pivot_circuits():
    # members C of the serving pool sandwiched as C, (H T on the first k qubits), C^dagger: their
    # cached engines have 13..15 pivots, more than one joint weight table indexes; the table then
    # covers the pivots the walked coordinates touch and the rest enter as a per-unit FP64 factor
    circs = [c for c, _ in workload_batch(64, seed=5, t_max=40)]
    out = []
    for i, k in ((12, 2), (5, 2), (11, 1), (37, 1), (3, 1)):
        cc = circs[i].copy()
        for q in range(k):
            cc.h(q)
            cc.t(q)
        out.append(cc.extend(circs[i].inverse()))
    return out


def test_many_pivot_engines_walk_in_fp32(gpu):
    checked = 0
    for cc in _many_pivot_circuits():
        s, r = Simulator(cc), O.OracleSim(cc)
        nb = s.stats_full()["num_branches"]
        sv = O.dense_statevector(cc, 0)
        ys = [int(i) for i in np.argsort(-np.abs(sv))[:48]] + random_outputs(cc.num_qubits, 16, 3)
        xs = [0] * len(ys)
        for b in range(nb):
            shp = s.engine_shape(b)
            assert shp["rank"] > 10 and shp["joint"] == 1, shp
            for y in ys[:2]:
                want = r.branch_phases(0, y, b)
                got = s.branch_phases(0, y, b)
                assert (want is None) == (got is None)
                if want is not None:
                    assert np.array_equal(got, want)
                    checked += 1
        assert np.array_equal(s.prepare_info(xs, ys), r.prepare_info(xs, ys))
        got, err = s.amplitudes(xs, ys, with_error=True)
        assert_amps(got, r.amplitudes(xs, ys), err)
        assert_amps(got, sv[ys], err)
        p = s.probabilities(xs, ys)
        assert np.max(np.abs(p - np.abs(sv[ys]) ** 2)) <= PROB_ABS
    assert checked >= 5


def test_many_pivot_engines_chunk_tables(gpu):
    # the chunk-sum tables of a partial table (FP64, indexed like the table, the other pivots'
    # weight applied per chunk) against the FP64 walk
    old = get_tuning()
    try:
        set_tuning(chunk_tables=1)
        for cc in _many_pivot_circuits()[:3]:
            s = Simulator(cc)
            sv = O.dense_statevector(cc, 0)
            ys = [int(i) for i in np.argsort(-np.abs(sv))[:32]]
            got = s.amplitudes([0] * len(ys), ys)
            ref = s.amplitudes_fp64([0] * len(ys), ys)
            assert np.max(np.abs(got - ref)) <= 1e-12 * float(np.max(np.abs(ref)))
    finally:
        set_tuning(chunk_tables=2)
