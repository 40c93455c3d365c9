"""Pin the CPU oracle against the reference's own known-answer and invariant tests.

Each test restates one test of the reference crate (same seeds, sizes and tolerances) and
runs it on the oracle (oracle/pq_oracle.c).  Seeded circuits come from the bit-exact
SplitMix64 generators in polyq_gb300.rng (src/rng.rs).
"""
import cmath
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from polyq_gb300.circuit import Circuit, phase_from_pi_fraction, phase_from_radians, phase_to_radians
from polyq_gb300.rng import Rng, random_clifford_t, random_layered

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def known():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def test_phase_ring_constants():
    # src/phase.rs:154-183
    q, h, pi = 1 << 29, 1 << 30, 1 << 31
    assert (q + q) % (1 << 32) == h and (h + h) % (1 << 32) == pi and (pi + pi) % (1 << 32) == 0
    for k in [0, 1, 12345, 1 << 29, (1 << 31) + 7, (1 << 32) - 1]:
        assert phase_from_radians(phase_to_radians(k)) == k
    assert phase_from_radians(-math.pi / 4) == (-q) % (1 << 32)
    assert phase_from_pi_fraction(-1, 2) == (-q) % (1 << 32)
    assert phase_from_pi_fraction(3, 2) & ((1 << 30) - 1) != 0


def test_bell_and_ghz():
    # src/engine.rs:777-787
    c = Circuit(3)
    c.h(0).cx(0, 1).cx(1, 2)
    s = O.OracleSim(c)
    for y in range(8):
        want = 1 / math.sqrt(2) if y in (0, 7) else 0.0
        assert abs(s.amplitude(0, y) - want) < 1e-12


def test_old_v1_bug_case():
    # src/engine.rs:790-802: H T Z H |0> = ((1-w)|0> + (1+w)|1>)/2, w = e^{i pi/4}
    c = Circuit(1)
    c.h(0).t(0).z(0).h(0)
    s = O.OracleSim(c)
    w = cmath.exp(1j * math.pi / 4)
    assert abs(s.amplitude(0, 0) - (1 - w) / 2) < 1e-12
    assert abs(s.amplitude(0, 1) - (1 + w) / 2) < 1e-12


def test_toffoli_truth_table():
    # src/circuit.rs:234-244
    for inp in range(8):
        c = Circuit(3)
        c.ccx(0, 1, 2)
        assert c.t_count() == 7
        sv = O.dense_statevector(c, inp)
        expect = inp ^ 4 if (inp & 3) == 3 else inp
        assert abs(abs(sv[expect]) - 1.0) < 1e-9


def test_inverse_is_inverse():
    # src/circuit.rs:224-231
    c = Circuit(3)
    c.h(0).t(0).cx(0, 1).s(1).tdg(2).cz(1, 2).swap(0, 2).x(1).y(0).p(2, phase_from_pi_fraction(3, 5))
    full = c.copy().extend(c.inverse())
    sv = O.dense_statevector(full, 0)
    assert abs(abs(sv[0]) - 1.0) < 1e-9


def test_pathsum_matches_dense_random():
    # src/pathsum.rs:504-530
    rng = Rng(7)
    checked = 0
    for trial in range(60):
        n = 1 + rng.below(3)
        c = random_clifford_t(n, 6 + rng.below(8), rng.below(4), trial % 2 == 0, rng)
        s = O.OracleSim(c, "cached")
        checked += 1
        for x in range(1 << n):
            sv = O.dense_statevector(c, x)
            for y in range(1 << n):
                assert abs(s.brute_force(x, y) - sv[y]) < 1e-9
    assert checked >= 40


def test_engine_matches_brute_force():
    # src/engine.rs:746-774 (seed 21, 120 trials, 1e-8)
    rng = Rng(21)
    checked = 0
    for trial in range(120):
        n = 1 + rng.below(4)
        c = random_clifford_t(n, 8 + rng.below(14), rng.below(6), trial % 3 == 0, rng)
        s = O.OracleSim(c, "cached")
        checked += 1
        for x in range(1 << n):
            for y in range(1 << n):
                assert abs(s.amplitude(x, y) - s.brute_force(x, y)) < 1e-8
    assert checked >= 60


def test_statevector_matches_dense_all_strategies():
    # src/sim.rs:330-342 (seed 99; Cached, Auto, Pairs(2), Pairs(100); 1e-8)
    rng = Rng(99)
    for trial in range(50):
        n = 1 + rng.below(5)
        if trial % 2 == 0:
            c = random_clifford_t(n, 25, rng.below(8), trial % 4 == 0, rng)
        else:
            c = random_layered(n, 2 + rng.below(2), rng)
        inp = sum(1 << q for q in range(n) if rng.next_f64() < 0.5)
        want = O.dense_statevector(c, inp)
        for strat, p in (("cached", 0), ("auto", 0), ("pairs", 2), ("pairs", 100)):
            s = O.OracleSim(c, strat, p)
            got = s.amplitudes([inp] * (1 << n), list(range(1 << n)))
            assert np.max(np.abs(got - want)) < 1e-8


def test_toffoli_circuit_exact():
    # src/sim.rs:345-351
    c = Circuit(4)
    c.h(0).h(1).ccx(0, 1, 2).cx(2, 3).ccz(0, 2, 3).h(3)
    s = O.OracleSim(c)
    got = s.amplitudes([0] * 16, list(range(16)))
    assert np.max(np.abs(got - O.dense_statevector(c, 0))) < 1e-9


def test_marginals_match_dense():
    # src/sim.rs:354-379 (seed 3)
    rng = Rng(3)
    for _ in range(12):
        n = 2 + rng.below(3)
        c = random_layered(n, 2, rng)
        sv = O.dense_statevector(c, 0)
        s = O.OracleSim(c)
        for _ in range(4):
            k = 1 + rng.below(n)
            qs = list(range(n))
            for i in range(n - 1, 0, -1):
                j = rng.below(i + 1)
                qs[i], qs[j] = qs[j], qs[i]
            meas = [(q, rng.next_f64() < 0.5) for q in qs[:k]]
            want = sum(abs(a) ** 2 for i, a in enumerate(sv) if all(((i >> q) & 1) == b for q, b in meas))
            assert abs(s.marginal(0, meas) - want) < 1e-9


def test_equivalence_known_answers():
    # src/sim.rs:402-438
    a = Circuit(1); a.h(0).z(0).h(0)
    b = Circuit(1); b.x(0)
    eq, ov = O.equivalence(a, b)
    assert eq and abs(cmath.phase(ov)) < 1e-9
    t2 = Circuit(2); t2.t(0).t(0).cx(0, 1)
    s1 = Circuit(2); s1.s(0).cx(0, 1)
    assert O.equivalence(t2, s1)[0]
    t1 = Circuit(2); t1.t(0).cx(0, 1)
    assert not O.equivalence(t1, s1)[0]
    y = Circuit(1); y.y(0)
    xz = Circuit(1); xz.z(0).x(0)
    eq, ov = O.equivalence(y, xz)
    assert eq and abs(cmath.phase(ov) - math.pi / 2) < 1e-9
    c1 = Circuit(3); c1.ccx(0, 1, 2)
    c2 = Circuit(3); c2.h(2).ccz(0, 1, 2).h(2)
    assert O.equivalence(c1, c2)[0]
    c3 = Circuit(3); c3.ccx(0, 1, 2).t(0)
    assert not O.equivalence(c1, c3)[0]


def _random_form(m, density, rng):
    B = np.zeros((m, m), np.uint8)
    for i in range(m):
        for j in range(i + 1, m):
            if rng.next_f64() < density:
                B[i, j] ^= 1
                B[j, i] ^= 1
    v = np.array([rng.below(4) for _ in range(m)], np.uint8)
    return B, v


@pytest.mark.parametrize("rule", [0, 1])
def test_basis_block_diagonalises_gram(rule):
    # src/normal_form.rs:555-606 (seed 1, 200 forms, m <= 40); rule 0 = First, 1 = MinWeight
    rng = Rng(1)
    for trial in range(200):
        m = 1 + rng.below(40)
        B, v = _random_form(m, [0.05, 0.2, 0.5][trial % 3], rng)
        rc, sizes = O.check_structure(B, v & 1, rule)
        assert rc == 0
        assert 2 * sizes[0] + sizes[1] + sizes[2] == m


def test_gauss_sum_matches_brute_force():
    # src/normal_form.rs:609-625 (seed 2, 400 trials, 1e-9)
    rng = Rng(2)
    for trial in range(400):
        m = 1 + rng.below(11)
        B, v = _random_form(m, [0.1, 0.3, 0.6][trial % 3], rng)
        shift = np.array([1 if rng.next_f64() < 0.4 else 0 for _ in range(m)], np.uint8)
        for rule in (0, 1):
            a, b = O.gauss_sum(B, v, shift, rule)
            assert abs(a - b) < 1e-9


def test_alternating_forms():
    # src/normal_form.rs:628-645 (seed 3): all-even v gives no odd lines
    rng = Rng(3)
    for _ in range(100):
        m = 2 + rng.below(9)
        B, v = _random_form(m, 0.4, rng)
        v = v & 2
        rc, sizes = O.check_structure(B, v & 1, 1)
        assert rc == 0 and sizes[1] == 0
        a, b = O.gauss_sum(B, v, np.zeros(m, np.uint8), 1)
        assert abs(a - b) < 1e-9


def test_rank_engine_matches_plain_engine():
    # src/rank.rs:244-276 (seed 5)
    rng = Rng(5)
    with_pairs = 0
    for trial in range(60):
        n = 2 + rng.below(3)
        if trial % 2 == 0:
            c = random_clifford_t(n, 20, 4 + rng.below(5), trial % 4 == 0, rng)
        else:
            c = random_layered(n, 3, rng)
        plain = O.OracleSim(c, "cached")
        xs = [x for x in range(1 << n) for _ in range(1 << n)]
        ys = [y for _ in range(1 << n) for y in range(1 << n)]
        a = plain.amplitudes(xs, ys)
        for pairs in (1, 2, 3, 6):
            r = O.OracleSim(c, "pairs", pairs)
            if r.stats()["pairs"] > 0:
                with_pairs += 1
            assert np.max(np.abs(a - r.amplitudes(xs, ys))) < 1e-8
    assert with_pairs >= 20


def test_t_pair_identity_is_clifford_in_both_branches():
    # src/rank.rs:321-331
    c = Circuit(2)
    c.h(0).h(1).t(0).t(1).h(0).h(1)
    r = O.OracleSim(c, "pairs", 1)
    st = r.stats()
    assert st["pairs"] == 1 and st["branches"] == 2 and st["terms"] == 0


def test_known_answer_fixture_matches_oracle():
    ka = known()
    for case in ka["amplitudes"]:
        c = Circuit(case["num_qubits"])
        for op in case["ops"]:
            c.push(*op)
        s = O.OracleSim(c)
        for x, y, re, im in case["values"]:
            assert abs(s.amplitude(x, y) - complex(re, im)) < case["tol"]


def test_sampling_follows_the_distribution():
    # src/sim.rs:382-399 (shots reduced from 40000 to 4000, tolerance scaled by sqrt(10))
    c = Circuit(3)
    c.h(0).t(0).h(0).cx(0, 1).h(2).t(2).h(2).cz(1, 2).h(1).t(1).h(1)
    sv = O.dense_statevector(c, 0)
    sim = O.OracleSim(c)
    shots = 4000
    hist = np.bincount(sim.sample_many(0, shots, 1234), minlength=8)
    for y in range(8):
        assert abs(abs(sv[y]) ** 2 - hist[y] / shots) < 0.012 * 10 ** 0.5


def _mc_cases(seed, iters, nq, lo, hi):
    rng = Rng(seed)
    for _ in range(iters):
        c = random_layered(nq, 3, rng)
        sim = O.OracleSim(c)
        st = sim.stats()
        if st["branch_dim"] < lo or st["branch_dim"] > hi or st["pairs"] != 0:
            continue
        yield c, sim, rng.below(1 << nq)


def test_subspace_monte_carlo_is_unbiased():
    # src/approx.rs:188-207 (there 2^d <= samples: the exact fallback)
    tested = 0
    for c, sim, y in _mc_cases(61, 40, 4, 6, 12):
        tested += 1
        want = O.dense_statevector(c, 0)[y]
        re, im, se = sim.amplitude_estimate(0, y, 200_000, 3)
        assert abs(complex(re, im) - want) < 6.0 * se + 5e-3
    assert tested >= 3


def test_subspace_monte_carlo_sampled():
    # fewer samples than branches: the sampled estimate, unbiased within its standard error
    tested = 0
    for c, sim, y in _mc_cases(61, 40, 4, 6, 12):
        tested += 1
        want = O.dense_statevector(c, 0)[y]
        re, im, se = sim.amplitude_estimate(0, y, 40, 11)
        assert se > 0.0
        assert abs(complex(re, im) - want) < 6.0 * se + 5e-3
    assert tested >= 3


def _lazy_pair_cases(seed, trials):
    # the circuits of src/approx.rs:210-229: random_layered(3, 3) with at least 3 pair
    # candidates and at most 20 live path-sum variables; y drawn after the filter
    rng = Rng(seed)
    for _ in range(trials):
        c = random_layered(3, 3, rng)
        sim = O.OracleSim(c, "cached")
        cands, live = sim.path_info()
        if cands < 3 or live > 20:
            continue
        yield c, sim, rng.below(1 << 3)


def test_lazy_pair_sampling_is_unbiased():
    # src/approx.rs:210-229: estimate_amplitude(ps, io vars, boundary, 3 pairs, 4000 samples,
    # seed 5, exact dimension limit 20) within 6 standard errors + 5e-3 of the dense amplitude
    tested = 0
    for c, sim, y in _lazy_pair_cases(62, 30):
        tested += 1
        want = O.dense_statevector(c, 0)[y]
        re, im, se = sim.amplitude_estimate_pairs(0, y, 3, 4000, 5, 20)
        assert abs(complex(re, im) - want) < 6.0 * se + 5e-3, (re, im, se, want)
    assert tested >= 3


def test_lazy_pair_sampling_monte_carlo_branches():
    # exact dimension limit 0: every sampled branch engine goes through Engine::estimate (here
    # with its exact fallback, 2^d <= 2^14); same tolerance
    tested = 0
    for c, sim, y in _lazy_pair_cases(62, 30):
        tested += 1
        want = O.dense_statevector(c, 0)[y]
        re, im, se = sim.amplitude_estimate_pairs(0, y, 3, 400, 9, 0)
        assert abs(complex(re, im) - want) < 6.0 * se + 5e-3
    assert tested >= 3


def test_prepare_integers_agree_with_branch_phases():
    # the oracle's Engine::prepare record (src/engine.rs:569-610) against its own per-branch Z8
    # indices (src/normal_form.rs:479-493) for every branch engine: k0 is the index at s = 0,
    # Lp_j half the increment along kernel column j (always even), and a job vanishes exactly
    # when the branch phases are undefined
    rng = Rng(5)
    checked = 0
    for trial in range(40):
        n = 1 + rng.below(4)
        c = random_clifford_t(n, 10 + rng.below(14), rng.below(7), trial % 3 == 0, rng)
        for strat, p in (("cached", 0), ("auto", 0), ("pairs", 2)):
            sim = O.OracleSim(c, strat, p)
            xs = [0, (1 << n) - 1]
            ys = [rng.below(1 << n), rng.below(1 << n)]
            info = sim.prepare_info(xs, ys)
            for i in range(2):
                for b in range(sim.stats()["branches"]):
                    rec = info[i, b]
                    ph = sim.branch_phases(xs[i], ys[i], b)
                    assert (ph is None) == bool(rec[0])
                    if ph is None:
                        assert not rec[1:].any()
                        continue
                    d = sim.branch_dim(b)
                    assert int(rec[2]) == int(ph[0])
                    lp = rec[4:].view(np.uint8)
                    for j in range(d):
                        assert int(lp[j]) == ((int(ph[1 << j]) - int(ph[0])) % 8) // 2
                    assert not lp[d:].any()
                    checked += 1
    assert checked > 100


# The reference README's benchmark table (README.md:203-208, harness src/bin/benchmark.rs:10-28:
# random_layered(n, rounds) from Rng::new(1000 + n), input 0): T count, the cached engine's
# branch dimension d and the pairs Auto chooses are printed by the reference itself.
README_TABLE = [(10, 3, 20, 12, 3), (12, 2, 16, 7, 0)]


@pytest.mark.parametrize("n,rounds,t,d,pairs", README_TABLE)
def test_readme_benchmark_structure(n, rounds, t, d, pairs):
    c = random_layered(n, rounds, Rng(1000 + n))
    assert c.t_count() == t
    cached, auto = O.OracleSim(c, "cached"), O.OracleSim(c, "auto")
    assert cached.stats()["branch_dim"] == d
    assert auto.stats()["pairs"] == pairs
    # the library's host producer (no device needed) builds the same structures
    from polyq_gb300 import Simulator
    hc = Simulator(c, "cached", host_only=True).stats_full()
    ha = Simulator(c, "auto", host_only=True).stats_full()
    assert hc["branch_dim"] == d and ha["pairs"] == pairs
    for k in ("free_vars", "planes", "lines", "radical", "terms"):
        assert hc[k] == cached.stats()[k] and ha[k] == auto.stats()[k]
