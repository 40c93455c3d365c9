"""Simulator::amplitude_estimate on the device (src/sim.rs:184-193, src/rank.rs:149-171,
src/engine.rs:616-659): the same seeds draw the same samples as the oracle's restatement."""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator
from polyq_gb300.rng import Rng, random_layered, workload_many_boundaries, workload_small

pytestmark = pytest.mark.gpu


def test_exact_fallback_and_unbiased(gpu):
    # src/approx.rs:188-207 on the device
    rng = Rng(61)
    tested = 0
    for _ in range(40):
        c = random_layered(4, 3, rng)
        sim = Simulator(c)
        st = sim.stats_full()
        if st["branch_dim"] < 6 or st["branch_dim"] > 12 or st["pairs"] != 0:
            continue
        tested += 1
        y = rng.below(16)
        want = O.dense_statevector(c, 0)[y]
        re, im, se = sim.amplitude_estimate(0, y, 200_000, 3)
        assert abs(complex(re, im) - want) < 6.0 * se + 5e-3
        re2, im2, se2 = sim.amplitude_estimate(0, y, 40, 11)  # sampled
        ore, oim, ose = O.OracleSim(c).amplitude_estimate(0, y, 40, 11)
        assert abs(complex(re2, im2) - complex(ore, oim)) <= 1e-9 * max(1.0, abs(complex(ore, oim)))
        assert se2 == pytest.approx(ose, rel=1e-9, abs=1e-12)
    assert tested >= 3


def test_sampled_single_engine_matches_oracle(gpu):
    # one cached engine of d = 29 sampled 20000 times: the oracle walks the same points
    c = workload_many_boundaries(0)
    sim = Simulator(c, "cached")
    ref = O.OracleSim(c, "cached")
    for y, seed in ((0, 5), (123456789, 6)):
        got = sim.amplitude_estimate(0, y, 20000, seed)
        want = ref.amplitude_estimate(0, y, 20000, seed)
        scale = max(abs(complex(want[0], want[1])), want[2], 1e-300)
        assert abs(complex(got[0], got[1]) - complex(want[0], want[1])) <= 1e-9 * scale
        assert got[2] == pytest.approx(want[2], rel=1e-9)


def test_branch_sampling_matches_oracle(gpu):
    # 2^p stabiliser branches (Pairs(2)): sampled branch engines evaluated exactly
    c = workload_small(2)
    sim = Simulator(c, pairs=2)
    assert sim.stats_full()["num_branches"] == 4
    ref = O.OracleSim(c, "pairs", 2)
    got = sim.amplitude_estimate(0, 0, 500, 9)
    want = ref.amplitude_estimate(0, 0, 500, 9)
    scale = max(abs(complex(want[0], want[1])), want[2], 1e-12)
    assert abs(complex(got[0], got[1]) - complex(want[0], want[1])) <= 1e-6 * scale
    assert got[2] == pytest.approx(want[2], rel=1e-6, abs=1e-12)


@pytest.mark.parametrize("per_layer", [2, 3, 8])
def test_sampled_large_subspace_matches_oracle(gpu, per_layer):
    # rotations with CCZ layers, one cached engine of d = 77, 104 and 239 (the last is the
    # rotation workload as written): points of more than one 64-bit word, the same draws
    from polyq_gb300.rng import workload_rotations
    c = workload_rotations(n=40, ngates=1500, n_rz=24, ccz_layers=4, ccz_per_layer=per_layer, seed=4)
    sim = Simulator(c, "cached")
    assert sim.stats_full()["branch_dim"] > 64
    ref = O.OracleSim(c, "cached")
    for y, seed in ((12345, 7), (0, 8)):
        got = sim.amplitude_estimate(0, y, 3000, seed)
        want = ref.amplitude_estimate(0, y, 3000, seed)
        scale = max(abs(complex(want[0], want[1])), want[2], 1e-300)
        assert abs(complex(got[0], got[1]) - complex(want[0], want[1])) <= 1e-9 * scale
        assert got[2] == pytest.approx(want[2], rel=1e-9)


def test_lazy_pair_sampling_matches_oracle(gpu):
    # src/approx.rs:96-135 on the device: the same draws as the oracle's restatement.  Exact
    # branches (the circuits of src/approx.rs:210-229): FP32 walk vs FP64, and unbiased within
    # 6 standard errors + 5e-3 of the dense amplitude
    rng = Rng(62)
    tested = 0
    for _ in range(30):
        c = random_layered(3, 3, rng)
        ref = O.OracleSim(c, "cached")
        cands, live = ref.path_info()
        if cands < 3 or live > 20:
            continue
        tested += 1
        y = rng.below(8)
        sim = Simulator(c, "cached")
        re, im, se = sim.amplitude_estimate_pairs(0, y, 3, 4000, 5, 20)
        ore, oim, ose = ref.amplitude_estimate_pairs(0, y, 3, 4000, 5, 20)
        assert abs(complex(re, im) - complex(ore, oim)) <= 1e-9
        assert se == pytest.approx(ose, rel=1e-6, abs=1e-9)
        want = O.dense_statevector(c, 0)[y]
        assert abs(complex(re, im) - want) < 6.0 * se + 5e-3
    assert tested >= 3
    # Monte-Carlo branches: 2 pairs of the many-boundaries circuit leave branch engines of
    # d ~ 25 > the limit 10, estimated with 2^14 points each from the sample's own seed
    from polyq_gb300.rng import random_outputs
    c = workload_many_boundaries(0)
    y = random_outputs(50, 1, 3)[0]
    sim = Simulator(c, "cached")
    ref = O.OracleSim(c, "cached")
    got = sim.amplitude_estimate_pairs(0, y, 2, 12, 7, 10)
    want = ref.amplitude_estimate_pairs(0, y, 2, 12, 7, 10)
    scale = max(abs(complex(want[0], want[1])), want[2], 1e-300)
    assert abs(complex(got[0], got[1]) - complex(want[0], want[1])) <= 1e-9 * scale
    assert got[2] == pytest.approx(want[2], rel=1e-6)
