"""The enumeration's bucket walk (units of 4 or 8 chunks summed as Walsh buckets, 8- and 16-point
groups) against the FP64 oracle, across the launch shapes that select its variants: chunk
lengths 2^8..2^10, units of 8 chunks (128-register build) and of 4 (a fourth-size unit and the
80-register build, which splits units of 8 into two of 4), on circuits whose branch engines
have d = 12..22 and 0..3 T-pairs."""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator, get_tuning, set_tuning
from polyq_gb300.rng import random_outputs, workload_circuit

pytestmark = pytest.mark.gpu

CIRCUITS = [(24, 400, 20, 1), (30, 600, 26, 4), (28, 500, 24, 6), (30, 600, 24, 3)]
SHAPES = [  # inner_dims, blocks_per_sm, unit_chunks
    (10, 2, 8), (9, 2, 8), (8, 2, 8), (10, 3, 8), (10, 2, 4)]


@pytest.mark.parametrize("shape", SHAPES)
def test_bucket_walk_matches_oracle(gpu, shape):
    inner, bps, unit = shape
    old = get_tuning()
    try:
        set_tuning(inner_dims=inner, blocks_per_sm=bps, unit_chunks=unit)
        checked = 0
        for n, g, t, seed in CIRCUITS:
            c = workload_circuit(n, g, t, seed)
            for strat in ("auto", "cached"):
                ref = O.OracleSim(c, strat)
                ys = random_outputs(n, 16, 100 + seed)
                xs = [0] * len(ys)
                sim = Simulator(c, strat)
                got, err = sim.amplitudes(xs, ys, with_error=True)
                want = np.asarray(ref.amplitudes(xs, ys))
                # the sums are enumerated, not zeros of a failed radical system
                assert np.count_nonzero(want) >= 8, (seed, strat)
                diff = np.abs(got - want)
                scale = float(np.max(np.abs(want)))
                # every result within its reported bound (plus the FP64 reference's own rounding)
                assert np.all(diff <= err + 1e-13 * max(scale, 1.0)), (shape, seed, strat)
                big = np.abs(want) >= 1e-3 * scale
                assert np.all(diff[big] <= 1e-6 * np.abs(want[big])), (shape, seed, strat)
                checked += len(ys)
        assert checked >= 2 * 8 * len(CIRCUITS)
    finally:
        set_tuning(inner_dims=old["inner_dims"], blocks_per_sm=old["blocks_per_sm"],
                   unit_chunks=old["unit_chunks"])
