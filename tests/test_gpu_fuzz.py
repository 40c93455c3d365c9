"""Randomised parity sweep: seeded circuits of varied size, T count and angle kind, every
strategy, and random launch shapes (chunk length, chunks per lane, warps, register budget,
chunks per load, chunk-sum tables), each against the oracle within the reported bound."""
import numpy as np
import pytest

import oracle as O
from polyq_gb300 import Simulator, get_tuning, set_tuning
from polyq_gb300.rng import Rng, random_outputs, workload_circuit

from test_gpu_parity import assert_amps

pytestmark = pytest.mark.gpu

SHAPES = [(10, 4, 8, 3, 4), (8, 1, 2, 4, 2), (9, 16, 4, 2, 8), (10, 2, 8, 2, 4), (8, 8, 8, 3, 1), (10, 16, 8, 2, 8)]


def test_random_circuits_and_shapes(gpu):
    old = get_tuning()
    rng = Rng(2024)
    tested = 0
    try:
        for case in range(60):
            n = 6 + rng.below(25)
            nt = 4 + rng.below(21)
            c = workload_circuit(n, 15 * n, nt, 1000 + case, rz_slots=bool(rng.below(2)))
            kind = rng.below(3)
            strategy, pairs = ("auto", None) if kind == 0 else (("cached", None) if kind == 1 else ("auto", rng.below(5)))
            if Simulator(c, strategy, pairs, host_only=True).stats_full()["branches_per_amplitude"] > 2.0 ** 21:
                continue
            di, cpl, bw, bps, unit = SHAPES[rng.below(len(SHAPES))]
            set_tuning(inner_dims=di, chunks_per_lane=cpl, block_warps=bw, blocks_per_sm=bps, unit_chunks=unit,
                       chunk_tables=1 + rng.below(2))
            sim = Simulator(c, strategy, pairs)
            ys = random_outputs(n, 6, case)
            got, err = sim.amplitudes([0] * 6, ys, with_error=True)
            ref = O.OracleSim(c, "pairs" if pairs is not None else strategy, pairs or 0)
            want = ref.amplitudes([0] * 6, ys)
            assert_amps(got, want, err)
            tested += 1
    finally:
        set_tuning(inner_dims=old["inner_dims"], chunks_per_lane=old["chunks_per_lane"], block_warps=old["block_warps"],
                   blocks_per_sm=old["blocks_per_sm"], unit_chunks=old["unit_chunks"], chunk_tables=2)
    assert tested >= 30
