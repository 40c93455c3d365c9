"""Python front-end of the GB300 amplitude path, with the reference's Simulator surface.

``Simulator(circuit, strategy="auto", pairs=None)`` mirrors the reference's Python class
(src/pybind.rs:133-181) and ``Simulator::with_options`` (src/sim.rs:144): amplitude(x, y)
returns (re, im), probability(x, y) returns |amplitude|^2, marginal(x, [(q, b), ...]),
stats() returns (free_vars, planes, lines, radical, terms, branch_dim, pairs).  Batched
variants take sequences of integer bitstrings (qubit q = bit q).
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _native as N
from .circuit import Circuit

STRATEGIES = {"auto": 0, "cached": 1}


def parse_strategy(strategy: str, pairs):
    """src/pybind.rs:124-131: an explicit pair count wins, else 'auto' or 'cached'."""
    if pairs is not None:
        if int(pairs) < 0:
            raise ValueError("pairs must be non-negative")
        return 2, int(pairs)
    if strategy not in STRATEGIES:
        raise ValueError("strategy must be 'auto' or 'cached'")
    return STRATEGIES[strategy], 0


def pack_bits(values, nq: int) -> np.ndarray:
    """Integer bitstrings -> (n, ceil(nq/64)) little-endian uint64 words."""
    nw = max(1, (nq + 63) // 64)
    if nw == 1:
        # one word per bitstring: converted and checked as an array
        if isinstance(values, np.ndarray) and values.dtype.kind in "iu":
            arr = values.reshape(-1)
            if arr.dtype.kind == "i" and arr.size and int(arr.min()) < 0:
                raise ValueError("negative bitstring")
            arr = arr.astype(np.uint64)
        else:
            try:
                arr = np.fromiter((int(v) for v in values), dtype=np.uint64)
            except OverflowError:
                raise ValueError("bitstring does not fit %d qubits" % nq) from None
        if nq < 64 and arr.size and int((arr >> np.uint64(nq)).max()) != 0:
            raise ValueError("bitstring %d does not fit %d qubits" % (int(arr[(arr >> np.uint64(nq)) != 0][0]), nq))
        return arr.reshape(-1, 1)
    vals = [int(v) for v in values]
    out = np.zeros((len(vals), nw), dtype=np.uint64)
    for i, v in enumerate(vals):
        if v < 0 or (v >> nq) != 0:
            raise ValueError("bitstring %d does not fit %d qubits" % (v, nq))
        for w in range(nw):
            out[i, w] = (v >> (64 * w)) & 0xFFFFFFFFFFFFFFFF
    return out


def _p(a, t):
    return a.ctypes.data_as(ct.POINTER(t))


def _desc(circ: Circuit):
    n, op, q0, q1, ph = circ.arrays()
    d = N.CircuitDesc(circ.num_qubits, n, _p(op, ct.c_uint8), _p(q0, ct.c_int32), _p(q1, ct.c_int32),
                      _p(ph, ct.c_uint32))
    return d, (op, q0, q1, ph)


class Simulator:
    """Resident GB300 simulator of one circuit (structures uploaded once, kept in HBM)."""

    def __init__(self, circuit: Circuit, strategy: str = "auto", pairs=None, host_only: bool = False):
        self._L = N.lib()
        st, p = parse_strategy(strategy, pairs)
        self.num_qubits = circuit.num_qubits
        self.circuit = circuit
        self.nw = max(1, (self.num_qubits + 63) // 64)
        d, keep = _desc(circuit)
        h = ct.c_void_p()
        create = self._L.pq_analyze if host_only else self._L.pq_sim_create
        N.check(create(ct.byref(d), st, p, ct.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._L.pq_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats_full(self) -> dict:
        s = N.Stats()
        N.check(self._L.pq_sim_stats(self._h, ct.byref(s)))
        return {k: getattr(s, k) for k, _ in N.Stats._fields_}

    def stats(self):
        """(free_vars, planes, lines, radical, terms, branch_dim, pairs) -- src/pybind.rs:177-180."""
        s = self.stats_full()
        return (s["free_vars"], s["planes"], s["lines"], s["radical"], s["terms"], s["branch_dim"], s["pairs"])

    def pairs(self) -> int:
        return self.stats_full()["pairs"]

    # ------------------------------------------------------------------ amplitudes
    def amplitudes(self, inputs, outputs, with_error: bool = False):
        xs = pack_bits(inputs, self.num_qubits)
        ys = pack_bits(outputs, self.num_qubits)
        if xs.shape[0] != ys.shape[0]:
            raise ValueError("inputs and outputs differ in length")
        n = xs.shape[0]
        out = np.zeros(2 * n, dtype=np.float64)
        err = np.zeros(n, dtype=np.float64)
        N.check(self._L.pq_amplitudes(self._h, n, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), _p(out, ct.c_double),
                                      _p(err, ct.c_double)))
        amps = out.view(np.complex128)
        return (amps, err) if with_error else amps

    def amplitude(self, input: int, output: int):
        """src/pybind.rs:146-149: (re, im) of <output|C|input>."""
        a = complex(self.amplitudes([input], [output])[0])
        return (a.real, a.imag)

    def probabilities(self, inputs, outputs):
        xs = pack_bits(inputs, self.num_qubits)
        ys = pack_bits(outputs, self.num_qubits)
        n = xs.shape[0]
        out = np.zeros(n, dtype=np.float64)
        N.check(self._L.pq_probabilities(self._h, n, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), _p(out, ct.c_double)))
        return out

    def probability(self, input: int, output: int) -> float:
        """src/pybind.rs:155-157."""
        return float(self.probabilities([input], [output])[0])

    def set_resident(self, idle_seconds: float):
        """Low-latency single amplitudes: one-boundary calls served by a resident kernel that
        returns after idle_seconds without a request (0 turns the mode off)."""
        N.check(self._L.pq_sim_set_resident(self._h, float(idle_seconds)))

    def amplitudes_plain(self, inputs, outputs):
        xs = pack_bits(inputs, self.num_qubits)
        ys = pack_bits(outputs, self.num_qubits)
        n = xs.shape[0]
        out = np.zeros(2 * n, dtype=np.float64)
        N.check(self._L.pq_amplitudes_plain(self._h, n, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64),
                                            _p(out, ct.c_double)))
        return out.view(np.complex128)

    def autotune(self, inputs, outputs, reps: int = 3):
        """Pick the fastest launch shape for boundaries like these (pq_sim_autotune); returns
        (tuning dict, device ms of one launch)."""
        xs = pack_bits(inputs, self.num_qubits)
        ys = pack_bits(outputs, self.num_qubits)
        t = N.Tuning()
        ms = ct.c_double(0.0)
        N.check(self._L.pq_sim_autotune(self._h, xs.shape[0], _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), reps,
                                        ct.byref(t), ct.byref(ms)))
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}, ms.value

    def tuning(self) -> dict:
        t = N.Tuning()
        N.check(self._L.pq_sim_get_tuning(self._h, ct.byref(t)))
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}

    def engine_shape(self, branch: int) -> dict:
        """d, pivots, table low coordinates, joint table, pair coordinate, pivot-free coordinates."""
        out = np.zeros(8, dtype=np.int64)
        N.check(self._L.pq_debug_engine_shape(self._h, branch, _p(out, ct.c_int64)))
        keys = ("d", "rank", "DI", "joint", "pairc", "free_of_pivots", "free_of_pivots_high", "terms")
        return dict(zip(keys, (int(v) for v in out)))

    def amplitudes_fp64(self, inputs, outputs):
        xs = pack_bits(inputs, self.num_qubits)
        ys = pack_bits(outputs, self.num_qubits)
        n = xs.shape[0]
        out = np.zeros(2 * n, dtype=np.float64)
        N.check(self._L.pq_amplitudes_fp64(self._h, n, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64),
                                           _p(out, ct.c_double)))
        return out.view(np.complex128)

    def marginal(self, input: int, measured) -> float:
        """src/pybind.rs:173-176 / src/sim.rs:225-231: P(measured qubits give these outcomes)."""
        xs = pack_bits([input], self.num_qubits)
        qs = np.array([int(q) for q, _ in measured] or [0], dtype=np.int32)
        bs = np.array([int(bool(b)) for _, b in measured] or [0], dtype=np.uint8)
        out = np.zeros(1, dtype=np.float64)
        N.check(self._L.pq_marginal(self._h, _p(xs, ct.c_uint64), len(measured), _p(qs, ct.c_int32),
                                    _p(bs, ct.c_uint8), _p(out, ct.c_double)))
        return float(out[0])

    def amplitude_estimate(self, input: int, output: int, samples: int, seed: int):
        """src/pybind.rs:150-153 / src/sim.rs:184-193: (re, im, standard_error) of an unbiased
        Monte-Carlo estimate of <output|C|input>."""
        xs = pack_bits([input], self.num_qubits)
        ys = pack_bits([output], self.num_qubits)
        out = np.zeros(2, dtype=np.float64)
        se = np.zeros(1, dtype=np.float64)
        N.check(self._L.pq_amplitude_estimate(self._h, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), int(samples),
                                              ct.c_uint64(seed & (2**64 - 1)), _p(out, ct.c_double),
                                              _p(se, ct.c_double)))
        return float(out[0]), float(out[1]), float(se[0])

    def amplitude_estimate_pairs(self, input: int, output: int, pairs: int, samples: int, seed: int,
                                 exact_dim_limit: int = 20):
        """src/approx.rs:96-135 (estimate_amplitude): (re, im, standard_error) of the lazy
        pair-sampling estimate of <output|C|input> -- `samples` random patterns of the first
        `pairs` pair candidates, each branch engine built on the fly and evaluated exactly (or by
        Monte Carlo above `exact_dim_limit`)."""
        xs = pack_bits([input], self.num_qubits)
        ys = pack_bits([output], self.num_qubits)
        out = np.zeros(2, dtype=np.float64)
        se = np.zeros(1, dtype=np.float64)
        N.check(self._L.pq_amplitude_estimate_pairs(self._h, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), int(pairs),
                                                    int(samples), ct.c_uint64(seed & (2**64 - 1)),
                                                    int(exact_dim_limit), _p(out, ct.c_double), _p(se, ct.c_double)))
        return float(out[0]), float(out[1]), float(se[0])

    def sample_many(self, input: int, shots: int, seed: int):
        """src/sim.rs:272-284 / src/pybind.rs sample_many: `shots` measurement outcomes of C|input>
        as basis-state indices (the reference's SplitMix64 streams: same seed, same samples)."""
        xs = pack_bits([input], self.num_qubits)
        nw = xs.shape[1]
        out = np.zeros((int(shots), nw), dtype=np.uint64)
        N.check(self._L.pq_sample_many(self._h, _p(xs, ct.c_uint64), int(shots), ct.c_uint64(seed & (2**64 - 1)),
                                       _p(out, ct.c_uint64)))
        return [sum(int(out[i, w]) << (64 * w) for w in range(nw)) for i in range(int(shots))]

    def statevector(self, input: int = 0) -> np.ndarray:
        """All 2^n amplitudes for one input (src/sim.rs:201-213), as one batched launch."""
        n = self.num_qubits
        if n > 24:
            raise ValueError("statevector limited to 24 qubits")
        return self.amplitudes(np.full(1 << n, input, dtype=np.uint64), np.arange(1 << n, dtype=np.uint64))

    # ------------------------------------------------------------------ checks
    def engine_dump(self, branch: int = 0) -> np.ndarray:
        n = self._L.pq_debug_engine_dump(self._h, branch, None, 0)
        if n < 0:
            raise N.PqError(1, self._L.pq_last_error().decode())
        out = np.zeros(max(n, 1), dtype=np.uint64)
        self._L.pq_debug_engine_dump(self._h, branch, _p(out, ct.c_uint64), n)
        return out[:n]

    def branch_phases(self, input: int, output: int, branch: int = 0):
        d = self.engine_shape(branch)["d"]
        if d > 24:
            raise ValueError("branch dimension above 24")
        xs = pack_bits([input], self.num_qubits)
        ys = pack_bits([output], self.num_qubits)
        buf = np.zeros(max(1, 1 << d), dtype=np.uint8)
        r = self._L.pq_debug_branch_phases(self._h, branch, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64),
                                           _p(buf, ct.c_uint8))
        if r == -2:
            raise N.PqError(8, self._L.pq_last_error().decode())
        if r == -1:
            return None
        return buf[: 1 << r]


    def prepare_info(self, inputs, outputs) -> np.ndarray:
        """Engine::prepare integers as the device computes them (pq_debug_prepare): an
        (n, branch engines, 12) uint64 array -- vanish flag, constant phase, k0, pivot bits
        y0, then the Z4 increments Lp_j as bytes in the reference's coordinate order."""
        xs = pack_bits(inputs, self.num_qubits)
        ys = pack_bits(outputs, self.num_qubits)
        n = xs.shape[0]
        nb = self.stats_full()["num_branches"]
        out = np.zeros((n, nb, 12), dtype=np.uint64)
        N.check(self._L.pq_debug_prepare(self._h, n, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64),
                                         _p(out, ct.c_uint64)))
        return out


class Batch:
    """Amplitudes of many circuits' boundaries in one persistent, graph-captured launch."""

    def __init__(self, sims, counts):
        self._L = N.lib()
        self.sims = list(sims)
        self.counts = [int(c) for c in counts]
        arr = (ct.c_void_p * len(self.sims))(*[s.handle for s in self.sims])
        cnt = np.array(self.counts, dtype=np.int64)
        h = ct.c_void_p()
        N.check(self._L.pq_batch_create(len(self.sims), arr, _p(cnt, ct.c_int64), ct.byref(h)))
        self._h = h
        self.nw = int(self._L.pq_batch_words(h))
        self.branches = int(self._L.pq_batch_branches(h))

    def pack(self, inputs, outputs):
        """Per-circuit lists of boundaries -> the concatenated word arrays."""
        xs, ys = [], []
        for s, xi, yi in zip(self.sims, inputs, outputs):
            nq = 64 * self.nw
            xs.append(pack_bits(xi, nq))
            ys.append(pack_bits(yi, nq))
        return np.ascontiguousarray(np.concatenate(xs)), np.ascontiguousarray(np.concatenate(ys))

    def run(self, xs, ys, with_error=False):
        n = sum(self.counts)
        out = np.zeros(2 * n, dtype=np.float64)
        err = np.zeros(n, dtype=np.float64)
        N.check(self._L.pq_batch_run(self._h, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), _p(out, ct.c_double),
                                     _p(err, ct.c_double)))
        amps = out.view(np.complex128)
        return (amps, err) if with_error else amps

    def autotune(self, xs, ys, reps: int = 3):
        """Pick the fastest launch shape for this batch on packed boundaries (pq_batch_autotune);
        returns (tuning dict, device ms of one launch)."""
        t = N.Tuning()
        ms = ct.c_double(0.0)
        N.check(self._L.pq_batch_autotune(self._h, _p(xs, ct.c_uint64), _p(ys, ct.c_uint64), reps, ct.byref(t),
                                          ct.byref(ms)))
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}, ms.value

    def run_device(self, x_ptr, y_ptr, out_ptr, err_ptr=None, stream=None):
        N.check(self._L.pq_batch_run_device(self._h, x_ptr, y_ptr, out_ptr, err_ptr, stream))

    def close(self):
        if getattr(self, "_h", None):
            self._L.pq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_tuning(inner_dims=0, chunks_per_lane=0, block_warps=0, max_branch_dim=0, blocks_per_sm=0, unit_chunks=0,
               chunk_tables=0):
    """Defaults for simulators and batches created afterwards (0 keeps a field unchanged)."""
    t = N.Tuning(inner_dims, chunks_per_lane, block_warps, max_branch_dim, blocks_per_sm, unit_chunks, chunk_tables)
    N.check(N.lib().pq_set_default_tuning(ct.byref(t)))


def get_tuning() -> dict:
    t = N.Tuning()
    N.check(N.lib().pq_get_default_tuning(ct.byref(t)))
    return {k: getattr(t, k) for k, _ in N.Tuning._fields_}
