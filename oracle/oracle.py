"""CPU oracle for the polyq amplitude path -- TEST INFRASTRUCTURE ONLY.

ctypes front-end for ``pq_oracle.c``, a plain-C FP64 restatement of the reference
crate's compiler, normal form, cached engine, rank strategy, simulator and dense
statevector (file:line citations are in the C file).  Only the test-suite,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module; the
product library never does.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpq_oracle.so")
SRC = os.path.join(HERE, "pq_oracle.c")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile pq_oracle.c with gcc (no fused multiply-add, so x86-64 and aarch64 agree)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "pq_oracle.h"))
    ):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ct.CDLL(LIB_PATH)
            P = ct.c_void_p
            u8p, i32p, u32p, u64p, f64p, i64p = (ct.POINTER(t) for t in (
                ct.c_uint8, ct.c_int32, ct.c_uint32, ct.c_uint64, ct.c_double, ct.c_int64))
            L.pqo_sim_new.restype = P
            L.pqo_sim_new.argtypes = [ct.c_int, ct.c_int, u8p, i32p, i32p, u32p, ct.c_int, ct.c_int]
            L.pqo_sim_free.argtypes = [P]
            L.pqo_stats.argtypes = [P, i64p]
            L.pqo_amplitudes.argtypes = [P, ct.c_int, u64p, u64p, f64p, ct.c_int]
            L.pqo_last_branches.restype = ct.c_double
            L.pqo_last_branches.argtypes = [P]
            L.pqo_marginal.restype = ct.c_double
            L.pqo_marginal.argtypes = [P, u64p, ct.c_int, i32p, u8p]
            L.pqo_sample_many.argtypes = [P, u64p, ct.c_int64, ct.c_uint64, u64p]
            L.pqo_amplitude_estimate.argtypes = [P, u64p, u64p, ct.c_int64, ct.c_uint64, f64p]
            L.pqo_amplitude_estimate_pairs.argtypes = [P, u64p, u64p, ct.c_int, ct.c_int64, ct.c_uint64, ct.c_int, f64p]
            L.pqo_path_info.argtypes = [P, i64p]
            L.pqo_brute_force.restype = ct.c_int
            L.pqo_brute_force.argtypes = [P, u64p, u64p, f64p]
            L.pqo_dense_statevector.argtypes = [ct.c_int, ct.c_int, u8p, i32p, i32p, u32p, u64p, f64p]
            L.pqo_equivalence.restype = ct.c_int
            L.pqo_equivalence.argtypes = [ct.c_int, ct.c_int, u8p, i32p, i32p, u32p,
                                          ct.c_int, ct.c_int, u8p, i32p, i32p, u32p, ct.c_double, f64p]
            L.pqo_engine_dump.restype = ct.c_int64
            L.pqo_engine_dump.argtypes = [P, ct.c_int, u64p, ct.c_int64]
            L.pqo_branch_phases.restype = ct.c_int
            L.pqo_branch_phases.argtypes = [P, ct.c_int, u64p, u64p, u8p]
            L.pqo_branch_dim.restype = ct.c_int
            L.pqo_branch_dim.argtypes = [P, ct.c_int]
            L.pqo_prepare_info.argtypes = [P, ct.c_int, u64p, u64p, u64p]
            L.pqo_check_structure.restype = ct.c_int
            L.pqo_check_structure.argtypes = [ct.c_int, u8p, u8p, ct.c_int, i32p]
            L.pqo_gauss_sum.argtypes = [ct.c_int, u8p, u8p, u8p, ct.c_int, f64p, f64p]
            _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(ct.POINTER(t))


def _gate_arrays(circ):
    """circ: object with .num_qubits and .ops (list of (code, q0, q1, phase))."""
    ops = circ.ops
    n = len(ops)
    op = np.array([g[0] for g in ops] or [0], dtype=np.uint8)
    q0 = np.array([g[1] for g in ops] or [0], dtype=np.int32)
    q1 = np.array([g[2] for g in ops] or [0], dtype=np.int32)
    ph = np.array([g[3] for g in ops] or [0], dtype=np.uint32)
    return n, op, q0, q1, ph


def pack_bits(values, nq):
    """Pack integer bitstrings (python ints, qubit q = bit q) into (len, nw) uint64 words."""
    nw = max(1, (nq + 63) // 64)
    vals = list(values)
    out = np.zeros((len(vals), nw), dtype=np.uint64)
    for i, v in enumerate(vals):
        v = int(v)
        for w in range(nw):
            out[i, w] = (v >> (64 * w)) & 0xFFFFFFFFFFFFFFFF
    return out


STRATEGY = {"auto": 0, "cached": 1, "pairs": 2}
PREP_WORDS = 12  # u64 words per job of prepare_info (PQO_PREP_WORDS)


class OracleSim:
    """FP64 CPU restatement of ``Simulator::with_options`` (src/sim.rs:139-198)."""

    def __init__(self, circ, strategy="auto", pairs=0):
        self.L = lib()
        self.nq = circ.num_qubits
        n, op, q0, q1, ph = _gate_arrays(circ)
        self._keep = (op, q0, q1, ph)
        self.h = self.L.pqo_sim_new(self.nq, n, _ptr(op, ct.c_uint8), _ptr(q0, ct.c_int32), _ptr(q1, ct.c_int32),
                                    _ptr(ph, ct.c_uint32), STRATEGY[strategy], int(pairs))

    def __del__(self):
        try:
            if self.h:
                self.L.pqo_sim_free(self.h)
                self.h = None
        except Exception:
            pass

    def stats(self):
        out = np.zeros(8, dtype=np.int64)
        self.L.pqo_stats(self.h, _ptr(out, ct.c_int64))
        keys = ("free_vars", "planes", "lines", "radical", "terms", "branch_dim", "pairs", "branches")
        return dict(zip(keys, (int(v) for v in out)))

    def amplitudes(self, xs, ys, nthreads=0):
        xs = pack_bits(xs, self.nq)
        ys = pack_bits(ys, self.nq)
        n = xs.shape[0]
        out = np.zeros(2 * max(n, 1), dtype=np.float64)
        self.L.pqo_amplitudes(self.h, n, _ptr(xs, ct.c_uint64), _ptr(ys, ct.c_uint64), _ptr(out, ct.c_double),
                              int(nthreads))
        return out[: 2 * n].view(np.complex128)

    def amplitude(self, x, y):
        return complex(self.amplitudes([x], [y])[0])

    def last_branches(self):
        """Branches enumerated by the last amplitudes() call (vanishing jobs excluded)."""
        return float(self.L.pqo_last_branches(self.h))

    def probability(self, x, y):
        return abs(self.amplitude(x, y)) ** 2

    def marginal(self, x, measured):
        xs = pack_bits([x], self.nq)
        qs = np.array([q for q, _ in measured] or [0], dtype=np.int32)
        bs = np.array([int(b) for _, b in measured] or [0], dtype=np.uint8)
        return float(self.L.pqo_marginal(self.h, _ptr(xs, ct.c_uint64), len(measured), _ptr(qs, ct.c_int32),
                                         _ptr(bs, ct.c_uint8)))

    def amplitude_estimate(self, x, y, samples, seed):
        """Simulator::amplitude_estimate (src/sim.rs:184-193): (re, im, standard error)."""
        xs = pack_bits([x], self.nq)
        ys = pack_bits([y], self.nq)
        out = np.zeros(3, dtype=np.float64)
        self.L.pqo_amplitude_estimate(self.h, _ptr(xs, ct.c_uint64), _ptr(ys, ct.c_uint64), samples,
                                      ct.c_uint64(seed & (2**64 - 1)), _ptr(out, ct.c_double))
        return float(out[0]), float(out[1]), float(out[2])

    def path_info(self):
        """(pair candidates with the io variables fixed, live variables) of the path sum."""
        out = np.zeros(2, dtype=np.int64)
        self.L.pqo_path_info(self.h, _ptr(out, ct.c_int64))
        return int(out[0]), int(out[1])

    def amplitude_estimate_pairs(self, x, y, pairs, samples, seed, exact_dim_limit=20):
        """approx::estimate_amplitude (src/approx.rs:96-135): (re, im, standard error)."""
        xs = pack_bits([x], self.nq)
        ys = pack_bits([y], self.nq)
        out = np.zeros(3, dtype=np.float64)
        self.L.pqo_amplitude_estimate_pairs(self.h, _ptr(xs, ct.c_uint64), _ptr(ys, ct.c_uint64), pairs, samples,
                                            ct.c_uint64(seed & (2**64 - 1)), exact_dim_limit, _ptr(out, ct.c_double))
        return float(out[0]), float(out[1]), float(out[2])

    def sample_many(self, x, shots, seed):
        """Simulator::sample_many (src/sim.rs:272-284): shots basis-state indices."""
        xs = pack_bits([x], self.nq)
        nw = xs.shape[1]
        out = np.zeros((shots, nw), dtype=np.uint64)
        self.L.pqo_sample_many(self.h, _ptr(xs, ct.c_uint64), shots, ct.c_uint64(seed & (2**64 - 1)),
                               _ptr(out, ct.c_uint64))
        return [sum(int(out[i, w]) << (64 * w) for w in range(nw)) for i in range(shots)]

    def brute_force(self, x, y):
        xs = pack_bits([x], self.nq)
        ys = pack_bits([y], self.nq)
        out = np.zeros(2, dtype=np.float64)
        rc = self.L.pqo_brute_force(self.h, _ptr(xs, ct.c_uint64), _ptr(ys, ct.c_uint64), _ptr(out, ct.c_double))
        if rc != 0:
            raise ValueError("brute force over more than 26 free variables")
        return complex(out[0], out[1])

    def engine_dump(self, branch=0):
        n = self.L.pqo_engine_dump(self.h, branch, None, 0)
        out = np.zeros(max(n, 1), dtype=np.uint64)
        self.L.pqo_engine_dump(self.h, branch, _ptr(out, ct.c_uint64), n)
        return out[:n]

    def branch_dim(self, branch=0):
        """Dimension d of branch engine `branch`'s affine branch subspace."""
        d = int(self.L.pqo_branch_dim(self.h, branch))
        if d < 0:
            raise ValueError("no branch engine %d" % branch)
        return d

    def prepare_info(self, xs, ys):
        """Engine::prepare integers (src/engine.rs:569-610) of every (boundary, branch engine)
        job, boundary-major: an (n, branches, PREP_WORDS) uint64 array -- vanish flag, constant
        phase, k0, pivot bits y0, then the Z4 increments Lp_j as bytes (0xFF: odd)."""
        xs = pack_bits(xs, self.nq)
        ys = pack_bits(ys, self.nq)
        n = xs.shape[0]
        nb = self.stats()["branches"]
        out = np.zeros((max(n, 1), nb, PREP_WORDS), dtype=np.uint64)
        self.L.pqo_prepare_info(self.h, n, _ptr(xs, ct.c_uint64), _ptr(ys, ct.c_uint64), _ptr(out, ct.c_uint64))
        return out[:n]

    def branch_phases(self, x, y, branch=0):
        d = self.branch_dim(branch)
        if d > 24:
            raise ValueError("d too large")
        xs = pack_bits([x], self.nq)
        ys = pack_bits([y], self.nq)
        out = np.zeros(1 << d, dtype=np.uint8)
        rc = self.L.pqo_branch_phases(self.h, branch, _ptr(xs, ct.c_uint64), _ptr(ys, ct.c_uint64),
                                      _ptr(out, ct.c_uint8))
        return None if rc < 0 else out


def dense_statevector(circ, x=0):
    L = lib()
    n, op, q0, q1, ph = _gate_arrays(circ)
    nq = circ.num_qubits
    xs = pack_bits([x], nq)
    out = np.zeros(2 << nq, dtype=np.float64)
    L.pqo_dense_statevector(nq, n, _ptr(op, ct.c_uint8), _ptr(q0, ct.c_int32), _ptr(q1, ct.c_int32),
                            _ptr(ph, ct.c_uint32), _ptr(xs, ct.c_uint64), _ptr(out, ct.c_double))
    return out.view(np.complex128)


def equivalence(c1, c2, tol=1e-9):
    L = lib()
    a = _gate_arrays(c1)
    b = _gate_arrays(c2)
    out = np.zeros(2, dtype=np.float64)
    eq = L.pqo_equivalence(c1.num_qubits, a[0], _ptr(a[1], ct.c_uint8), _ptr(a[2], ct.c_int32), _ptr(a[3], ct.c_int32),
                           _ptr(a[4], ct.c_uint32), c2.num_qubits, b[0], _ptr(b[1], ct.c_uint8), _ptr(b[2], ct.c_int32),
                           _ptr(b[3], ct.c_int32), _ptr(b[4], ct.c_uint32), tol, _ptr(out, ct.c_double))
    return bool(eq), complex(out[0], out[1])


def check_structure(bmat, parity, rule):
    L = lib()
    m = int(parity.shape[0])
    bm = np.ascontiguousarray(bmat, dtype=np.uint8)
    par = np.ascontiguousarray(parity, dtype=np.uint8)
    sizes = np.zeros(3, dtype=np.int32)
    rc = L.pqo_check_structure(m, _ptr(bm, ct.c_uint8), _ptr(par, ct.c_uint8), int(rule), _ptr(sizes, ct.c_int32))
    return rc, tuple(int(v) for v in sizes)


def gauss_sum(bmat, v, shift, rule):
    L = lib()
    m = int(v.shape[0])
    bm = np.ascontiguousarray(bmat, dtype=np.uint8)
    vv = np.ascontiguousarray(v, dtype=np.uint8)
    sh = np.ascontiguousarray(shift, dtype=np.uint8)
    a = np.zeros(2, dtype=np.float64)
    b = np.zeros(2, dtype=np.float64)
    L.pqo_gauss_sum(m, _ptr(bm, ct.c_uint8), _ptr(vv, ct.c_uint8), _ptr(sh, ct.c_uint8), int(rule),
                    _ptr(a, ct.c_double), _ptr(b, ct.c_double))
    return complex(a[0], a[1]), complex(b[0], b[1])
