"""SplitMix64 and the seeded circuit generators.

``Rng``, ``random_clifford_t`` and ``random_layered`` restate src/rng.rs:9-101 bit for
bit, so the reference's seeded test circuits can be regenerated.  The ``workload_*``
functions build the synthetic benchmark circuits (shapes of the five evaluation
configurations): gate slots are drawn from {H:0.3, S:0.2, CX:0.25, CZ:0.15, T:0.1}
conditioned on an exact T count, which is sampled exactly by placing the T slots
uniformly without replacement and drawing every other slot from the renormalised
{H:1/3, S:2/9, CX:5/18, CZ:1/6} mix on uniformly chosen distinct qubits.
"""
from __future__ import annotations

import math

from .circuit import Circuit, phase_from_pi_fraction

M64 = 0xFFFFFFFFFFFFFFFF
GOLDEN = 0x9E3779B97F4A7C15


class Rng:
    """SplitMix64 (src/rng.rs:9-31)."""

    def __init__(self, seed: int):
        self.state = (int(seed) + GOLDEN) & M64

    def next_u64(self) -> int:
        self.state = (self.state + GOLDEN) & M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)

    def next_f64(self) -> float:
        return (self.next_u64() >> 11) / float(1 << 53)

    def below(self, n: int) -> int:
        return self.next_u64() % n


def random_clifford_t(n: int, depth: int, t_count: int, generic_angles: bool, rng: Rng) -> Circuit:
    """src/rng.rs:36-74."""
    c = Circuit(n)
    t_left = t_count
    total = max(depth, t_count)
    for step in range(total):
        if t_left > 0 and (total - step <= t_left or rng.next_f64() < 0.3):
            q = rng.below(n)
            k = rng.below(4 if generic_angles else 2)
            if k == 0:
                c.t(q)
            elif k == 1:
                c.tdg(q)
            elif k == 2:
                c.p(q, phase_from_pi_fraction(1 + 2 * rng.below(7), 4))
            else:
                c.p(q, phase_from_pi_fraction(1 + 2 * rng.below(3), 3))
            t_left -= 1
            continue
        q = rng.below(n)
        r = rng.below(9 if n > 1 else 5)
        if r in (0, 1):
            c.h(q)
        elif r == 2:
            c.s(q)
        elif r == 3:
            c.z(q)
        elif r == 4:
            c.x(q)
        else:
            q2 = rng.below(n)
            while q2 == q:
                q2 = rng.below(n)
            if r in (5, 6):
                c.cz(q, q2)
            elif r == 7:
                c.cx(q, q2)
            else:
                c.swap(q, q2)
    return c


def random_layered(n: int, rounds: int, rng: Rng) -> Circuit:
    """src/rng.rs:79-101."""
    c = Circuit(n)
    for _ in range(rounds):
        for q in range(n):
            c.h(q)
        for q in range(n):
            k = rng.below(3)
            if k == 0:
                c.t(q)
            elif k == 1:
                c.tdg(q)
            else:
                c.s(q)
        if n > 1:
            for _ in range(n):
                a, b = rng.below(n), rng.below(n)
                if a != b:
                    c.cz(a, b)
    return c


# ----------------------------------------------------------------------------- workloads

def _distinct_pair(rng: Rng, n: int):
    a = rng.below(n)
    b = rng.below(n)
    while b == a:
        b = rng.below(n)
    return a, b


def workload_circuit(n: int, ngates: int, nt: int, seed: int, rz_slots: bool = False) -> Circuit:
    """Clifford+T circuit with exactly ``nt`` non-Clifford slots among ``ngates``.

    The non-Clifford slots are T gates, or rz(theta) with theta uniform in [0, 2*pi)
    when ``rz_slots`` is set.  Every other slot is H/S/CX/CZ with probabilities
    1/3, 2/9, 5/18, 1/6 on uniformly chosen distinct qubits.
    """
    rng = Rng(seed)
    slots = list(range(ngates))
    for i in range(nt):  # partial Fisher-Yates: nt distinct slots
        j = i + rng.below(ngates - i)
        slots[i], slots[j] = slots[j], slots[i]
    tset = set(slots[:nt])
    c = Circuit(n)
    for g in range(ngates):
        if g in tset:
            q = rng.below(n)
            if rz_slots:
                c.rz(q, 2.0 * math.pi * rng.next_f64())
            else:
                c.t(q)
            continue
        u = rng.next_f64()
        if u < 1.0 / 3.0:
            c.h(rng.below(n))
        elif u < 1.0 / 3.0 + 2.0 / 9.0:
            c.s(rng.below(n))
        elif u < 1.0 / 3.0 + 2.0 / 9.0 + 5.0 / 18.0:
            a, b = _distinct_pair(rng, n)
            c.cx(a, b)
        else:
            a, b = _distinct_pair(rng, n)
            c.cz(a, b)
    return c


def random_outputs(n: int, count: int, seed: int):
    """``count`` uniform n-bit output bitstrings (python ints, qubit q = bit q)."""
    rng = Rng(seed ^ 0x5DEECE66D)
    out = []
    for _ in range(count):
        v = 0
        for w in range((n + 63) // 64):
            v |= rng.next_u64() << (64 * w)
        out.append(v & ((1 << n) - 1))
    return out


def workload_small(seed: int = 1) -> Circuit:
    """Small single amplitude: n=20, 200 gates, 16 T."""
    return workload_circuit(20, 200, 16, seed)


def workload_many_boundaries(seed: int):
    """One circuit, many boundaries: n=50, 2000 gates, 32 T (caller picks the seed)."""
    return workload_circuit(50, 2000, 32, seed)


def workload_batch(num_circuits: int = 256, seed: int = 3, t_max: int = 36):
    """Uneven batch: n ~ U[16,64], 40n gates, T ~ U[8, t_max]; returns [(circuit, seed_i)]."""
    rng = Rng(seed)
    out = []
    for i in range(num_circuits):
        n = 16 + rng.below(49)
        nt = 8 + rng.below(t_max - 7)
        s = rng.next_u64() & 0xFFFFFFFF
        out.append((workload_circuit(n, 40 * n, nt, s), s))
    return out


def workload_rotations(n: int = 40, ngates: int = 1500, n_rz: int = 24, ccz_layers: int = 4,
                       ccz_per_layer: int = 8, seed: int = 4) -> Circuit:
    """Arbitrary-angle stress: rz(theta) slots plus layers of CCZ on disjoint random triples.

    CCZ layer L (L = 0..ccz_layers-1) is inserted after gate slot (L+1)*ngates/(ccz_layers+1)
    and expands through the 7-T Toffoli decomposition.
    """
    base = workload_circuit(n, ngates, n_rz, seed, rz_slots=True)
    rng = Rng(seed ^ 0xC0FFEE)
    cut = [(L + 1) * ngates // (ccz_layers + 1) for L in range(ccz_layers)]
    c = Circuit(n)
    pos = 0
    for L in range(ccz_layers):
        c.ops.extend(base.ops[pos:cut[L]])
        pos = cut[L]
        perm = list(range(n))
        for i in range(n - 1, 0, -1):
            j = rng.below(i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        for k in range(min(ccz_per_layer, n // 3)):
            a, b, t = perm[3 * k], perm[3 * k + 1], perm[3 * k + 2]
            c.ccz(a, b, t)
    c.ops.extend(base.ops[pos:])
    c.num_qubits = max(c.num_qubits, n)
    return c
