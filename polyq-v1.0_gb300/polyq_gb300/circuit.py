"""Gate set, circuits and the dyadic phase ring.

Restates the reference's ``Circuit`` builders (src/circuit.rs:97-216) and ``Phase``
constructors (src/phase.rs:38-57).  A circuit is a list of ``(code, q0, q1, phase)``
tuples; the codes are the ones the C-ABI takes in ``pq_circuit_desc``.
"""
from __future__ import annotations

import math

H, X, Y, Z, S, SDG, T, TDG, P, CZ, CX, SWAP, GPHASE = range(13)
GATE_NAMES = ("H", "X", "Y", "Z", "S", "SDG", "T", "TDG", "P", "CZ", "CX", "SWAP", "GPHASE")

MASK32 = 0xFFFFFFFF
PHASE_PI = 1 << 31
PHASE_HALF_PI = 1 << 30
PHASE_QUARTER_PI = 1 << 29


def phase_from_radians(radians: float) -> int:
    """Nearest point of the 2^32 grid (src/phase.rs:39-44; round half away from zero)."""
    turns = radians / (2.0 * math.pi)
    frac = turns - math.floor(turns)
    k = math.floor(frac * 4294967296.0 + 0.5)
    return int(k) & MASK32


def phase_from_pi_fraction(num: int, log2_den: int) -> int:
    """Exact angle pi*num/2^log2_den (src/phase.rs:47-52)."""
    if not 0 <= log2_den <= 31:
        raise ValueError("denominator too fine for the 2^32 phase ring")
    return (num << (31 - log2_den)) % (1 << 32)


def phase_to_radians(p: int) -> float:
    return 2.0 * math.pi * float(p) / 4294967296.0


class Circuit:
    """Ordered gate list on ``num_qubits`` wires (src/circuit.rs:79-110)."""

    def __init__(self, num_qubits: int = 0):
        self.num_qubits = int(num_qubits)
        self.ops: list[tuple[int, int, int, int]] = []

    def __len__(self):
        return len(self.ops)

    def push(self, code: int, q0: int = 0, q1: int = 0, phase: int = 0) -> "Circuit":
        if code in (CZ, CX, SWAP):
            if q0 == q1:
                raise ValueError("two-qubit gate on a single wire")
            self.num_qubits = max(self.num_qubits, q0 + 1, q1 + 1)
        elif code != GPHASE:
            self.num_qubits = max(self.num_qubits, q0 + 1)
        if q0 < 0 or q1 < 0:
            raise ValueError("negative qubit index")
        self.ops.append((int(code), int(q0), int(q1), int(phase) & MASK32))
        return self

    def h(self, q): return self.push(H, q)
    def x(self, q): return self.push(X, q)
    def y(self, q): return self.push(Y, q)
    def z(self, q): return self.push(Z, q)
    def s(self, q): return self.push(S, q)
    def sdg(self, q): return self.push(SDG, q)
    def t(self, q): return self.push(T, q)
    def tdg(self, q): return self.push(TDG, q)
    def cz(self, a, b): return self.push(CZ, a, b)
    def cx(self, c, t): return self.push(CX, c, t)
    def swap(self, a, b): return self.push(SWAP, a, b)

    def p(self, q, phase):
        """diag(1, e^{i theta}).  An int is an exact ring phase (2 pi phase / 2^32, the Rust
        Circuit::p, src/circuit.rs:130-132); a float is an angle in radians, as the reference's
        Python binding takes it (src/pybind.rs:80-82)."""
        if isinstance(phase, float):
            return self.push(P, q, 0, phase_from_radians(phase))
        return self.push(P, q, 0, int(phase) & MASK32)

    def p_radians(self, q, radians: float):
        return self.push(P, q, 0, phase_from_radians(radians))

    def rz(self, q, radians: float):
        """RZ = P(theta) + global phase e^{-i theta/2} (src/circuit.rs:136-139)."""
        self.push(P, q, 0, phase_from_radians(radians))
        return self.push(GPHASE, 0, 0, phase_from_radians(-radians / 2.0))

    def gphase(self, phase: int):
        return self.push(GPHASE, 0, 0, phase)

    def ccx(self, a, b, c):
        """Toffoli as Clifford + 7 T/T-dagger (src/circuit.rs:163-179)."""
        self.h(c); self.cx(b, c); self.tdg(c); self.cx(a, c); self.t(c); self.cx(b, c); self.tdg(c)
        self.cx(a, c); self.t(b); self.t(c); self.h(c); self.cx(a, b); self.t(a); self.tdg(b)
        return self.cx(a, b)

    def ccz(self, a, b, c):
        """H(c) . CCX . H(c) (src/circuit.rs:182-186)."""
        self.h(c)
        self.ccx(a, b, c)
        return self.h(c)

    def inverse(self) -> "Circuit":
        """Reverse order, each gate inverted (src/circuit.rs:46-56, :189-191)."""
        inv = {S: SDG, SDG: S, T: TDG, TDG: T}
        out = Circuit(self.num_qubits)
        for code, a, b, ph in reversed(self.ops):
            if code in inv:
                out.ops.append((inv[code], a, b, ph))
            elif code in (P, GPHASE):
                out.ops.append((code, a, b, (-ph) & MASK32))
            else:
                out.ops.append((code, a, b, ph))
        return out

    _NAMED = {"H": (H, 1), "X": (X, 1), "Y": (Y, 1), "Z": (Z, 1), "S": (S, 1), "SDG": (SDG, 1), "T": (T, 1),
              "TDG": (TDG, 1), "CX": (CX, 2), "CZ": (CZ, 2), "SWAP": (SWAP, 2)}

    def extend(self, other) -> "Circuit":
        """Append another Circuit's gates, or a flat list of (name, qubits) ops as the reference's
        Python binding takes them (src/pybind.rs:101-121; a bad op raises ValueError)."""
        if isinstance(other, Circuit):
            self.num_qubits = max(self.num_qubits, other.num_qubits)
            self.ops.extend(other.ops)
            return self
        for name, qs in other:
            qs = list(qs)
            code = self._NAMED.get(name)
            if code is None or len(qs) != code[1]:
                raise ValueError("bad op %s %s" % (name, qs))
            self.push(code[0], *qs)
        return self

    def copy(self) -> "Circuit":
        c = Circuit(self.num_qubits)
        c.ops = list(self.ops)
        return c

    def t_count(self) -> int:
        """Non-Clifford rotations (src/circuit.rs:201-203)."""
        n = 0
        for code, _, _, ph in self.ops:
            if code in (T, TDG) or (code == P and (ph & ((1 << 30) - 1)) != 0):
                n += 1
        return n

    def h_count(self) -> int:
        return sum(1 if c == H else (2 if c == CX else 0) for c, _, _, _ in self.ops)

    def arrays(self):
        """(op u8, q0 i32, q1 i32, phase u32) numpy arrays for the C-ABI."""
        import numpy as np
        n = len(self.ops)
        op = np.zeros(max(n, 1), dtype=np.uint8)
        q0 = np.zeros(max(n, 1), dtype=np.int32)
        q1 = np.zeros(max(n, 1), dtype=np.int32)
        ph = np.zeros(max(n, 1), dtype=np.uint32)
        for i, (c, a, b, p) in enumerate(self.ops):
            op[i], q0[i], q1[i], ph[i] = c, a, b, p
        return n, op, q0, q1, ph
