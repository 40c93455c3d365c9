"""Write known_answers.json: the reference's analytic known-answer tests as fixtures.

Every value below is the closed-form answer asserted by a test of the reference crate
(cited per case); nothing here is computed by the oracle or the product.
Run: python tests/golden/make_known_answers.py
"""
import cmath
import json
import math
import os

H, X, Y, Z, S, SDG, T, TDG, P, CZ, CX, SWAP, GPHASE = range(13)
r2 = 1 / math.sqrt(2)
w = cmath.exp(1j * math.pi / 4)


def ccx_ops(a, b, c):
    # Nielsen & Chuang Fig. 4.9 expansion used by src/circuit.rs:163-179
    return [(H, c), (CX, b, c), (TDG, c), (CX, a, c), (T, c), (CX, b, c), (TDG, c), (CX, a, c), (T, b), (T, c),
            (H, c), (CX, a, b), (T, a), (TDG, b), (CX, a, b)]


cases = []
# src/engine.rs:777-787 -- GHZ: <y|H0 CX01 CX12|000> = 1/sqrt2 for y in {000, 111}
cases.append({"source": "src/engine.rs:777-787", "num_qubits": 3, "tol": 1e-12,
              "ops": [[H, 0], [CX, 0, 1], [CX, 1, 2]],
              "values": [[0, y, (r2 if y in (0, 7) else 0.0), 0.0] for y in range(8)]})
# src/engine.rs:790-802 -- H T Z H |0> = ((1-w)|0> + (1+w)|1>)/2
a0, a1 = (1 - w) / 2, (1 + w) / 2
cases.append({"source": "src/engine.rs:790-802", "num_qubits": 1, "tol": 1e-12,
              "ops": [[H, 0], [T, 0], [Z, 0], [H, 0]],
              "values": [[0, 0, a0.real, a0.imag], [0, 1, a1.real, a1.imag]]})
# src/circuit.rs:234-244 -- Toffoli truth table: <expect|CCX|inp> = 1 (global phase 1 here:
# the expansion is exactly CCX)
vals = []
for inp in range(8):
    exp = inp ^ 4 if (inp & 3) == 3 else inp
    for y in range(8):
        vals.append([inp, y, 1.0 if y == exp else 0.0, 0.0])
cases.append({"source": "src/circuit.rs:234-244", "num_qubits": 3, "tol": 1e-9,
              "ops": [list(o) for o in ccx_ops(0, 1, 2)], "values": vals})
# src/sim.rs:402-410 -- H Z H = X: <1|HZH|0> = 1
cases.append({"source": "src/sim.rs:402-410", "num_qubits": 1, "tol": 1e-12,
              "ops": [[H, 0], [Z, 0], [H, 0]], "values": [[0, 1, 1.0, 0.0], [0, 0, 0.0, 0.0], [1, 0, 1.0, 0.0]]})
# src/sim.rs:421-428 -- Y = i X Z: <1|Y|0> = i, <0|Y|1> = -i
cases.append({"source": "src/sim.rs:421-428", "num_qubits": 1, "tol": 1e-12,
              "ops": [[Y, 0]], "values": [[0, 1, 0.0, 1.0], [1, 0, 0.0, -1.0]]})

with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json"), "w") as f:
    json.dump({"amplitudes": cases}, f, indent=1)
