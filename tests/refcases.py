"""The reference's own known-answer tests, restated once and run against two
backends: the oracle (CPU restatement) and the GPU library.

Each `case_*` function repeats the setup of one #[test] of QuState/spinoza
(file:line in its docstring) and checks the expected values recorded in
tests/golden/reference_goldens.json, at the reference's tolerance.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300.gates import Gate

PI = math.pi
GOLDENS = json.loads((Path(__file__).parent / "golden" / "reference_goldens.json").read_text())["tests"]


# ----------------------------------------------------------------- backends
def _og(g: Gate) -> oracle.Gate:
    return oracle.gate(g.kind, g.params, *g.qubits)


class OracleBackend:
    name = "oracle"

    def new_state(self, n):
        return list(oracle.zero_state(n))

    def from_arrays(self, re, im):
        return [np.array(re, dtype=np.float64), np.array(im, dtype=np.float64)]

    def arrays(self, s):
        return s[0], s[1]

    def apply(self, g, s, t):
        oracle.apply(_og(g), s[0], s[1], t)

    def c_apply(self, g, s, c, t):
        oracle.c_apply(_og(g), s[0], s[1], c, t)

    def cc_apply(self, g, s, c0, c1, t):
        oracle.cc_apply(_og(g), s[0], s[1], c0, c1, t)

    def mc_apply(self, g, s, controls, zeros, t):
        oracle.mc_apply(_og(g), s[0], s[1], controls, zeros, t)

    def iqft(self, s, targets):
        oracle.iqft(s[0], s[1], targets)

    def measure_qubit(self, s, target, reset, v=None, u=0.0):
        return oracle.measure_qubit(s[0], s[1], target, reset, v, u)[0]

    def xyz_expectation_value(self, obs, s, targets):
        return oracle.xyz_expectation_value(obs, s[0], s[1], targets)

    def qubit_expectation_value(self, s, t):
        return oracle.qubit_expectation_value(s[0], s[1], t)

    def execute(self, s, ops, measured=0, values=0):
        return oracle.execute(ops, s[0], s[1], measured, values)


class GpuBackend:
    name = "gpu"

    def __init__(self, fused: bool = True):
        from spinoza_gb300 import core, gates, measurement

        self.core, self.gates, self.measurement = core, gates, measurement
        self.fused = fused

    def new_state(self, n):
        return self.core.State(n)

    def from_arrays(self, re, im):
        return self.core.State.from_arrays(re, im)

    def arrays(self, s):
        return s.to_numpy()

    def apply(self, g, s, t):
        self.gates.apply(g, s, t)

    def c_apply(self, g, s, c, t):
        self.gates.c_apply(g, s, c, t)

    def cc_apply(self, g, s, c0, c1, t):
        self.gates.cc_apply(g, s, c0, c1, t)

    def mc_apply(self, g, s, controls, zeros, t):
        self.gates.mc_apply(g, s, controls, zeros, t)

    def iqft(self, s, targets):
        self.core.iqft(s, targets)

    def measure_qubit(self, s, target, reset, v=None, u=0.0):
        return self.measurement.measure_qubit(s, target, reset, v, u)

    def xyz_expectation_value(self, obs, s, targets):
        return self.core.xyz_expectation_value(obs, s, targets)

    def qubit_expectation_value(self, s, t):
        return self.core.qubit_expectation_value(s, t)

    def execute(self, s, ops, measured=0, values=0):
        from ctypes import byref

        tr = nat.spz_tracker(measured, values)
        ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
        flags = nat.EXEC_DEFAULT if self.fused else nat.EXEC_UNFUSED
        nat.check(nat.lib().spz_circuit_execute(s.handle, nat.ptr(ops), len(ops), byref(tr), flags, None))
        return tr.measured, tr.values


# ------------------------------------------------------------------ helpers
def _eval_index(expr: str, env: dict) -> int:
    return int(eval(expr, {"__builtins__": {}}, dict(env)))


def check_literal_asserts(key: str, re: np.ndarray, im: np.ndarray, env: dict, select=None) -> int:
    """Check every recorded assert of test `key` (optionally a subset)."""
    arrays = {"reals": re, "imags": im}
    n_checked = 0
    asserts = GOLDENS[key]["asserts"]
    for a in (asserts if select is None else [asserts[i] for i in select]):
        if a["array"] is None:  # closure form `.for_each(|(z_re, z_im)| ...)`: element i
            arr = {"*z_re": "reals", "*z_im": "imags"}[a["target"]]
            idx = env["i"]
        else:
            arr = a["array"]
            idx = _eval_index(a["index"], env)
        got = float(arrays[arr][idx])
        assert abs(got - a["expected"]) < a["eps"], f"{key} line {a['line']}: {a['target']} = {got}, want {a['expected']}"
        n_checked += 1
    return n_checked


def qcbm_functional(B, n):
    """gates.rs:1499-1529."""
    s = B.new_state(n)
    pairs = [(i, (i + 1) % n) for i in range(n)]
    for i in range(n):
        B.apply(Gate.RX(1.0), s, i)
        B.apply(Gate.RZ(1.0), s, i)
    for p0, p1 in pairs[: n - 1]:
        B.c_apply(Gate.X, s, p0, p1)
    for _ in range(9):
        for i in range(n):
            B.apply(Gate.RZ(1.0), s, i)
            B.apply(Gate.RX(1.0), s, i)
            B.apply(Gate.RZ(1.0), s, i)
        for p0, p1 in pairs[: n - 1]:
            B.c_apply(Gate.X, s, p0, p1)
    for i in range(n):
        B.apply(Gate.RZ(1.0), s, i)
        B.apply(Gate.RX(1.0), s, i)
    return s


# -------------------------------------------------------------------- cases
def case_h_gate_3_qubits(B):
    """gates.rs:1531-1544."""
    n = 3
    s = B.new_state(n)
    for i in range(n):
        B.apply(Gate.H, s, i)
    re, im = B.arrays(s)
    return sum(check_literal_asserts("gates.rs::h_gate_3_qubits", re, im, {"i": i}) for i in range(1 << n))


def _all_targets_case(B, key, gate, n):
    s = B.new_state(n)
    for i in range(n):
        B.apply(gate, s, i)
    re, im = B.arrays(s)
    return check_literal_asserts(key, re, im, {"n": n})


def case_x_gate_3_qubits(B):
    """gates.rs:1546-1560."""
    return _all_targets_case(B, "gates.rs::x_gate_3_qubits", Gate.X, 3)


def case_x_gate_20_qubits(B):
    """gates.rs:1562-1576."""
    return _all_targets_case(B, "gates.rs::x_gate_20_qubits", Gate.X, 20)


def case_y_gate_3_qubits(B):
    """gates.rs:1578-1592."""
    return _all_targets_case(B, "gates.rs::y_gate_3_qubits", Gate.Y, 3)


def case_y_gate_20_qubits(B):
    """gates.rs:1594-1608."""
    return _all_targets_case(B, "gates.rs::y_gate_20_qubits", Gate.Y, 20)


def _basis0_case(B, key, gate):
    n = 3
    s = B.new_state(n)
    for i in range(n):
        B.apply(gate, s, i)
    re, im = B.arrays(s)
    k = 0
    for i in range(1 << n):  # asserts 0,1 for i == 0; 2,3 otherwise
        k += check_literal_asserts(key, re, im, {"i": i}, select=[0, 1] if i == 0 else [2, 3])
    return k


def case_z_gate_3_qubits(B):
    """gates.rs:1610-1628."""
    return _basis0_case(B, "gates.rs::z_gate_3_qubits", Gate.Z)


def case_p_gate_3_qubits(B):
    """gates.rs:1630-1648."""
    return _basis0_case(B, "gates.rs::p_gate_3_qubits", Gate.P(PI))


def case_rx_gate_3_qubits(B):
    """gates.rs:1650-1682."""
    return _all_targets_case(B, "gates.rs::rx_gate_3_qubits", Gate.RX(1.0), 3)


def case_ry_gate_3_qubits(B):
    """gates.rs:1684-1716."""
    return _all_targets_case(B, "gates.rs::ry_gate_3_qubits", Gate.RY(1.0), 3)


def case_rz_gate_3_qubits(B):
    """gates.rs:1718-1750."""
    return _all_targets_case(B, "gates.rs::rz_gate_3_qubits", Gate.RZ(1.0), 3)


def case_qcbm_3_qubits(B):
    """gates.rs:1786-1795."""
    re, im = B.arrays(qcbm_functional(B, 3))
    return check_literal_asserts("gates.rs::qcbm_3_qubits", re, im, {})


def case_qcbm_20_qubits(B):
    """gates.rs:1797-1809 (runs the reference's parallel RX/RZ/CX paths)."""
    re, im = B.arrays(qcbm_functional(B, 20))
    return check_literal_asserts("gates.rs::qcbm_20_qubits", re, im, {})


def case_u_gate_3_qubits(B):
    """gates.rs:1811-1843."""
    return _all_targets_case(B, "gates.rs::u_gate_3_qubits", Gate.U(1.0, 1.0, 1.0), 3)


def case_u_gate_1_qubit(B):
    """gates.rs:1845-1870: U(theta=2, phi=3, lambda=1) on |0> (asserts 0-3) and on X|0> (4-7)."""
    g = Gate.U(2.0, 3.0, 1.0)
    s = B.new_state(1)
    B.apply(g, s, 0)
    k = check_literal_asserts("gates.rs::u_gate_1_qubit", *B.arrays(s), {}, select=[0, 1, 2, 3])
    s = B.new_state(1)
    B.apply(Gate.X, s, 0)
    B.apply(g, s, 0)
    return k + check_literal_asserts("gates.rs::u_gate_1_qubit", *B.arrays(s), {}, select=[4, 5, 6, 7])


def _controlled_pattern_case(B, key, gate):
    n = 3
    s = B.new_state(n)
    for t in range(n):
        B.apply(Gate.H, s, t)
    re, im = B.arrays(s)
    k = 0
    for i in range(1 << n):  # first two asserts: the H-layer check over every amplitude
        k += check_literal_asserts(key, re, im, {"i": i}, select=[0, 1])
    B.c_apply(gate, s, 0, 1)
    re, im = B.arrays(s)
    i = 0
    while i < (1 << n) - 3:
        k += check_literal_asserts(key, re, im, {"i": i}, select=list(range(2, 10)))
        i += 4
    return k


def case_ch(B):
    """gates.rs:2099-2133."""
    return _controlled_pattern_case(B, "gates.rs::ch", Gate.H)


def case_crz(B):
    """gates.rs:2135-2171."""
    return _controlled_pattern_case(B, "gates.rs::crz", Gate.RZ(PI / 2.0))


def case_controlled_u(B):
    """gates.rs:2197-2236: H on all 3 qubits, then c_apply(U(1,2,3), 0, 1)."""
    g = GOLDENS["gates.rs::controlled_u"]["arrays"]
    s = B.new_state(3)
    for t in range(3):
        B.apply(Gate.H, s, t)
    B.c_apply(Gate.U(1.0, 2.0, 3.0), s, 0, 1)
    re, im = B.arrays(s)
    np.testing.assert_allclose(re, g["expected_reals"]["values"], atol=1e-5, rtol=0)
    np.testing.assert_allclose(im, g["expected_imags"]["values"], atol=1e-5, rtol=0)
    return 16


def case_xyz_exp_val(B):
    """core.rs:293-301: RX(0.54), RY(0.12) on one qubit; <Z> = 0.8515405859048367."""
    s = B.new_state(1)
    B.apply(Gate.RX(0.54), s, 0)
    B.apply(Gate.RY(0.12), s, 0)
    got = B.xyz_expectation_value("z", s, [0])[0]
    a = GOLDENS["core.rs::xyz_exp_val"]["asserts"][0]
    assert abs(got - a["expected"]) < a["eps"]
    q = B.qubit_expectation_value(s, 0)  # core.rs:328-339
    assert abs(q - got) < 1e-4
    return 2


def case_measure_qubit_known_state(B):
    """measurement.rs:143-246: fixed 8-amplitude state, forced outcomes 0, 0, 1."""
    key = "measurement.rs::test_measure_qubit_known_state"
    vals = GOLDENS[key]["arrays"]["vals"]["values"]
    s = B.from_arrays(vals[0::2], vals[1::2])
    k = 0
    B.measure_qubit(s, 0, True, 0)
    k += check_literal_asserts(key, *B.arrays(s), {}, select=list(range(0, 16)))
    B.measure_qubit(s, 1, True, 0)
    k += check_literal_asserts(key, *B.arrays(s), {}, select=list(range(16, 32)))
    B.measure_qubit(s, 2, True, 1)
    k += check_literal_asserts(key, *B.arrays(s), {}, select=list(range(32, 48)))
    return k


def case_value_encoding(B, via: str):
    """circuit.rs:1075-1192 (append / c_append / mc_append value encoding, v = 4):
    H on all 3 qubits, P(2 pi v / 2^(t+1)) on each, then the inverse QFT built
    with single controls -> |4>."""
    key = {"append": "circuit.rs::append_value_encoding", "c_append": "circuit.rs::c_append_value_encoding",
           "mc_append": "circuit.rs::mc_append_value_encoding"}[via]
    n, v = 3, 4.0
    s = B.new_state(n)
    for t in range(n):
        B.apply(Gate.H, s, t)
    for t in range(n):
        B.apply(Gate.P(2.0 * PI / (2.0 ** (t + 1)) * v), s, t)
    targets = list(range(n - 1, -1, -1))
    for j in range(len(targets) - 1, -1, -1):
        B.apply(Gate.H, s, targets[j])
        for k in range(j - 1, -1, -1):
            B.c_apply(Gate.P(-PI / 2.0 ** (j - k)), s, targets[j], targets[k])
    re, im = B.arrays(s)
    k = 0
    for i in range(1 << n):
        k += check_literal_asserts(key, re, im, {"i": i}, select=[0, 1] if i == int(v) else [2, 3])
    return k


ALL_CASES = [
    case_h_gate_3_qubits, case_x_gate_3_qubits, case_x_gate_20_qubits, case_y_gate_3_qubits,
    case_y_gate_20_qubits, case_z_gate_3_qubits, case_p_gate_3_qubits, case_rx_gate_3_qubits,
    case_ry_gate_3_qubits, case_rz_gate_3_qubits, case_qcbm_3_qubits, case_qcbm_20_qubits,
    case_u_gate_3_qubits, case_u_gate_1_qubit, case_ch, case_crz, case_controlled_u, case_xyz_exp_val,
    case_measure_qubit_known_state,
]
