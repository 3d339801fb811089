"""Pin the oracle: the reference's own known-answer tests (golden values copied
from its Rust test modules by tests/golden/extract_reference_goldens.py), plus
independent checks of the restated pair enumeration against dense matrices."""
import itertools
import math

import numpy as np
import pytest

import oracle
import refcases as rc
from spinoza_gb300.gates import Gate

B = rc.OracleBackend()


@pytest.mark.parametrize("case", rc.ALL_CASES, ids=lambda c: c.__name__[5:])
def test_reference_known_answers(case):
    assert case(B) > 0


@pytest.mark.parametrize("via", ["append", "c_append", "mc_append"])
def test_reference_value_encoding(via):
    assert rc.case_value_encoding(B, via) > 0


def test_goldens_cover_every_reference_gate_test():
    keys = set(rc.GOLDENS)
    for k in ["gates.rs::qcbm_20_qubits", "gates.rs::u_gate_1_qubit", "gates.rs::ch", "gates.rs::crz",
              "gates.rs::controlled_u", "core.rs::xyz_exp_val", "measurement.rs::test_measure_qubit_known_state"]:
        assert k in keys


@pytest.mark.parametrize("g", [Gate.H, Gate.X, Gate.Y, Gate.Z, Gate.P(2.03), Gate.RX(2.03), Gate.RZ(3.03),
                               Gate.RY(3.03), Gate.U(1.0, 2.0, 3.0)], ids=repr)
def test_inverse_identities(g):
    """gates.rs:1903-2045: G * G.inverse() == I (reference tolerance 1e-3; we use 1e-14)."""
    ident = g.to_matrix() @ g.inverse().to_matrix()
    np.testing.assert_allclose(ident, np.eye(2), atol=1e-14)


def test_m_and_swap_have_no_inverse_matrix():
    """gates.rs:2050-2062 (#[should_panic])."""
    with pytest.raises(NotImplementedError):
        Gate.M.inverse()
    with pytest.raises(NotImplementedError):
        Gate.SWAP(0, 1).inverse().to_matrix()


# ---------------------------------------------------------------- dense check
def _dense(n, g: Gate, target, ones=(), zeros=()):
    """Full 2^n x 2^n matrix of a (multi-)controlled 1-qubit gate, built independently."""
    m = g.to_matrix()
    N = 1 << n
    D = np.zeros((N, N), dtype=complex)
    for col in range(N):
        ok = all((col >> c) & 1 for c in ones) and not any((col >> z) & 1 for z in zeros)
        if not ok:
            D[col, col] = 1
            continue
        b = (col >> target) & 1
        for out_b in (0, 1):
            row = (col & ~(1 << target)) | (out_b << target)
            D[row, col] += m[out_b, b]
    return D


GATES = [Gate.H, Gate.X, Gate.Y, Gate.Z, Gate.P(0.7), Gate.RX(1.1), Gate.RY(-0.4), Gate.RZ(2.2),
         Gate.U(0.3, 1.4, -2.5)]


@pytest.mark.parametrize("g", GATES, ids=repr)
def test_oracle_mc_apply_matches_dense_matrices(g):
    """Every (target, control set, zeros) on 4 qubits: the restated enumeration
    equals the dense matrix — including the target >= 1 cases that the
    reference's mc loop mis-pairs (gates.rs:425-446)."""
    n = 4
    re0, im0 = oracle.uniform_state(n, 11)
    psi = re0 + 1j * im0
    for t in range(n):
        others = [q for q in range(n) if q != t]
        for r in range(0, 4):
            for ctrls in itertools.combinations(others, r):
                for nz in range(len(ctrls) + 1):
                    zeros = ctrls[:nz]
                    ones = ctrls[nz:]
                    re, im = re0.copy(), im0.copy()
                    oracle.mc_apply(oracle.gate(g.kind, g.params), re, im, ctrls, zeros, t)
                    want = _dense(n, g, t, ones, zeros) @ psi
                    np.testing.assert_allclose(re + 1j * im, want, atol=1e-14)


def test_oracle_swap_equals_three_cx():
    """gates.rs:1872-1901: swap_apply == CX(a,b) CX(b,a) CX(a,b), exactly."""
    n = 9
    for a, b in [(0, 1), (0, 8), (3, 5)]:
        r1, i1 = oracle.uniform_state(n, 5)
        r2, i2 = r1.copy(), i1.copy()
        oracle.apply(oracle.gate(oracle.SWAP, (), a, b), r1, i1, 0)
        x = oracle.gate(oracle.X)
        oracle.c_apply(x, r2, i2, a, b)
        oracle.c_apply(x, r2, i2, b, a)
        oracle.c_apply(x, r2, i2, a, b)
        assert np.array_equal(r1, r2) and np.array_equal(i1, i2)


def test_oracle_parallel_h_is_correct_at_16_qubits():
    """The reference's parallel H writes imag[s0] = b1 + c1 (gates.rs:593); the
    oracle follows the correct serial formula at every size: H H = I."""
    n = 16
    re, im = oracle.uniform_state(n, 3)
    r0, i0 = re.copy(), im.copy()
    h = oracle.gate(oracle.H)
    for t in (0, 7, 15):
        oracle.apply(h, re, im, t)
        oracle.apply(h, re, im, t)
    np.testing.assert_allclose(re, r0, atol=1e-15)
    np.testing.assert_allclose(im, i0, atol=1e-15)


def test_oracle_iqft_round_trip():
    """circuit.rs:962-989: iqft then its inverse restores the state."""
    n = 6
    re, im = oracle.uniform_state(n, 9)
    r0, i0 = re.copy(), im.copy()
    t = list(range(n - 1, -1, -1))
    oracle.iqft(re, im, t)
    # inverse: reverse order, negated angles
    for j in range(len(t)):
        for k in range(j):
            oracle.c_apply(oracle.gate(oracle.P, (math.pi / 2.0 ** (j - k),)), re, im, t[j], t[k])
        oracle.apply(oracle.gate(oracle.H), re, im, t[j])
    np.testing.assert_allclose(re, r0, atol=1e-13)
    np.testing.assert_allclose(im, i0, atol=1e-13)


def test_oracle_measurement_rule():
    """Outcome 1 iff u < 1 - prob0; collapse renormalises (measurement.rs:12-92)."""
    n = 5
    re, im = oracle.uniform_state(n, 2)
    s = 1 / math.sqrt(np.sum(re * re + im * im))
    re *= s
    im *= s
    p0 = oracle.prob0(re, im, 2)
    for u, want in [(0.0, 1 if p0 < 1 else 0), (0.999999, 0)]:
        r, i = re.copy(), im.copy()
        v, p = oracle.measure_qubit(r, i, 2, False, None, u)
        assert p == p0 and v == (1 if u < 1 - p0 else 0) and v == want
        assert abs(np.sum(r * r + i * i) - 1) < 1e-12


def test_oracle_sampling_rule_matches_a_direct_cdf():
    """The blocked-CDF sampler agrees with a plain inverse CDF away from ties."""
    n = 12
    re, im = oracle.uniform_state(n, 4)
    u = np.array([oracle.stream_uniform(8, i) for i in range(2000)])
    got = oracle.sample(re, im, u)
    p = re * re + im * im
    cdf = np.cumsum(p)
    want = np.searchsorted(cdf, u * cdf[-1], side="right")
    close = np.abs(cdf[np.minimum(want, len(cdf) - 1)] - u * cdf[-1]) < 1e-9
    assert np.array_equal(got[~close], want[~close])
