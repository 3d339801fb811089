"""Dense unitaries: transform_u / c_transform_u (gates.rs:1427-1487) and
unitaries.rs.  The oracle's restatement is pinned against independent numpy
Kronecker products; the GPU path must match the oracle bit for bit."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import rng
from spinoza_gb300.gates import Gate
from spinoza_gb300.unitaries import Unitary


def random_unitary(m, seed):
    r = np.random.default_rng(seed)
    a = r.normal(size=(1 << m, 1 << m)) + 1j * r.normal(size=(1 << m, 1 << m))
    q, rr = np.linalg.qr(a)
    return q * (np.diag(rr) / np.abs(np.diag(rr)))


def dense_block(n, U, t, control=-1):
    """Full 2^n matrix: U on qubits t..t+m-1 (bit t+j = bit j), optionally controlled."""
    m = int(U.shape[0]).bit_length() - 1
    full = np.kron(np.kron(np.eye(1 << (n - t - m)), U), np.eye(1 << t))
    if control < 0:
        return full
    P1 = np.diag([(x >> control) & 1 for x in range(1 << n)]).astype(complex)
    return P1 @ full + (np.eye(1 << n) - P1)


@pytest.mark.parametrize("n,m,t,c", [(3, 1, 0, -1), (4, 2, 1, -1), (5, 3, 2, -1), (5, 2, 0, 4), (6, 3, 3, 1),
                                     (4, 4, 0, -1)])
def test_oracle_unitary_matches_dense(n, m, t, c):
    U = random_unitary(m, 10 * n + m)
    re, im = oracle.uniform_state(n, 3)
    psi = re + 1j * im
    oracle.apply_unitary(re, im, U, t, c)
    np.testing.assert_allclose(re + 1j * im, dense_block(n, U, t, c) @ psi, atol=1e-13)


def test_oracle_rejects_control_inside_block():
    re, im = oracle.uniform_state(4, 1)
    with pytest.raises(Exception):
        oracle.apply_unitary(re, im, random_unitary(2, 1), 1, 2)


def test_unitary_host_methods():
    """unitaries.rs:165-339: conj_t, multiply, from_single_qubit_gate."""
    U = Unitary.from_matrix(random_unitary(2, 5))
    V = Unitary(U.reals.copy(), U.imags.copy(), 4, 4)
    V.conj_t()
    np.testing.assert_allclose(U.multiply(V).matrix(), np.eye(4), atol=1e-14)
    G = Unitary.from_single_qubit_gate(3, Gate.H, 1)
    np.testing.assert_allclose(G.matrix(), np.kron(np.kron(np.eye(2), Gate.H.to_matrix()), np.eye(2)), atol=0)
    inv = Gate.Unitary(U).inverse()
    np.testing.assert_allclose(inv.matrix.matrix(), U.matrix().conj().T, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("n,m,t,c", [(1, 1, 0, -1), (5, 2, 1, -1), (9, 3, 4, -1), (9, 2, 0, 7), (12, 4, 6, 2),
                                     (14, 1, 13, 0), (6, 6, 0, -1)])
def test_gpu_unitary_bit_exact(gpu, n, m, t, c):
    from spinoza_gb300.core import State
    from spinoza_gb300.unitaries import c_transform_u, transform_u

    U = random_unitary(m, 7 * n + m)
    re, im = rng.uniform_state(n, 4)
    s = State.from_arrays(re, im)
    u = Unitary.from_matrix(U)
    if c < 0:
        transform_u(s, u, t)
    else:
        c_transform_u(s, u, c, t)
    oracle.apply_unitary(re, im, U, t, c)
    gre, gim = s.to_numpy()
    assert np.array_equal(gre, re) and np.array_equal(gim, im)


@pytest.mark.gpu
@pytest.mark.parametrize("g", [Gate.H, Gate.X, Gate.Y, Gate.Z, Gate.P(0.3), Gate.RX(1.0), Gate.RY(2.0),
                               Gate.RZ(-0.7), Gate.U(1.0, 2.0, 3.0)], ids=repr)
def test_gpu_gate_equals_its_unitary(gpu, g):
    """unitaries.rs tests: a gate and its full-state Unitary give the same state."""
    from spinoza_gb300 import gates as G
    from spinoza_gb300.core import State
    from spinoza_gb300.unitaries import apply_unitary

    n = 4
    for t in range(n):
        s = State.from_arrays(*rng.normal_state(n, t))
        out = apply_unitary(s, Unitary.from_single_qubit_gate(s, g, t))
        G.apply(g, s, t)
        a, b = s.to_numpy(), out.to_numpy()
        np.testing.assert_allclose(a[0], b[0], atol=1e-14)
        np.testing.assert_allclose(a[1], b[1], atol=1e-14)


@pytest.mark.gpu
def test_gpu_circuit_with_unitaries(gpu):
    """circuit.rs:514-558: unitary / c_unitary / append_u between gate runs."""
    from spinoza_gb300.circuit import QuantumCircuit, QuantumRegister

    U2, U1 = random_unitary(2, 1), random_unitary(1, 2)
    a, b = QuantumRegister(2), QuantumRegister(3)
    qc = QuantumCircuit(a, b)
    qc.h(0)
    qc.append_u(Unitary.from_matrix(U2), a)
    qc.cx(1, 2)
    qc.c_unitary(Unitary.from_matrix(U1), 0, 4)
    qc.ry(0.3, 3)
    qc.execute()
    re, im = oracle.zero_state(5)
    oracle.apply(oracle.gate(oracle.H), re, im, 0)
    oracle.apply_unitary(re, im, U2, 0)
    oracle.c_apply(oracle.gate(oracle.X), re, im, 1, 2)
    oracle.apply_unitary(re, im, U1, 4, 0)
    oracle.apply(oracle.gate(oracle.RY, (0.3,)), re, im, 3)
    gre, gim = qc.state.to_numpy()
    assert np.array_equal(gre, re) and np.array_equal(gim, im)
    _ = math
