"""Parity at the benchmark configurations' full sizes, against the oracle.

* Brickwork at 30 qubits (16 GiB state): the first two of the 20 layers
  (118 gates), run on the GPU in the exact mode (bit-identical to the oracle)
  and in the fast mode (within 1e-12), and on the oracle.
* Measurement at 28 qubits: a seeded N(0,1) normalised state, 1e6 shots from
  seeded uniforms (outcomes bit-identical to the oracle's), and the Ising
  <H> = sum a_i Z_i Z_{i+1} + b_i X_i (within 1e-12 of the oracle).
* Adjoint at 24 qubits, 8 layers, 384 parameters: the gradient against the
  parameter-shift rule (exact for RY and RZ) at 1e-9, for all 384 parameters
  with GPU forward circuits (fast mode, within rounding of the exact one) and
  for 16 sampled ones with oracle forward circuits; and against central differences (h = 1e-6) for all 384, at 1e-7.
  Central differences cannot reach 1e-9 in FP64 at this size: the energy
  (|E| ~ 10, a sum over 2^24 amplitudes) carries a rounding error of about
  1e-14, which divided by 2h = 2e-6 leaves about 5e-9 in each difference.

The host of the GPU machine holds the oracle's state (up to 16 GiB) and one
downloaded copy of the GPU's."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import adjoint, core, rng
from spinoza_gb300.circuit import QuantumCircuit
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


def _brickwork_oracle_ops(n: int, layers: int, seed: int = 2) -> np.ndarray:
    """The 30-qubit brickwork's first `layers` layers, built from the oracle's
    own record layout and stream (U on every qubit, then CX even, CX odd)."""
    ang = oracle.uniforms(seed, 3 * n * 20)[: 3 * n * layers] * (2.0 * math.pi)
    rows, k = [], 0
    for _ in range(layers):
        for q in range(n):
            rows.append(((oracle.U, 0, 0, 0, (ang[k], ang[k + 1], ang[k + 2])), q, oracle.CONTROLS_NONE, 0, 0))
            k += 3
        for q in list(range(0, n - 1, 2)) + list(range(1, n - 1, 2)):
            rows.append(((oracle.X, 0, 0, 0, (0.0, 0.0, 0.0)), q + 1, oracle.CONTROLS_SINGLE, 1 << q, 0))
    ops = np.zeros(len(rows), dtype=oracle.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    return ops


def test_brickwork_30_qubits_two_layers_match_oracle(gpu):
    n, layers = 30, 2
    ops = _brickwork_oracle_ops(n, layers)
    assert len(ops) == layers * (2 * n - 1)
    re, im = oracle.zero_state(n)
    oracle.execute(ops, re, im)
    s = State(n)
    for fast in (False, True):
        s.reset_zero()
        QuantumCircuit.from_state(s, fast=fast).execute_ops(ops.view(nat.OP_DTYPE))
        gre, gim = s.to_numpy()
        if not fast:
            assert np.array_equal(gre, re) and np.array_equal(gim, im), "exact mode differs from the oracle"
        else:
            d = max(float(np.max(np.abs(gre - re))), float(np.max(np.abs(gim - im))))
            assert d <= 1e-12, d
        del gre, gim


def test_measurement_28_qubits_shots_and_hamiltonian_match_oracle(gpu):
    n = 28
    s = State(n)
    s.fill_random(3, "normal", normalise=True)
    re, im = s.to_numpy()  # the oracle reads exactly the GPU's input state
    u = rng.uniforms(4, 1_000_000)
    got = core.sample(s, u)
    want = oracle.sample(re, im, u)
    assert np.array_equal(got, want)
    ab = rng.uniforms(5, 4 * n)
    a = np.sqrt(-2 * np.log1p(-ab[:n - 1])) * np.cos(2 * math.pi * ab[n:2 * n - 1])
    b = np.sqrt(-2 * np.log1p(-ab[2 * n:3 * n])) * np.cos(2 * math.pi * ab[3 * n:4 * n])
    H = core.ising_hamiltonian(a, b)
    e_gpu = core.pauli_expectation(s, H)
    e_orc = oracle.pauli_expectation(re, im, H)
    assert abs(e_gpu - e_orc) <= 1e-12, (e_gpu, e_orc)


def _adjoint24():
    n, layers = 24, 8
    ops, pidx = adjoint.hardware_efficient_ansatz(n, layers)
    theta = (rng.uniforms(6, len(pidx)) * 2 - 1) * math.pi
    u = rng.uniforms(7, 4 * n)
    a = np.sqrt(-2 * np.log1p(-u[:n - 1])) * np.cos(2 * math.pi * u[n:2 * n - 1])
    b = np.sqrt(-2 * np.log1p(-u[2 * n:3 * n])) * np.cos(2 * math.pi * u[3 * n:4 * n])
    return n, ops, pidx, theta, core.ising_hamiltonian(a, b)


def test_adjoint_24_qubits_384_parameters(gpu):
    n, ops, pidx, theta, H = _adjoint24()
    assert len(pidx) == 384
    s = State(n)
    e, g = adjoint.adjoint_gradient(s, adjoint.set_params(ops, pidx, theta), pidx, H)
    s.reset_zero()  # the handle now holds psi(theta); the circuit starts from |0...0>
    e_fast, g_fast = adjoint.adjoint_gradient(s, adjoint.set_params(ops, pidx, theta), pidx, H, fast=True)
    f = State(n)

    runner = QuantumCircuit.from_state(f, fast=True)

    def energy_gpu(th):  # fast-mode forward: within rounding of the exact one, half the FP64 work
        f.reset_zero()
        runner.execute_ops(adjoint.set_params(ops, pidx, th))
        return core.pauli_expectation(f, H)

    def energy_oracle(th):
        re, im = oracle.zero_state(n)
        oracle.execute(adjoint.set_params(ops, pidx, th).view(oracle.OP_DTYPE), re, im)
        return oracle.pauli_expectation(re, im, H)

    assert abs(e - energy_oracle(theta)) <= 1e-12
    assert abs(e_fast - e) <= 1e-12
    shift = np.empty(len(pidx))
    cdiff = np.empty(len(pidx))
    h = 1e-6
    for j in range(len(pidx)):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += math.pi / 2
        tm[j] -= math.pi / 2
        shift[j] = 0.5 * (energy_gpu(tp) - energy_gpu(tm))
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        cdiff[j] = (energy_gpu(tp) - energy_gpu(tm)) / (2 * h)
    assert np.max(np.abs(g - shift)) <= 1e-9, np.max(np.abs(g - shift))
    assert np.max(np.abs(g_fast - shift)) <= 1e-9, np.max(np.abs(g_fast - shift))
    assert np.max(np.abs(g - cdiff)) <= 1e-7, np.max(np.abs(g - cdiff))
    sample = np.sort(np.floor(rng.uniforms(61, 16) * len(pidx)).astype(int))
    for j in sample:
        tp, tm = theta.copy(), theta.copy()
        tp[j] += math.pi / 2
        tm[j] -= math.pi / 2
        ps = 0.5 * (energy_oracle(tp) - energy_oracle(tm))
        assert abs(g[j] - ps) <= 1e-9, (j, g[j], ps)
        assert abs(g_fast[j] - ps) <= 1e-9, (j, g_fast[j], ps)
