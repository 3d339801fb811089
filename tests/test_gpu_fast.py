"""Fast mode (SPZ_EXEC_FAST) vs the oracle: the same circuits, rewritten to
need fewer FP64 instructions (lazy scaling, U = P RY P, phases pushed through
permutations).  Not bit-identical by design; the bound is the parity bound of
1e-12 on every amplitude (states here have |amplitude| <= 1)."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import circuit, rng
from spinoza_gb300.circuit import QuantumCircuit
from spinoza_gb300.core import State
from test_gpu_circuits import brickwork, qft_with_swaps, random_circuit

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _fast(ops, init):
    s = State.from_arrays(*init)
    qc = QuantumCircuit.from_state(s, fast=True)
    qc.execute_ops(ops)
    return s.to_numpy(), qc


def _oracle(ops, init):
    re, im = init[0].copy(), init[1].copy()
    oracle.execute(ops, re, im)
    return re, im


def _maxdiff(a, b):
    return max(float(np.max(np.abs(a[0] - b[0]))), float(np.max(np.abs(a[1] - b[1]))))


@pytest.mark.parametrize("n,seed", [(3, 1), (6, 2), (13, 3), (15, 4), (16, 5)])
def test_fast_random_circuits(gpu, n, seed):
    init = rng.uniform_state(n, seed)
    ops = random_circuit(n, 400, seed)
    g, _ = _fast(ops, init)
    assert _maxdiff(g, _oracle(ops, init)) <= TOL


@pytest.mark.parametrize("kind", [nat.H, nat.X, nat.Y, nat.Z, nat.P, nat.RX, nat.RY, nat.RZ, nat.U, nat.SWAP])
def test_fast_single_kind_chains(gpu, kind):
    """Long chains of one gate kind (plus CX ladders) on every qubit."""
    n = 14
    r = np.random.default_rng(kind)
    rows = []
    for layer in range(6):
        for q in range(n):
            rows.append(((kind, q, (q + 3) % n, 0, r.uniform(-4, 4, 3)), q, 0, 0, 0))
        for q in range(layer % 2, n - 1, 2):
            rows.append(((nat.X, 0, 0, 0, (0, 0, 0)), q + 1, nat.CONTROLS_SINGLE, 1 << q, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, row in enumerate(rows):
        ops[i] = row
    init = rng.uniform_state(n, 9)
    g, _ = _fast(ops, init)
    assert _maxdiff(g, _oracle(ops, init)) <= TOL


def test_fast_u_edge_angles(gpu):
    """U with sin(theta/2) = 0, cos(theta/2) < 0, and theta near pi."""
    n = 5
    rows = []
    for q, (t, p, l) in enumerate([(0.0, 0.7, 0.4), (2 * math.pi, 1.1, -0.3), (math.pi, 0.2, 2.0),
                                   (-3.0, -2.5, 1.0), (4.0, 0.0, 0.0)]):
        rows.append(((nat.U, 0, 0, 0, (t, p, l)), q, 0, 0, 0))
        rows.append(((nat.RY, 0, 0, 0, (t, 0, 0)), (q + 1) % n, 0, 0, 0))
        rows.append(((nat.RX, 0, 0, 0, (-t, 0, 0)), (q + 2) % n, 0, 0, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, row in enumerate(rows):
        ops[i] = row
    init = rng.uniform_state(n, 4)
    g, _ = _fast(ops, init)
    assert _maxdiff(g, _oracle(ops, init)) <= TOL


def test_fast_brickwork_and_qft(gpu):
    for n, ops, init in [(17, brickwork(17, 4), rng.uniform_state(17, 2)),
                         (20, qft_with_swaps(20), rng.normal_state(20, 1))]:
        g, qc = _fast(ops, init)
        assert _maxdiff(g, _oracle(ops, init)) <= TOL
        exact = circuit.plan_stats(n, ops)
        assert qc.last_stats.fp64_ops < exact["fp64_ops"]


def test_fast_long_circuit_renormalises(gpu):
    """Thousands of lazy rotations: the carried scale factor is folded back
    before it leaves the exponent range."""
    n = 4
    r = np.random.default_rng(3)
    rows = [((nat.H if i % 3 == 0 else nat.RY, 0, 0, 0, (r.uniform(1.2, 1.9), 0, 0)), i % n, 0, 0, 0)
            for i in range(3000)]
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, row in enumerate(rows):
        ops[i] = row
    init = rng.normal_state(n, 8)
    g, _ = _fast(ops, init)
    assert np.all(np.isfinite(g[0])) and _maxdiff(g, _oracle(ops, init)) <= 1e-11


def test_fast_mid_circuit_measurement(gpu):
    n = 8
    init = rng.normal_state(n, 3)
    qc = QuantumCircuit.__new__(QuantumCircuit)
    qc.transformations = []
    qc._seed, qc._draw_index = 0, 0
    for q in range(n):
        qc.u(0.3 * q, 0.2, -0.4, q)
    qc.measure(2)
    qc.cx(2, 5)
    qc.ry(0.4, 2)
    qc.rz(1.3, 6)
    qc.measure(6)
    ops = qc.ops()
    ops["gate"]["p"][[n, n + 4], 0] = 0.37
    s = State.from_arrays(*init)
    run = QuantumCircuit.from_state(s, fast=True)
    run.execute_ops(ops)
    re, im = init[0].copy(), init[1].copy()
    tr = oracle.execute(ops, re, im)
    assert (run.qubit_tracker.c.measured, run.qubit_tracker.c.values) == tr
    assert _maxdiff(s.to_numpy(), (re, im)) <= TOL
