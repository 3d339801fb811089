"""Randomised differential tests of the circuit executor against the oracle.

The circuits mix the structures that the planner and the fast lowering treat
specially: rotation layers, CX ladders, singly controlled diagonals (CZ, CP,
CRZ; parity phase terms in fast mode), SWAPs that carry pending phases,
multi-controlled gates with zero-controls, gates on the qubits above a tile,
bit-flip noise with fixed draws, and mid-circuit measurements followed by
classically conditioned gates (circuit.rs:559-578).

Without measurements the fused mode, a replayed program and the host-array
execute must equal the oracle bit for bit; the fast mode must agree within 1e-12 on every amplitude.
With measurements the outcomes must equal the oracle's and the amplitudes agree
within 1e-12 (the collapse scale comes from a sum taken in another order).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import rng
from spinoza_gb300.circuit import Program, QuantumCircuit, execute_host
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu

TOL = 1e-12
ONE_QUBIT = [nat.H, nat.X, nat.Y, nat.Z, nat.P, nat.RX, nat.RY, nat.RZ, nat.U]
CATEGORIES = ["rot", "cx", "cdiag", "swap", "mc", "bitflip", "layer"]
WEIGHTS = [0.34, 0.18, 0.16, 0.08, 0.12, 0.04, 0.08]


def fuzz_circuit(n: int, ngates: int, seed: int, measure: bool = False) -> np.ndarray:
    r = np.random.default_rng(seed)
    rows = []

    def qubit():
        # a third of the picks land on the top three qubits (outside a tile when n > 10)
        if n > 3 and r.random() < 0.33:
            return int(r.integers(n - 3, n))
        return int(r.integers(0, n))

    def add(kind, target, p=(0.0, 0.0, 0.0), ck=nat.CONTROLS_NONE, cm=0, zeros=0, q0=0, q1=0):
        rows.append(((kind, q0, q1, 0, tuple(p)), target, ck, cm, zeros))

    measured = []
    while len(rows) < ngates:
        cat = str(r.choice(CATEGORIES, p=WEIGHTS))
        if measure and r.random() < 0.03:
            t = qubit()
            add(nat.M, t, (float(r.random()), 0.0, 0.0))
            measured.append(t)
            continue
        if cat == "rot":
            add(int(r.choice(ONE_QUBIT)), qubit(), r.uniform(-np.pi, np.pi, 3))
        elif cat in ("cx", "cdiag") and n >= 2:
            if measured and r.random() < 0.3:
                c = int(r.choice(measured))  # a classical condition
            else:
                c = qubit()
            t = qubit()
            if t == c:
                t = (c + 1 + int(r.integers(0, n - 1))) % n
            kind = nat.X if cat == "cx" else int(r.choice([nat.Z, nat.P, nat.RZ]))
            add(kind, t, r.uniform(-np.pi, np.pi, 3), nat.CONTROLS_SINGLE, 1 << c)
        elif cat == "swap" and n >= 2:
            a, b = (int(x) for x in r.choice(n, 2, replace=False))
            add(nat.SWAP, 0, q0=a, q1=b)
        elif cat == "mc" and n >= 3:
            q = r.permutation(n)
            nc = int(r.integers(2, min(4, n - 1) + 1))
            ctrls = [int(c) for c in q[1:1 + nc]]
            cm = sum(1 << c for c in ctrls)
            ck, zeros = nat.CONTROLS_ONES, 0
            if r.random() < 0.5:
                ck, zeros = nat.CONTROLS_MIXED, 1 << ctrls[int(r.integers(0, nc))]
            add(int(r.choice(ONE_QUBIT)), int(q[0]), r.uniform(-np.pi, np.pi, 3), ck, cm, zeros)
        elif cat == "bitflip":
            add(nat.BITFLIP, qubit(), (0.5, float(r.random()), 0.0))
        elif cat == "layer":
            for t in range(n):
                add(nat.RY, t, (float(r.uniform(-np.pi, np.pi)), 0.0, 0.0))
            for t in range(n if n > 2 else n - 1):
                c, tt = t, (t + 1) % n
                if c != tt:
                    add(nat.Z, tt, ck=nat.CONTROLS_SINGLE, cm=1 << c)
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, row in enumerate(rows):
        ops[i] = row
    return ops


def _oracle(ops, init):
    re, im = init[0].copy(), init[1].copy()
    tr = oracle.execute(ops, re, im)
    return (re, im), tr


def _gpu(ops, init, fused=True, fast=False):
    s = State.from_arrays(*init)
    qc = QuantumCircuit.from_state(s, fused=fused, fast=fast)
    qc.execute_ops(ops)
    return s.to_numpy(), (qc.qubit_tracker.c.measured, qc.qubit_tracker.c.values)


def _maxdiff(a, b):
    return max(float(np.max(np.abs(a[0] - b[0]))), float(np.max(np.abs(a[1] - b[1]))))


def _same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


CASES = [(n, seed) for n in range(1, 21) for seed in range(3)]


@pytest.mark.parametrize("n,seed", CASES)
def test_fuzz_exact_fast_program(gpu, n, seed):
    init = rng.uniform_state(n, 500 + seed)
    ops = fuzz_circuit(n, 300, 1000 * n + seed)
    o, _ = _oracle(ops, init)
    g, _ = _gpu(ops, init)
    assert _same(g, o), _maxdiff(g, o)
    f, _ = _gpu(ops, init, fast=True)
    assert _maxdiff(f, o) <= TOL
    h = (init[0].copy(), init[1].copy())
    execute_host(ops, h[0], h[1])
    assert _same(h, o), _maxdiff(h, o)
    for fast in (False, True):
        s = State.from_arrays(*init)
        prog = Program(n, ops, fast=fast)
        try:
            prog.run(s)
            p = s.to_numpy()
        finally:
            prog.close()
        if fast:
            assert _maxdiff(p, o) <= TOL
        else:
            assert _same(p, o), _maxdiff(p, o)


@pytest.mark.parametrize("n,seed", [(12, 7), (18, 8), (20, 9)])
def test_fuzz_long_circuits(gpu, n, seed):
    """1500 gates: the fused planner's longest runs and the fast mode's drift."""
    init = rng.uniform_state(n, 600 + seed)
    ops = fuzz_circuit(n, 1500, 3000 * n + seed)
    o, _ = _oracle(ops, init)
    g, _ = _gpu(ops, init)
    assert _same(g, o), _maxdiff(g, o)
    f, _ = _gpu(ops, init, fast=True)
    assert _maxdiff(f, o) <= TOL


@pytest.mark.parametrize("n,seed", [(3, 5), (5, 0), (8, 6), (9, 1), (12, 2), (14, 3), (17, 4), (20, 10)])
def test_fuzz_measurements(gpu, n, seed):
    init = rng.normal_state(n, 700 + seed)
    ops = fuzz_circuit(n, 250, 2000 * n + seed, measure=True)
    assert np.any(ops["gate"]["kind"] == nat.M)
    o, otr = _oracle(ops, init)
    for fused, fast in ((True, False), (True, True), (False, False)):
        g, gtr = _gpu(ops, init, fused, fast)
        assert gtr == otr, (fused, fast)
        assert _maxdiff(g, o) <= TOL, (fused, fast)
