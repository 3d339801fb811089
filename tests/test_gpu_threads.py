"""Handles driven from several host threads at once.

Each thread owns its states (one stream each) and runs fused, fast and adjoint
work on them while the others do the same; every result must equal what the
same call gives alone (the oracle for circuits; a serial run for gradients).
The library's one-time per-device setup (kernel attributes, launch shapes) is
shared between the threads.
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

import oracle
from spinoza_gb300 import adjoint, core, rng
from spinoza_gb300.circuit import QuantumCircuit
from spinoza_gb300.core import State
from test_gpu_fuzz import fuzz_circuit

pytestmark = pytest.mark.gpu

THREADS = 4


def _oracle(ops, init):
    re, im = init[0].copy(), init[1].copy()
    oracle.execute(ops, re, im)
    return re, im


def test_threads_run_circuits_and_gradients_concurrently(gpu):
    cases = []
    for k in range(THREADS):
        n = 14 + k
        init = rng.uniform_state(n, 900 + k)
        ops = fuzz_circuit(n, 200, 7000 + k)
        cases.append((n, init, ops, _oracle(ops, init)))
    ansatz, pidx = adjoint.hardware_efficient_ansatz(12, 3)
    theta = (rng.uniforms(61, len(pidx)) * 2 - 1) * np.pi
    ham = core.ising_hamiltonian(np.linspace(-1, 1, 11), np.linspace(0.5, -0.5, 12))
    opsv = adjoint.set_params(ansatz, pidx, theta)
    ref_state = State(12)
    e_ref, g_ref = adjoint.adjoint_gradient(ref_state, opsv, pidx, ham)

    errors: list[str] = []
    start = threading.Barrier(THREADS)

    def work(k):
        try:
            n, init, ops, want = cases[k]
            start.wait()
            for rep in range(3):
                for fast in (False, True):
                    s = State.from_arrays(*init)
                    qc = QuantumCircuit.from_state(s, fast=fast)
                    qc.execute_ops(ops)
                    got = s.to_numpy()
                    d = max(float(np.max(np.abs(got[0] - want[0]))), float(np.max(np.abs(got[1] - want[1]))))
                    if fast and d > 1e-12:
                        errors.append(f"thread {k} rep {rep} fast: max |d| = {d}")
                    if not fast and not (np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])):
                        errors.append(f"thread {k} rep {rep} exact: max |d| = {d}")
                s = State(12)
                e, g = adjoint.adjoint_gradient(s, opsv, pidx, ham)
                if e != e_ref or not np.array_equal(g, g_ref):
                    errors.append(f"thread {k} rep {rep}: gradient differs from the serial run")
        except Exception as exc:  # reported below, with the thread
            errors.append(f"thread {k}: {exc!r}")

    threads = [threading.Thread(target=work, args=(k,)) for k in range(THREADS)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads), "a worker thread did not finish"
    assert not errors, errors
