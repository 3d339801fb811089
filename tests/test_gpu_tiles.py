"""The fused executor's tile geometry (spz_state_set_tile) and its autotuner:
every geometry gives the exact mode's bit-identical result (checked against
the oracle), and the autotuner picks a candidate, sets it and caches it."""
import numpy as np
import pytest

import oracle
from spinoza_gb300 import circuit, rng
from spinoza_gb300.circuit import QuantumCircuit
from spinoza_gb300.core import State

from test_gpu_circuits import brickwork, random_circuit

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [6, 12, 16])
def test_every_tile_geometry_is_bit_identical(gpu, n):
    init = rng.normal_state(n, 300 + n)
    for ops in (brickwork(n, 3), random_circuit(n, 250, 7 * n)):
        re, im = init[0].copy(), init[1].copy()
        oracle.execute(ops, re, im)
        for k, t in [(10, 64), (10, 32), (9, 64), (8, 32), (6, 64), (4, 32)]:
            s = State.from_arrays(*init)
            s.set_tile(k, t)
            QuantumCircuit.from_state(s).execute_ops(ops)
            gre, gim = s.to_numpy()
            assert np.array_equal(gre, re) and np.array_equal(gim, im), (k, t)


def test_set_tile_rejects_bad_geometry(gpu):
    s = State(5)
    with pytest.raises(ValueError):
        s.set_tile(11, 64)
    with pytest.raises(ValueError):
        s.set_tile(10, 48)


def test_executor_autotuner_sets_and_caches(gpu, tmp_path, monkeypatch):
    monkeypatch.setenv("SPZ_AUTOTUNE_CACHE", str(tmp_path))
    n = 14
    ops = brickwork(n, 4)
    s = State(n)
    best = circuit.autotune_executor(s, ops, fast=True, candidates=[(10, 64), (9, 32)], reps=1)
    assert (best["tile_qubits"], best["threads"]) in [(10, 64), (9, 32)] and len(best["candidates"]) == 2
    assert (tmp_path / "executor_autotune.json").exists()
    again = circuit.autotune_executor(State(n), ops, fast=True, candidates=[(8, 64)])
    assert again == best  # from the cache
    # the tuned state still computes the fast-mode result of the default geometry
    s.reset_zero()
    QuantumCircuit.from_state(s, fast=True).execute_ops(ops)
    d = State(n)
    QuantumCircuit.from_state(d, fast=True).execute_ops(ops)
    (a, b), (c, e) = s.to_numpy(), d.to_numpy()
    assert max(np.max(np.abs(a - c)), np.max(np.abs(b - e))) <= 1e-12
