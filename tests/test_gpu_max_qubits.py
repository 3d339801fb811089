"""The largest state a handle takes: 34 qubits (2 x 128 GiB).

A fused circuit on qubits {0, 17, 33} (64-bit tile indices, the top qubit
outside every tile) runs on a state filled from the counter-based stream; its
result is checked on sampled groups of the 8 amplitudes that share all other
bits, against the oracle running the same circuit on those 8 amplitudes as a
3-qubit state (qubit 0 -> 0, 17 -> 1, 33 -> 2).  Bit-exact in the exact mode,
1e-12 in fast mode.
"""
from __future__ import annotations

import gc

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import rng
from spinoza_gb300.circuit import QuantumCircuit
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu

N_QUBITS = 34
QUBITS = (0, 17, 33)
GROUPS = 1 << 16
SEED = 21


def _circuit(qmap):
    """A circuit on three qubits, named through qmap (big state or packed)."""
    a, b, c = qmap
    rows = []

    def add(kind, target, p=(0.0, 0.0, 0.0), ck=nat.CONTROLS_NONE, cm=0, q0=0, q1=0):
        rows.append(((kind, q0, q1, 0, tuple(p)), target, ck, cm, 0))

    add(nat.H, c)
    add(nat.X, a, ck=nat.CONTROLS_SINGLE, cm=1 << c)
    add(nat.RY, b, (0.3, 0, 0))
    add(nat.U, c, (0.7, -1.1, 2.3))
    add(nat.P, a, (0.45, 0, 0), nat.CONTROLS_SINGLE, 1 << b)
    add(nat.SWAP, 0, q0=a, q1=c)
    add(nat.RX, a, (-0.8, 0, 0))
    add(nat.Z, b, ck=nat.CONTROLS_SINGLE, cm=1 << c)
    add(nat.U, b, (1.9, 0.2, -0.6))
    add(nat.RZ, c, (0.35, 0, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    return ops


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
def test_34_qubit_state_sampled_groups(gpu, fast):
    import torch

    n = N_QUBITS
    gc.collect()  # states of earlier tests, and torch's cached blocks
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    if free < (16 << n) + (4 << 30):
        pytest.skip(f"needs {16 << n >> 30} GiB of free device memory, {free >> 30} GiB free")
    re = torch.empty(1 << n, dtype=torch.float64, device="cuda")
    im = torch.empty_like(re)
    try:
        s = State.from_torch(re, im)
        s.fill_random(SEED, "uniform", normalise=False)
        qc = QuantumCircuit.from_state(s, fast=fast)
        qc.execute_ops(_circuit(QUBITS))
        s.synchronize()

        gen = np.random.default_rng(34)
        mask = np.uint64(sum(1 << q for q in QUBITS))
        base = gen.integers(0, 1 << n, size=GROUPS, dtype=np.uint64) & ~mask
        off = np.array([sum(1 << QUBITS[b] for b in range(3) if (j >> b) & 1) for j in range(8)], dtype=np.uint64)
        idx = (base[:, None] | off[None, :]).reshape(-1)
        ti = torch.from_numpy(idx.astype(np.int64)).to(re.device)
        gre = re.index_select(0, ti).cpu().numpy()
        gim = im.index_select(0, ti).cpu().numpy()
        del s
    finally:
        del re, im
        torch.cuda.empty_cache()

    ore, oim = rng.uniform_amplitudes(SEED, idx)
    oracle.execute(_circuit((0, 1, 2)), ore, oim)
    d = max(float(np.max(np.abs(gre - ore))), float(np.max(np.abs(gim - oim))))
    if fast:
        assert d <= 1e-12, d
    else:
        assert np.array_equal(gre, ore) and np.array_equal(gim, oim), d
