"""Parity of the 33-qubit per-gate sweep (a 128 GiB state) by sampled amplitude groups.

The host cannot hold 2^33 amplitudes, so each check regenerates only the input
amplitudes it needs from the counter-based stream that filled the device state
(rng.uniform_amplitudes), and compares the device's outputs with the oracle's
update of the same amplitudes packed into a small state.  A gate on target t
with controls C changes amplitude i only through the 2^(1+|C|) amplitudes that
differ from i in bits {t} u C, so the packed update is the full update
restricted to those amplitudes, and the comparison is bit-exact.

Gates as in the sweep: H, RZ(0.7), CX with control (t+1) mod n and X with the
three controls (t+1..t+3) mod n, on every target; 2^15 groups per target, so
33 x 32768 = 1.08e6 sampled pairs per gate.
"""
from __future__ import annotations

import gc

import numpy as np
import pytest

import oracle
from spinoza_gb300 import gates as G
from spinoza_gb300 import rng
from spinoza_gb300.core import State
from spinoza_gb300.gates import Gate

pytestmark = pytest.mark.gpu

N_QUBITS = 33
GROUPS = 1 << 15
SEED = 11

KINDS = {
    "H": (Gate.H, lambda t, n: []),
    "RZ": (Gate.RZ(0.7), lambda t, n: []),
    "CX": (Gate.X, lambda t, n: [(t + 1) % n]),
    "MCX3": (Gate.X, lambda t, n: [(t + 1) % n, (t + 2) % n, (t + 3) % n]),
}


@pytest.fixture(scope="module")
def big_state(gpu):
    import torch

    n = N_QUBITS
    gc.collect()  # states of earlier tests, and torch's cached blocks
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    if free < (16 << n) + (8 << 30):
        pytest.skip(f"needs {16 << n >> 30} GiB of free device memory, {free >> 30} GiB free")
    re = torch.empty(1 << n, dtype=torch.float64, device="cuda")
    im = torch.empty_like(re)
    s = State.from_torch(re, im)
    yield s, re, im
    s.synchronize()
    del s, re, im
    torch.cuda.empty_cache()


def _group_offsets(loc: list[int]) -> np.ndarray:
    """Offset of packed amplitude j: bit b of j is qubit loc[b] of the big state."""
    k = len(loc)
    off = np.zeros(1 << k, dtype=np.uint64)
    for j in range(1 << k):
        for b in range(k):
            if (j >> b) & 1:
                off[j] |= np.uint64(1 << loc[b])
    return off


@pytest.mark.parametrize("kind", list(KINDS))
def test_sweep33_sampled_pairs(big_state, kind):
    import torch

    s, re, im = big_state
    n = N_QUBITS
    g, controls = KINDS[kind]
    og = oracle.gate(g.kind, g.params, *g.qubits)
    gen = np.random.default_rng(1000 + list(KINDS).index(kind))
    checked = 0
    for t in range(n):
        cs = controls(t, n)
        loc = [t] + cs
        k = len(loc)
        s.fill_random(SEED, "uniform", normalise=False)
        if not cs:
            G.apply(g, s, t)
        elif len(cs) == 1:
            G.c_apply(g, s, cs[0], t)
        else:
            G.mc_apply(g, s, cs, None, t)
        mask = np.uint64(sum(1 << q for q in loc))
        base = gen.integers(0, 1 << n, size=GROUPS, dtype=np.uint64) & ~mask
        idx = (base[:, None] | _group_offsets(loc)[None, :]).reshape(-1)
        ti = torch.from_numpy(idx.astype(np.int64)).to(re.device)
        gre = re.index_select(0, ti).cpu().numpy()
        gim = im.index_select(0, ti).cpu().numpy()
        # packed state of log2(GROUPS) + k qubits: index m * 2^k + j, target at qubit 0
        ore, oim = rng.uniform_amplitudes(SEED, idx)
        if not cs:
            oracle.apply(og, ore, oim, 0)
        elif len(cs) == 1:
            oracle.c_apply(og, ore, oim, 1, 0)
        else:
            oracle.mc_apply(og, ore, oim, list(range(1, k)), None, 0)
        assert np.array_equal(gre, ore) and np.array_equal(gim, oim), (
            f"{kind} target {t}: max |d| = {max(np.max(np.abs(gre - ore)), np.max(np.abs(gim - oim)))}")
        checked += GROUPS
    assert checked >= 1_000_000
