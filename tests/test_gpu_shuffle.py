"""Warp-shuffle runs in the fused tile passes (SPZ_EXEC_SHUFFLE): runs of
gates whose pairs lie in rows of 32 amplitudes are applied in registers with
__shfl_xor_sync and no block barrier between them.  Each lane forms its own
member's outputs with the same operations, in the same order, as the
shared-memory ops, so results must be bit-identical to the default executor
(exact and fast mode), and the exact mode to the oracle."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import rng
from spinoza_gb300.circuit import Program
from spinoza_gb300.core import State

from test_gpu_circuits import brickwork, qft_with_swaps, random_circuit

pytestmark = pytest.mark.gpu


def low_qubit_circuit(n, ngates, seed):
    """Mostly uncontrolled gates on qubits 0..4 (the ones a run can hold), with
    controlled X / Y / Z (controls anywhere) and some gates elsewhere."""
    r = np.random.default_rng(seed)
    ops = np.zeros(ngates, dtype=nat.OP_DTYPE)
    kinds = [nat.H, nat.X, nat.Y, nat.Z, nat.P, nat.RX, nat.RY, nat.RZ, nat.U]
    for i in range(ngates):
        k = int(r.choice(kinds))
        t = int(r.integers(0, min(5, n))) if r.random() < 0.8 else int(r.integers(0, n))
        others = [q for q in range(n) if q != t]
        nc = 0
        if k in (nat.X, nat.Y, nat.Z) and r.random() < 0.5:
            nc = int(r.integers(1, 3))
        ctrls = [int(c) for c in r.choice(others, size=nc, replace=False)] if nc else []
        ck = [nat.CONTROLS_NONE, nat.CONTROLS_SINGLE, nat.CONTROLS_ONES][nc]
        zeros = 0
        if nc == 2 and r.random() < 0.5:
            ck = nat.CONTROLS_MIXED
            zeros = 1 << ctrls[0]
        p = r.uniform(-math.pi, math.pi, 3)
        ops[i] = ((k, t, 0, 0, p), t, ck, sum(1 << c for c in ctrls), zeros)
    return ops


def _run(ops, init, flags):
    s = State.from_arrays(*init)
    tr = nat.spz_tracker(0, 0)
    st = nat.spz_exec_stats()
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    nat.check(nat.lib().spz_circuit_execute(s.handle, nat.ptr(ops), len(ops), nat.byref(tr), flags, nat.byref(st)))
    return s.to_numpy(), st


@pytest.mark.parametrize("n", [7, 9, 12, 17, 20])
def test_shuffle_runs_are_bit_identical(gpu, n):
    init = rng.normal_state(n, 200 + n)
    circuits = {"brickwork": brickwork(n, 3), "random": random_circuit(n, 300, n),
                "qft": qft_with_swaps(n), "low": low_qubit_circuit(n, 400, n)}
    for name, ops in circuits.items():
        for fast in (False, True):
            base = nat.EXEC_FAST if fast else nat.EXEC_DEFAULT
            (a_re, a_im), st = _run(ops, init, base)
            (b_re, b_im), st2 = _run(ops, init, base | nat.EXEC_SHUFFLE)
            assert np.array_equal(a_re, b_re) and np.array_equal(a_im, b_im), (name, fast)
            assert st2.tile_passes == st.tile_passes and st.shuffle_gates == 0
            if name == "low" or (name == "brickwork" and fast):
                assert st2.shuffle_gates > 0, (name, fast)
            if not fast:
                re, im = init[0].copy(), init[1].copy()
                oracle.execute(ops, re, im)
                assert np.array_equal(b_re, re) and np.array_equal(b_im, im), name


def test_shuffle_program_replay_matches(gpu):
    n = 16
    ops = low_qubit_circuit(n, 300, 5)
    init = rng.normal_state(n, 7)
    for fast in (False, True):
        (want_re, want_im), _ = _run(ops, init, nat.EXEC_FAST if fast else nat.EXEC_DEFAULT)
        prog = Program(n, ops, fast=fast, extra_flags=nat.EXEC_SHUFFLE)
        assert prog.stats()["shuffle_gates"] > 0
        s = State.from_arrays(*init)
        prog.run(s)
        got_re, got_im = s.to_numpy()
        assert np.array_equal(got_re, want_re) and np.array_equal(got_im, want_im)
        prog.close()


def test_shuffle_with_small_tiles_and_one_warp(gpu):
    """Tile geometries at the edge of the run layout: 2^7 amplitudes (four rows,
    one warp busy) and 32-thread blocks."""
    n = 14
    ops = low_qubit_circuit(n, 300, 9)
    init = rng.normal_state(n, 11)
    for tile_qubits, threads in ((7, 64), (7, 32), (8, 32), (10, 32)):
        for fast in (False, True):
            base = nat.EXEC_FAST if fast else nat.EXEC_DEFAULT
            outs = []
            for flags in (base, base | nat.EXEC_SHUFFLE):
                s = State.from_arrays(*init)
                s.set_tile(tile_qubits, threads)
                tr, st = nat.spz_tracker(0, 0), nat.spz_exec_stats()
                o = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
                nat.check(nat.lib().spz_circuit_execute(s.handle, nat.ptr(o), len(o), nat.byref(tr), flags,
                                                        nat.byref(st)))
                outs.append(s.to_numpy())
            assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1]), \
                (tile_qubits, threads, fast)
