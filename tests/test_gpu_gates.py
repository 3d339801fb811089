"""GPU gate kernels vs the oracle, through the C ABI.

The kernels perform the reference's own floating-point operations in the same
order, so single-gate results must be bit-identical to the oracle's; the
assertion is exact equality (the 1e-12 parity bound is implied)."""
import itertools

import numpy as np
import pytest

import oracle
import refcases as rc
from spinoza_gb300 import gates as G
from spinoza_gb300 import rng
from spinoza_gb300.core import State
from spinoza_gb300.gates import Gate

pytestmark = pytest.mark.gpu

ONE_QUBIT = [Gate.H, Gate.X, Gate.Y, Gate.Z, Gate.P(0.7), Gate.RX(1.1), Gate.RY(-0.4), Gate.RZ(2.2),
             Gate.U(0.3, 1.4, -2.5), Gate.U(2.0, 3.0, 1.0)]


def _og(g):
    return oracle.gate(g.kind, g.params, *g.qubits)


def _pair(n, seed):
    re, im = rng.uniform_state(n, seed)
    return State.from_arrays(re, im), re.copy(), im.copy()


def _assert_same(s, re, im):
    gre, gim = s.to_numpy()
    assert np.array_equal(gre, re) and np.array_equal(gim, im), (
        f"max |d| = {max(np.max(np.abs(gre - re)), np.max(np.abs(gim - im)))}")


@pytest.mark.parametrize("n", [1, 2, 3, 5, 9])
@pytest.mark.parametrize("g", ONE_QUBIT, ids=repr)
def test_apply_every_target(gpu, g, n):
    s, re, im = _pair(n, 100 + n)
    for t in range(n):
        G.apply(g, s, t)
        oracle.apply(_og(g), re, im, t)
    _assert_same(s, re, im)


@pytest.mark.parametrize("g", ONE_QUBIT, ids=repr)
def test_c_apply_every_pair(gpu, g):
    n = 5
    s, re, im = _pair(n, 7)
    for c, t in itertools.permutations(range(n), 2):
        G.c_apply(g, s, c, t)
        oracle.c_apply(_og(g), re, im, c, t)
    _assert_same(s, re, im)


@pytest.mark.parametrize("g", ONE_QUBIT, ids=repr)
def test_mc_apply_every_mask_with_zeros(gpu, g):
    """Every target, every control set of size 2-3, every zeros subset, n = 5."""
    n = 5
    s, re, im = _pair(n, 8)
    for t in range(n):
        others = [q for q in range(n) if q != t]
        for r in (2, 3):
            for ctrls in itertools.combinations(others, r):
                for nz in range(len(ctrls) + 1):
                    zeros = ctrls[:nz]
                    G.mc_apply(g, s, ctrls, zeros, t)
                    oracle.mc_apply(_og(g), re, im, ctrls, zeros, t)
    _assert_same(s, re, im)


def test_cc_apply(gpu):
    n = 6
    s, re, im = _pair(n, 9)
    for c0, c1, t in [(0, 1, 2), (5, 0, 3), (2, 4, 0), (1, 3, 5)]:
        for g in (Gate.X, Gate.RY(0.3), Gate.U(0.1, 0.2, 0.3)):
            G.cc_apply(g, s, c0, c1, t)
            oracle.cc_apply(_og(g), re, im, c0, c1, t)
    _assert_same(s, re, im)


def test_swap_every_pair_and_controlled(gpu):
    n = 6
    s, re, im = _pair(n, 10)
    for a, b in itertools.permutations(range(n), 2):
        G.apply(Gate.SWAP(a, b), s, 0)
        oracle.apply(oracle.gate(oracle.SWAP, (), a, b), re, im, 0)
    G.c_apply(Gate.SWAP(1, 4), s, 0, 0)
    oracle.c_apply(oracle.gate(oracle.SWAP, (), 1, 4), re, im, 0, 0)
    G.mc_apply(Gate.SWAP(0, 5), s, [2, 3], [3], 0)
    oracle.mc_apply(oracle.gate(oracle.SWAP, (), 0, 5), re, im, [2, 3], [3], 0)
    _assert_same(s, re, im)


@pytest.mark.parametrize("n", [16, 21])
def test_vector_paths_at_larger_sizes(gpu, n):
    """The double2 paths (targets and controls >= 1), target 0, control 0."""
    s, re, im = _pair(n, 12)
    plan = [(Gate.H, (), n - 1), (Gate.U(1, 2, 3), (), 0), (Gate.RX(0.4), (0,), 5), (Gate.RZ(0.9), (3,), 0),
            (Gate.P(0.2), (0, n - 1), 1), (Gate.Y, (2,), n - 2), (Gate.RY(0.5), (n - 1, 1), 4)]
    for g, ctrls, t in plan:
        G.mc_apply(g, s, ctrls, None, t)
        oracle.mc_apply(_og(g), re, im, ctrls, None, t)
    _assert_same(s, re, im)


def test_bit_flip_noise(gpu):
    """gates.rs:2173-2195: prob 0 leaves the state, prob 1 is X."""
    s, re, im = _pair(1, 3)
    G.apply(Gate.BitFlipNoise(0.0, draw=0.5), s, 0)
    _assert_same(s, re, im)
    G.apply(Gate.BitFlipNoise(1.0, draw=0.5), s, 0)
    _assert_same(s, re[::-1].copy(), im[::-1].copy())


def test_errors_are_raised_not_faulted(gpu):
    s = State(3)
    with pytest.raises(ValueError):
        G.apply(Gate.H, s, 3)
    with pytest.raises(ValueError):
        G.c_apply(Gate.X, s, 1, 1)
    with pytest.raises(ValueError):
        G.mc_apply(Gate.X, s, [0, 0], None, 2)
    with pytest.raises(NotImplementedError):
        G.apply(Gate.M, s, 0)
    with pytest.raises(ValueError):
        State(0)


@pytest.mark.parametrize("case", rc.ALL_CASES, ids=lambda c: c.__name__[5:])
def test_reference_known_answers_on_gpu(gpu, case):
    assert case(rc.GpuBackend()) > 0


@pytest.mark.parametrize("via", ["append", "c_append", "mc_append"])
def test_reference_value_encoding_on_gpu(gpu, via):
    assert rc.case_value_encoding(rc.GpuBackend(), via) > 0


def test_qcbm_20_gpu_equals_oracle_bitwise(gpu):
    o = rc.qcbm_functional(rc.OracleBackend(), 20)
    g = rc.qcbm_functional(rc.GpuBackend(), 20)
    gre, gim = g.to_numpy()
    assert np.array_equal(gre, o[0]) and np.array_equal(gim, o[1])
