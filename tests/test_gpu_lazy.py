"""The opt-in lazy per-gate mode (spz_state_set_lazy) against the oracle.

Uncontrolled H / RX / RY run as the gate divided by a scalar and RZ as P times
a phase, the handle carrying the pending factor; every read folds it in first.
Results equal the reference's arithmetic up to rounding, so the bar is 1e-12
on amplitudes of normalised states, and the reads (reductions, sampling,
copies, execution, the adjoint) are checked after lazy gates."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import adjoint, core, gates, rng
from spinoza_gb300.circuit import QuantumCircuit
from spinoza_gb300.core import State
from spinoza_gb300.gates import Gate

pytestmark = pytest.mark.gpu


def _random_gates(n, count, seed):
    """(kind, params, controls, target) tuples, mostly uncontrolled H/RX/RY/RZ."""
    r = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        t = int(r.integers(n))
        kind = [nat.H, nat.RX, nat.RY, nat.RZ, nat.U, nat.X, nat.Y, nat.Z, nat.P][int(r.integers(9))]
        p = (float(r.uniform(-4, 4)), float(r.uniform(-4, 4)), float(r.uniform(-4, 4)))
        ctl = []
        if n > 1 and r.random() < 0.2:
            ctl = [int(c) for c in r.choice([q for q in range(n) if q != t], size=min(n - 1, 1 + int(r.integers(2))),
                                           replace=False)]
        out.append((kind, p, ctl, t))
    return out


def _apply_both(s: State, re, im, seq):
    for kind, p, ctl, t in seq:
        g = Gate(kind, p)
        og = oracle.gate(kind, p)
        if not ctl:
            gates.apply(g, s, t)
            oracle.apply(og, re, im, t)
        elif len(ctl) == 1:
            gates.c_apply(g, s, ctl[0], t)
            oracle.c_apply(og, re, im, ctl[0], t)
        else:
            gates.mc_apply(g, s, ctl, None, t)
            oracle.mc_apply(og, re, im, ctl, None, t)


def _maxdiff(s: State, re, im) -> float:
    gre, gim = s.to_numpy()
    return max(float(np.max(np.abs(gre - re))), float(np.max(np.abs(gim - im))))


@pytest.mark.parametrize("n,count", [(1, 40), (2, 60), (11, 400), (17, 200)])
def test_lazy_gate_sequences_match_oracle(gpu, n, count):
    re, im = rng.normal_state(n, 70 + n)
    s = State.from_arrays(re, im)
    s.set_lazy(True)
    re, im = re.copy(), im.copy()
    _apply_both(s, re, im, _random_gates(n, count, n))
    assert _maxdiff(s, re, im) <= 1e-12


def test_lazy_every_target_and_kind(gpu):
    n = 9
    for kind, p in [(nat.H, ()), (nat.RX, (0.3,)), (nat.RX, (2.9,)), (nat.RY, (-0.4,)), (nat.RY, (3.0,)),
                    (nat.RZ, (1.3,))]:
        re, im = rng.normal_state(n, 5)
        s = State.from_arrays(re, im)
        s.set_lazy(True)
        re, im = re.copy(), im.copy()
        for t in range(n):
            gates.apply(Gate(kind, p), s, t)
            oracle.apply(oracle.gate(kind, p), re, im, t)
        assert _maxdiff(s, re, im) <= 1e-12, (kind, p)


def test_lazy_deep_sequence_settles_before_overflow(gpu):
    """4000 lazy H gates grow the stored arrays by 2^1000 in total: the factor
    is folded in on the way, so nothing overflows."""
    n = 3
    s = State(n)
    s.set_lazy(True)
    re, im = oracle.zero_state(n)
    for k in range(4000):
        gates.apply(Gate.H, s, k % n)
    for k in range(4000):
        oracle.apply(oracle.gate(oracle.H), re, im, k % n)
    assert _maxdiff(s, re, im) <= 1e-12
    assert abs(s.norm_sqr() - 1.0) <= 1e-12


def test_lazy_reads_fold_the_factor_in(gpu):
    n = 12
    re0, im0 = rng.normal_state(n, 9)
    s = State.from_arrays(re0, im0)
    s.set_lazy(True)
    re, im = re0.copy(), im0.copy()
    seq = _random_gates(n, 120, 3)
    _apply_both(s, re, im, seq)
    # reductions
    assert abs(s.norm_sqr() - 1.0) <= 1e-12
    for t in (0, 5, 11):
        assert abs(core.qubit_expectation_value(s, t) - oracle.qubit_expectation_value(re, im, t)) <= 1e-12
    for obs in "xyz":
        np.testing.assert_allclose(core.xyz_expectation_value(obs, s, [0, 7]),
                                   oracle.xyz_expectation_value(obs, re, im, [0, 7]), atol=1e-12, rtol=0)
    H = core.pauli_terms([(0.5, 0b11, 0), (-1.25, 0, 0b101), (0.75, 0b1000, 0b1000)])
    assert abs(core.pauli_expectation(s, H) - oracle.pauli_expectation(re, im, H)) <= 1e-12
    # more lazy gates, then a copy, device arrays and sampling of the settled state
    _apply_both(s, re, im, _random_gates(n, 50, 4))
    c = s.clone()
    assert _maxdiff(c, re, im) <= 1e-12
    _apply_both(s, re, im, _random_gates(n, 50, 5))
    import torch

    dre, dim = s.device_arrays()
    assert dre and dim
    gre, gim = s.to_numpy()
    u = rng.uniforms(8, 5000)
    assert np.array_equal(core.sample(s, u), oracle.sample(gre, gim, u))
    torch.cuda.synchronize()
    # execution after lazy gates (the circuit runs on the settled state)
    _apply_both(s, re, im, _random_gates(n, 30, 6))
    ops = np.zeros(2, dtype=nat.OP_DTYPE)
    ops[0] = ((nat.U, 0, 0, 0, (0.4, 0.5, 0.6)), 3, nat.CONTROLS_NONE, 0, 0)
    ops[1] = ((nat.X, 0, 0, 0, (0, 0, 0)), 4, nat.CONTROLS_SINGLE, 1 << 3, 0)
    QuantumCircuit.from_state(s).execute_ops(ops)
    oracle.execute(ops, re, im)
    assert _maxdiff(s, re, im) <= 1e-12
    # back to the exact mode settles
    _apply_both(s, re, im, _random_gates(n, 30, 7))
    s.set_lazy(False)
    gates.apply(Gate.H, s, 2)
    oracle.apply(oracle.gate(oracle.H), re, im, 2)
    assert _maxdiff(s, re, im) <= 1e-12


def test_lazy_measurement_and_adjoint(gpu):
    from spinoza_gb300 import measurement

    n = 8
    re, im = rng.normal_state(n, 21)
    s = State.from_arrays(re, im)
    s.set_lazy(True)
    re, im = re.copy(), im.copy()
    _apply_both(s, re, im, _random_gates(n, 80, 8))
    v = measurement.measure_qubit(s, 2, True, u=0.4)
    ov, _ = oracle.measure_qubit(re, im, 2, True, None, 0.4)
    assert v == ov
    assert _maxdiff(s, re, im) <= 1e-12
    # adjoint from |0...0> after lazy gates were applied and then reset
    ops, pidx = adjoint.hardware_efficient_ansatz(n, 2)
    theta = (rng.uniforms(2, len(pidx)) * 2 - 1) * math.pi
    H = core.ising_hamiltonian(np.linspace(-1, 1, n - 1), np.linspace(0.5, -0.5, n))
    gates.apply(Gate.H, s, 0)
    s.reset_zero()
    e, g = adjoint.adjoint_gradient(s, adjoint.set_params(ops, pidx, theta), pidx, H)
    e0, g0 = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, H)
    assert e == e0 and np.array_equal(g, g0)


def test_lazy_on_wrapped_torch_arrays_needs_settle(gpu):
    import torch

    n = 10
    re0, im0 = rng.normal_state(n, 4)
    tre = torch.tensor(re0, device="cuda")
    tim = torch.tensor(im0, device="cuda")
    s = State.from_torch(tre, tim)
    s.set_lazy(True)
    re, im = re0.copy(), im0.copy()
    for t in range(n):
        gates.apply(Gate.H, s, t)
        oracle.apply(oracle.gate(oracle.H), re, im, t)
    s.settle()
    torch.cuda.synchronize()
    d = max(float(np.max(np.abs(tre.cpu().numpy() - re))), float(np.max(np.abs(tim.cpu().numpy() - im))))
    assert d <= 1e-12
