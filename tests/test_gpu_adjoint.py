"""Adjoint gradients vs the oracle's parameter shift and vs central differences.

Parameter shift is exact for RY/RZ (dE/dtheta = [E(theta + pi/2) - E(theta - pi/2)] / 2),
so it pins the gradient to rounding level; the tolerance written here is 1e-9."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import adjoint, core, rng
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


def _problem(n, layers, seed):
    ops, pidx = adjoint.hardware_efficient_ansatz(n, layers)
    theta = (rng.uniforms(seed, len(pidx)) * 2 - 1) * math.pi
    u = rng.uniforms(seed + 1, 4 * n)
    a = np.sqrt(-2 * np.log1p(-u[:n - 1])) * np.cos(2 * math.pi * u[n:2 * n - 1])
    b = np.sqrt(-2 * np.log1p(-u[2 * n:3 * n])) * np.cos(2 * math.pi * u[3 * n:4 * n])
    return ops, pidx, theta, core.ising_hamiltonian(a, b)


def _oracle_energy(n, ops, terms):
    re, im = oracle.zero_state(n)
    oracle.execute(ops, re, im)
    return oracle.pauli_expectation(re, im, terms)


@pytest.mark.parametrize("n,layers", [(4, 2), (9, 3)])
def test_adjoint_matches_oracle_parameter_shift(gpu, n, layers):
    ops, pidx, theta, H = _problem(n, layers, 6)
    e, g = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, H)
    e0 = _oracle_energy(n, adjoint.set_params(ops, pidx, theta), H)
    assert abs(e - e0) < 1e-12
    for j in range(len(pidx)):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += math.pi / 2
        tm[j] -= math.pi / 2
        ps = 0.5 * (_oracle_energy(n, adjoint.set_params(ops, pidx, tp), H)
                    - _oracle_energy(n, adjoint.set_params(ops, pidx, tm), H))
        assert abs(g[j] - ps) < 1e-9, (j, g[j], ps)


def _mixed_circuit(n, seed):
    """H, RX, RY, RZ, P, controlled rotations and CZ, with parameters on every
    rotation (the fast sweep turns the uncontrolled ones into lazy ops / P)."""
    from spinoza_gb300 import _native as nat

    r = np.random.default_rng(seed)
    rows, pidx = [], []
    for layer in range(3):
        for q in range(n):
            k = [nat.H, nat.RX, nat.RY, nat.RZ, nat.P][(q + layer) % 5]
            if k != nat.H:
                pidx.append(len(rows))
            rows.append(((k, 0, 0, 0, (r.uniform(-3, 3), 0, 0)), q, nat.CONTROLS_NONE, 0, 0))
        for q in range(n - 1):
            k = [nat.RY, nat.RZ, nat.Z][(q + layer) % 3]
            if k != nat.Z:
                pidx.append(len(rows))
            rows.append(((k, 0, 0, 0, (r.uniform(-3, 3), 0, 0)), q + 1, nat.CONTROLS_SINGLE, 1 << q, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, row in enumerate(rows):
        ops[i] = row
    return ops, np.array(pidx, dtype=np.uint32)


@pytest.mark.parametrize("n", [3, 7, 12])
def test_fast_adjoint_equals_exact_and_parameter_shift(gpu, n):
    """Fast mode (lazy inverses, RZ as P, scale folded into the gradients)
    gives the exact adjoint's numbers up to rounding, and the oracle's
    parameter-shift gradients within 1e-9."""
    ops, pidx = _mixed_circuit(n, 40 + n)
    _, _, _, H = _problem(n, 1, 9)
    e0, g0 = adjoint.adjoint_gradient(State(n), ops, pidx, H)
    e1, g1 = adjoint.adjoint_gradient(State(n), ops, pidx, H, fast=True)
    assert abs(e1 - e0) < 1e-12
    np.testing.assert_allclose(g1, g0, atol=1e-12, rtol=0)
    theta = ops["gate"]["p"][pidx.astype(np.int64), 0].copy()
    for j in range(0, len(pidx), max(1, len(pidx) // 6)):
        if ops["gate"]["kind"][pidx[j]] == 5 or ops["controls_kind"][pidx[j]] != 0:
            continue  # parameter shift with +-pi/2 is exact for uncontrolled RX/RY/RZ only
        tp, tm = theta.copy(), theta.copy()
        tp[j] += math.pi / 2
        tm[j] -= math.pi / 2
        ps = 0.5 * (_oracle_energy(n, adjoint.set_params(ops, pidx, tp), H) -
                    _oracle_energy(n, adjoint.set_params(ops, pidx, tm), H))
        assert abs(g1[j] - ps) < 1e-9, (j, g1[j], ps)


def test_fast_adjoint_falls_back_to_exact_for_very_deep_circuits(gpu):
    """More than 800 lazy inverses: the sweep stays exact (the scale would
    leave the exponent range); results still match the exact adjoint."""
    n, layers = 3, 300
    ops, pidx = adjoint.hardware_efficient_ansatz(n, layers)
    theta = (rng.uniforms(3, len(pidx)) * 2 - 1) * math.pi
    _, _, _, H = _problem(n, 1, 9)
    opsv = adjoint.set_params(ops, pidx, theta)
    e0, g0 = adjoint.adjoint_gradient(State(n), opsv, pidx, H)
    e1, g1 = adjoint.adjoint_gradient(State(n), opsv, pidx, H, fast=True)
    assert abs(e1 - e0) < 1e-12
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)


def test_adjoint_matches_central_differences_on_gpu(gpu):
    n, layers = 12, 3
    ops, pidx, theta, H = _problem(n, layers, 7)
    _, g = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, H)
    h = 1e-6
    for j in range(0, len(pidx), 5):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        fd = (adjoint.expectation(State(n), adjoint.set_params(ops, pidx, tp), H)
              - adjoint.expectation(State(n), adjoint.set_params(ops, pidx, tm), H)) / (2 * h)
        assert abs(g[j] - fd) < 1e-7 * max(1.0, abs(fd)), (j, g[j], fd)


def test_adjoint_controlled_rotations_and_phase(gpu):
    """P, CRX and CRY parameters (generators with control projectors)."""
    from spinoza_gb300 import _native as nat

    n = 5
    rows = [((nat.H, 0, 0, 0, (0, 0, 0)), q, 0, 0, 0) for q in range(n)]
    rows += [((nat.RX, 0, 0, 0, (0.3, 0, 0)), 1, nat.CONTROLS_SINGLE, 1 << 0, 0),
             ((nat.RY, 0, 0, 0, (-0.7, 0, 0)), 3, nat.CONTROLS_ONES, (1 << 1) | (1 << 2), 0),
             ((nat.P, 0, 0, 0, (1.1, 0, 0)), 4, nat.CONTROLS_MIXED, (1 << 0) | (1 << 2), 1 << 2),
             ((nat.RZ, 0, 0, 0, (0.4, 0, 0)), 2, 0, 0, 0),
             ((nat.U, 0, 0, 0, (0.2, 0.3, 0.4)), 0, 0, 0, 0)]
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    pidx = np.array([n, n + 1, n + 2, n + 3], dtype=np.uint32)
    H = core.pauli_terms([(0.7, 0b00011, 0), (-1.2, 0, 0b11000), (0.5, 0b10100, 0b00100), (0.3, 0b01000, 0b01001)])
    _, g = adjoint.adjoint_gradient(State(n), ops, pidx, H)
    theta = ops["gate"]["p"][pidx.astype(int), 0].copy()
    for j in range(len(pidx)):
        for sign in (+1,):
            tp, tm = theta.copy(), theta.copy()
            tp[j] += 1e-5
            tm[j] -= 1e-5
            ep = _oracle_energy(n, adjoint.set_params(ops, pidx, tp), H)
            em = _oracle_energy(n, adjoint.set_params(ops, pidx, tm), H)
            assert abs(g[j] - (ep - em) / 2e-5) < 1e-7 * sign


def test_torch_autograd_function(gpu):
    import torch

    n, layers = 6, 2
    ops, pidx, theta, H = _problem(n, layers, 9)
    t = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    e = adjoint.energy(t, n, ops, pidx, H)
    e.backward()
    _, g = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, H)
    assert abs(e.item() - _oracle_energy(n, adjoint.set_params(ops, pidx, theta), H)) < 1e-12
    np.testing.assert_array_equal(t.grad.numpy(), g)


def test_torch_autograd_function_fast(gpu):
    import torch

    n, layers = 6, 2
    ops, pidx, theta, H = _problem(n, layers, 10)
    t = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    e = adjoint.energy(t, n, ops, pidx, H, fast=True)
    e.backward()
    _, g = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, H)
    assert abs(e.item() - _oracle_energy(n, adjoint.set_params(ops, pidx, theta), H)) < 1e-12
    np.testing.assert_allclose(t.grad.numpy(), g, atol=1e-12, rtol=0)
