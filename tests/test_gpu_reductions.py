"""Measurement, probability, expectation and sampling reductions vs the oracle."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import core, measurement, rng
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 4, 12, 19])
def test_prob0_and_qubit_expectation(gpu, n):
    re, im = rng.normal_state(n, 10 + n)
    s = State.from_arrays(re, im)
    for t in range(n):
        assert abs(measurement.prob0(s, t) - oracle.prob0(re, im, t)) < 1e-13
        assert abs(core.qubit_expectation_value(s, t) - oracle.qubit_expectation_value(re, im, t)) < 1e-13


@pytest.mark.parametrize("obs", ["x", "y", "z"])
def test_xyz_expectation_value(gpu, obs):
    n = 13
    re, im = rng.normal_state(n, 3)
    s = State.from_arrays(re, im)
    targets = list(range(n))
    got = core.xyz_expectation_value(obs, s, targets)
    want = oracle.xyz_expectation_value(obs, re, im, targets)
    np.testing.assert_allclose(got, want, atol=1e-13, rtol=0)


def test_xyz_rejects_bad_observable(gpu):
    """core.rs:303-310 (#[should_panic])."""
    with pytest.raises(ValueError):
        core.xyz_expectation_value("a", State(1), [0])


@pytest.mark.parametrize("n", [6, 15])
def test_pauli_sum_matches_oracle(gpu, n):
    """General Pauli strings: diagonal, X-type and Y-containing terms."""
    re, im = rng.normal_state(n, 4)
    s = State.from_arrays(re, im)
    r = np.random.default_rng(n)
    terms = []
    for _ in range(40):
        x = int(r.integers(0, 1 << n)) if r.random() < 0.6 else 0
        z = int(r.integers(0, 1 << n)) if r.random() < 0.7 else 0
        terms.append((float(r.normal()), x, z))
    arr = core.pauli_terms(terms)
    got = core.pauli_expectation(s, arr)
    want = oracle.pauli_expectation(re, im, arr)
    assert abs(got - want) < 1e-12 * max(1.0, abs(want))


@pytest.mark.parametrize("n", [2, 7, 14, 19])
def test_pauli_sum_tile_path(gpu, n):
    """Terms that fit the fused tile passes: X/Y masks of up to 3 qubits, any Z
    mask, identity terms, and more than 8 diagonal terms (several chunks)."""
    re, im = rng.normal_state(n, 40 + n)
    s = State.from_arrays(re, im)
    r = np.random.default_rng(100 + n)
    terms = [(0.5, 0, 0)]
    for _ in range(30):
        z = int(r.integers(0, 1 << n))
        terms.append((float(r.normal()), 0, z))
    for _ in range(40):
        qs = r.choice(n, size=min(n, int(r.integers(1, 4))), replace=False)
        x = sum(1 << int(q) for q in qs)
        z = int(r.integers(0, 1 << n)) if r.random() < 0.5 else 0
        terms.append((float(r.normal()), x, z))
    arr = core.pauli_terms(terms)
    got = core.pauli_expectation(s, arr)
    want = oracle.pauli_expectation(re, im, arr)
    assert abs(got - want) < 1e-12 * max(1.0, sum(abs(t[0]) for t in terms))


def test_ising_hamiltonian_chain_form(gpu):
    n = 16
    re, im = rng.normal_state(n, 3)
    s = State.from_arrays(re, im)
    ab = rng.uniforms(5, 2 * n)
    a = np.sqrt(-2 * np.log1p(-ab[:n - 1])) * np.cos(2 * math.pi * ab[n:2 * n - 1])
    b = np.sqrt(-2 * np.log1p(-ab[n - 1:2 * n - 1])) * np.sin(2 * math.pi * ab[:n])
    H = core.ising_hamiltonian(a, b)
    got = core.pauli_expectation(s, H)
    want = oracle.pauli_expectation(re, im, H)
    assert abs(got - want) < 1e-12 * max(1.0, abs(want))


def test_measure_qubit_drawn_outcomes_match_oracle(gpu):
    n = 10
    re, im = rng.normal_state(n, 8)
    s = State.from_arrays(re, im)
    ore, oim = re.copy(), im.copy()
    u = rng.uniforms(44, n)
    for t in range(n):
        v = measurement.measure_qubit(s, t, reset=True, u=float(u[t]))
        ov, _ = oracle.measure_qubit(ore, oim, t, True, None, float(u[t]))
        assert v == ov
    gre, gim = s.to_numpy()
    np.testing.assert_allclose(gre, ore, atol=1e-13)
    np.testing.assert_allclose(gim, oim, atol=1e-13)
    assert abs(s.norm_sqr() - 1.0) < 1e-12


def test_measure_repeatability(gpu):
    """circuit.rs:825-889: measuring again after a measurement repeats the values."""
    n = 12
    s = State.from_arrays(*rng.normal_state(n, 21))
    first = [measurement.measure_qubit(s, t, reset=False, u=float(x)) for t, x in enumerate(rng.uniforms(1, n))]
    second = [measurement.measure_qubit(s, t, reset=False, u=float(x)) for t, x in enumerate(rng.uniforms(2, n))]
    assert first == second


@pytest.mark.parametrize("n,shots", [(3, 1000), (10, 20000), (18, 100000)])
def test_sampling_bit_exact(gpu, n, shots):
    """Outcomes are bit-identical to the oracle's for the same uniforms."""
    re, im = rng.normal_state(n, 3)
    s = State.from_arrays(re, im)
    u = rng.uniforms(4, shots)
    got = core.sample(s, u)
    want = oracle.sample(re, im, u)
    assert np.array_equal(got, want)


def test_sampling_basis_states(gpu):
    """core.rs:271-291: a basis state always samples to itself."""
    n = 3
    for i in range(1 << n):
        re = np.zeros(1 << n)
        re[i] = 1.0
        s = State.from_arrays(re, np.zeros(1 << n))
        hist = core.reservoir_sampling(s, 1 << n, (1 << n) * 10000).get_outcome_count()
        assert hist == {i: 1 << n}


def test_device_fill_uniform_matches_host_stream(gpu):
    n = 14
    s = State(n)
    s.fill_random(99, "uniform", normalise=False)
    re, im = s.to_numpy()
    hre, him = rng.uniform_state(n, 99)
    assert np.array_equal(re, hre) and np.array_equal(im, him)
    s.fill_random(99, "normal", normalise=True)
    assert abs(s.norm_sqr() - 1.0) < 1e-12
