"""Failure handling without a GPU fault: allocation failures are injected on the
host (SPZ_INJECT_ALLOC_FAILURE=1 makes the library's allocation wrapper report
cudaErrorMemoryAllocation without allocating), and every call that needed
memory must return SPZ_ERR_OUT_OF_MEMORY, leave its handle usable and its
state untouched.  The reference panics on allocation failure instead."""
import os

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import adjoint, core, rng
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


class _inject:
    def __enter__(self):
        os.environ["SPZ_INJECT_ALLOC_FAILURE"] = "1"

    def __exit__(self, *exc):
        os.environ.pop("SPZ_INJECT_ALLOC_FAILURE", None)


def _code(fn):
    with pytest.raises(nat.SpzError) as info:
        fn()
    return info.value.code


def test_state_creation_reports_out_of_memory(gpu):
    with _inject():
        assert _code(lambda: State(8)) == nat.SPZ_ERR_OUT_OF_MEMORY
    assert State(8).norm_sqr() == 1.0


def test_calls_needing_scratch_fail_cleanly_and_recover(gpu):
    n = 9
    re, im = rng.normal_state(n, 3)
    s = State.from_arrays(re, im)  # no reduction scratch allocated yet
    with _inject():
        assert _code(lambda: s.norm_sqr()) == nat.SPZ_ERR_OUT_OF_MEMORY
        assert _code(lambda: core.sample(s, rng.uniforms(1, 10))) == nat.SPZ_ERR_OUT_OF_MEMORY
    gre, gim = s.to_numpy()
    assert np.array_equal(gre, re) and np.array_equal(gim, im)  # untouched
    assert abs(s.norm_sqr() - float(np.sum(re * re + im * im))) < 1e-12
    u = rng.uniforms(1, 100)
    assert np.array_equal(core.sample(s, u), oracle.sample(re, im, u))


def test_adjoint_work_vectors_fail_cleanly_and_recover(gpu):
    n = 6
    ops, pidx = adjoint.hardware_efficient_ansatz(n, 2)
    theta = np.linspace(-1.0, 1.0, len(pidx))
    H = core.ising_hamiltonian(np.ones(n - 1), np.ones(n) * 0.5)
    s = State(n)
    with _inject():
        assert _code(lambda: adjoint.adjoint_gradient(s, adjoint.set_params(ops, pidx, theta), pidx, H)) \
            == nat.SPZ_ERR_OUT_OF_MEMORY
    s.reset_zero()
    e, g = adjoint.adjoint_gradient(s, adjoint.set_params(ops, pidx, theta), pidx, H)
    e0, g0 = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, H)
    assert e == e0 and np.array_equal(g, g0)
