"""The allocation-free expectation entry point, for callers that cannot call
cudaMalloc (code inside another framework's memory pool, inside a graph
capture that must not allocate, or under a fixed memory budget).

Called through the C ABI on raw device arrays, twice in a row, and compared
with spz_xyz_expectation_value on the same state at the tolerance the other
expectation tests use (1e-13).  Collected last (test_zz_*) so that a run that
stops at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from spinoza_gb300 import _native as nat
from spinoza_gb300 import core, rng
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


def _noalloc(s: State, obs: str, targets) -> np.ndarray:
    dre, dim = s.device_arrays()
    t = np.ascontiguousarray(np.array(targets, dtype=np.uint32))
    out = np.full(len(t), np.nan)
    nat.check(nat.lib().spz_xyz_expectation_value_noalloc(
        ctypes.c_void_p(dre), ctypes.c_void_p(dim), s.n, obs.encode(), nat.ptr(t), len(t), nat.ptr(out), None))
    return out


@pytest.mark.parametrize("n", [1, 9, 18])
def test_noalloc_matches_existing_entry_point_twice(gpu, n):
    s = State.from_arrays(*rng.normal_state(n, 40 + n))
    targets = list(range(n))
    for obs in ("x", "y", "z"):
        want = np.array(core.xyz_expectation_value(obs, s, targets))
        for _ in range(2):  # the static scratch keeps the previous call's contents
            np.testing.assert_allclose(_noalloc(s, obs, targets), want, atol=1e-13, rtol=0)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    s = State(3)
    with pytest.raises(ValueError, match="SPZ_NOALLOC_MAX_TARGETS"):
        _noalloc(s, "z", [0] * 65)
    with pytest.raises(ValueError):
        _noalloc(s, "q", [0])
