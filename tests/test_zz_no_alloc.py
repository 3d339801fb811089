"""The allocation-free expectation entry point, for callers that cannot call
cudaMalloc (code inside another framework's memory pool or arena, or under a
fixed memory budget).

Called through the C ABI on raw device arrays, twice in a row (the static
scratch keeps the previous call's contents), and compared with the oracle's
xyz_expectation_value and with spz_xyz_expectation_value on the same state, at
the tolerance the other expectation tests use (1e-13).  Also covers a
non-default stream, a device-memory `out` and an empty target list.  Collected
last (test_zz_*) so that a run that stops at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import core, rng
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


def _noalloc(s: State, obs: str, targets, out=None, stream=None) -> np.ndarray:
    dre, dim = s.device_arrays()
    t = np.ascontiguousarray(np.array(targets, dtype=np.uint32))
    host = out is None
    if host:
        out = np.full(max(1, len(t)), np.nan)
    optr = nat.ptr(out) if host else ctypes.c_void_p(out.data_ptr())
    nat.check(nat.lib().spz_xyz_expectation_value_noalloc(
        ctypes.c_void_p(dre), ctypes.c_void_p(dim), s.n, obs.encode(), nat.ptr(t), len(t), optr,
        None if stream is None else ctypes.c_void_p(stream)))
    return out[:len(t)] if host else out


@pytest.mark.parametrize("n", [1, 9, 18])
def test_noalloc_matches_oracle_and_existing_entry_point_twice(gpu, n):
    re, im = rng.normal_state(n, 40 + n)
    s = State.from_arrays(re, im)
    targets = list(range(n))
    for obs in ("x", "y", "z"):
        want = np.array(oracle.xyz_expectation_value(obs, re.copy(), im.copy(), targets))
        lib_value = np.array(core.xyz_expectation_value(obs, s, targets))
        for _ in range(2):  # the static scratch keeps the previous call's contents
            got = _noalloc(s, obs, targets)
            np.testing.assert_allclose(got, want, atol=1e-13, rtol=0)
            np.testing.assert_allclose(got, lib_value, atol=1e-13, rtol=0)


def test_noalloc_on_a_side_stream_into_device_memory(gpu):
    import torch

    n = 14
    re, im = rng.normal_state(n, 7)
    s = State.from_arrays(re, im)
    targets = [0, 3, 13, 5]
    want = np.array(oracle.xyz_expectation_value("y", re.copy(), im.copy(), targets))
    side = torch.cuda.Stream()
    out = torch.full((len(targets),), float("nan"), dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        _noalloc(s, "y", targets, out=out, stream=side.cuda_stream)
        np.testing.assert_allclose(out.cpu().numpy(), want, atol=1e-13, rtol=0)


def test_noalloc_empty_target_list_is_ok(gpu):
    s = State(3)
    assert _noalloc(s, "x", []).size == 0


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    s = State(3)
    with pytest.raises(ValueError, match="SPZ_NOALLOC_MAX_TARGETS"):
        _noalloc(s, "z", [0] * 65)
    with pytest.raises(ValueError):
        _noalloc(s, "q", [0])
