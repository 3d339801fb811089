"""TMA-staged tile passes (SPZ_EXEC_TMA, SPZ_EXEC_TMA_PREFETCH): each tile is
fetched by tile::gather4 tensor copies instead of thread loads; compute and
store are unchanged, so results must be bit-identical to the default staging
(exact and fast mode), and the exact mode to the oracle."""
import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import rng
from spinoza_gb300.core import State

from test_gpu_circuits import brickwork, qft_with_swaps, random_circuit

pytestmark = pytest.mark.gpu


def _run(n, ops, init, flags):
    s = State.from_arrays(*init)
    tr = nat.spz_tracker(0, 0)
    st = nat.spz_exec_stats()
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    nat.check(nat.lib().spz_circuit_execute(s.handle, nat.ptr(ops), len(ops), nat.byref(tr), flags, nat.byref(st)))
    return s.to_numpy(), st


@pytest.mark.parametrize("n", [5, 9, 12, 17, 20])
@pytest.mark.parametrize("staging", [nat.EXEC_TMA, nat.EXEC_TMA_PREFETCH])
def test_tma_staging_is_bit_identical(gpu, n, staging):
    init = rng.normal_state(n, 100 + n)
    for ops in (brickwork(n, 3), random_circuit(n, 300, n), qft_with_swaps(n)):
        for fast in (False, True):
            base = nat.EXEC_FAST if fast else nat.EXEC_DEFAULT
            (a_re, a_im), st = _run(n, ops, init, base)
            (b_re, b_im), st2 = _run(n, ops, init, base | staging)
            assert np.array_equal(a_re, b_re) and np.array_equal(a_im, b_im)
            assert st2.tile_passes == st.tile_passes
            if not fast:
                re, im = init[0].copy(), init[1].copy()
                oracle.execute(ops, re, im)
                assert np.array_equal(b_re, re) and np.array_equal(b_im, im)
