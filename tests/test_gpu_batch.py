"""The batched forward + adjoint launch vs the single-instance adjoint path and
the oracle.  Small tiles (tile_qubits=4..6) force the streaming (non-resident)
path, multiple Hamiltonian passes and split backward passes at small sizes."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import adjoint, batch
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu


def _single(inst):
    n, ops, pidx, theta, terms = inst
    return adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, terms)


def _instances():
    shapes = [(3, 1), (5, 2), (8, 3), (2, 2), (13, 2), (14, 1), (9, 4), (1, 2), (11, 1), (6, 3)]
    return [batch.hea_instance(n, d, 100 + i) for i, (n, d) in enumerate(shapes)]


@pytest.mark.parametrize("tile_qubits,threads", [(12, 512), (4, 64), (5, 128), (6, 1024)])
def test_batch_matches_single_instance_adjoint(gpu, tile_qubits, threads):
    insts = _instances()
    b = batch.Batch(insts, tile_qubits=tile_qubits, threads=threads)
    e, g = b.run()
    for i, inst in enumerate(insts):
        e1, g1 = _single(inst)
        assert abs(e[i] - e1) < 1e-12 * max(1.0, abs(e1)), (i, e[i], e1)
        np.testing.assert_allclose(b.split(g)[i], g1, atol=1e-11, rtol=0)
    info = b.info()
    assert info["instances"] == len(insts)
    if tile_qubits == 4:
        assert info["resident_instances"] < len(insts) and info["workspace_bytes"] > 0


@pytest.mark.parametrize("wide,tpi", [(8, 0), (8, 1), (7, 3), (1, 2)])
def test_batch_wide_instances_as_work_items_in_one_launch(gpu, wide, tpi):
    """Instances of at least `wide` qubits (and more than the tile's) are
    spread over CTAs as (pass, tile range) work items inside the persistent
    kernel, ordered by completion counters; the rest run one per CTA; replays
    with new angles stay right."""
    insts = _instances()
    b = batch.Batch(insts, tile_qubits=6, threads=128, wide_qubits=wide, tiles_per_item=tpi)
    info = b.info()
    assert info["wide_in_kernel"] == sum(1 for i in insts if i[0] >= max(wide, 7)) and info["wide_separate"] == 0
    assert info["work_items"] > len(insts) - info["wide_in_kernel"]
    for shift in (0.0, 0.21):
        theta = b.theta + shift
        e, g = b.run(theta)
        for i, (n, ops, pidx, _, terms) in enumerate(insts):
            th = b.split(theta)[i]
            e1, g1 = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, th), pidx, terms)
            assert abs(e[i] - e1) < 1e-12 * max(1.0, abs(e1)), (i, e[i], e1)
            np.testing.assert_allclose(b.split(g)[i], g1, atol=1e-11, rtol=0)
    e2, g2 = b.run(b.theta + 0.21)  # deterministic: fixed items, slots and fold order
    assert np.array_equal(e2, e) and np.array_equal(g2, g)


def test_batch_wide_item_wait_times_out_cleanly(gpu):
    """A dependency wait that never completes (a host-side injection makes the
    wide items of later passes wait for a count no item reaches) ends the
    launch with SPZ_ERR_TIMEOUT instead of hanging; the context stays usable."""
    import os

    from spinoza_gb300 import _native as nat

    insts = _instances()
    os.environ["SPZ_BATCH_TEST_STALL"] = "1"
    try:
        b = batch.Batch(insts, tile_qubits=6, threads=128, wide_qubits=8)
    finally:
        os.environ.pop("SPZ_BATCH_TEST_STALL", None)
    with pytest.raises(nat.SpzError) as info:
        b.run()
    assert info.value.code == nat.SPZ_ERR_TIMEOUT
    b.close()
    ok = batch.Batch(insts, tile_qubits=6, threads=128, wide_qubits=8)
    e, g = ok.run()
    e1, g1 = _single(insts[4])
    assert abs(e[4] - e1) < 1e-12 * max(1.0, abs(e1))
    np.testing.assert_allclose(ok.split(g)[4], g1, atol=1e-11, rtol=0)


@pytest.mark.parametrize("wide", [8, 1])
def test_batch_wide_instances_fast_run_across_the_gpu(gpu, wide):
    """With the fast adjoint, instances of at least `wide` qubits take the
    whole-GPU path (fused executor + fused fast adjoint sweep, results written
    on the device); the others stay in the persistent kernel."""
    insts = _instances()
    b = batch.Batch(insts, tile_qubits=6, threads=128, wide_qubits=wide, fast=True)
    assert b.info()["wide_separate"] == sum(1 for i in insts if i[0] >= max(wide, 7))
    for shift in (0.0, 0.21):
        theta = b.theta + shift
        e, g = b.run(theta)
        for i, (n, ops, pidx, _, terms) in enumerate(insts):
            th = b.split(theta)[i]
            e1, g1 = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, th), pidx, terms,
                                              fast=n >= max(wide, 7))
            assert abs(e[i] - e1) < 1e-12 * max(1.0, abs(e1)), (i, e[i], e1)
            np.testing.assert_allclose(b.split(g)[i], g1, atol=1e-11, rtol=0)


def test_batch_graph_replay_with_new_angles(gpu):
    insts = _instances()[:5]
    b = batch.Batch(insts, tile_qubits=5, threads=128)
    b.run()
    theta2 = b.theta + 0.37
    e, g = b.run(theta2)
    for i, (n, ops, pidx, _, terms) in enumerate(insts):
        th = b.split(theta2)[i]
        e1, g1 = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, th), pidx, terms)
        assert abs(e[i] - e1) < 1e-12 * max(1.0, abs(e1))
        np.testing.assert_allclose(b.split(g)[i], g1, atol=1e-11, rtol=0)


def test_batch_gradient_matches_oracle_parameter_shift(gpu):
    n, ops, pidx, theta, terms = batch.hea_instance(4, 2, 7)
    b = batch.Batch([(n, ops, pidx, theta, terms)], tile_qubits=4, threads=64)
    _, g = b.run()

    def energy(th):
        re, im = oracle.zero_state(n)
        oracle.execute(adjoint.set_params(ops, pidx, th), re, im)
        return oracle.pauli_expectation(re, im, terms)

    for j in range(len(pidx)):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += math.pi / 2
        tm[j] -= math.pi / 2
        assert abs(g[j] - 0.5 * (energy(tp) - energy(tm))) < 1e-9


def test_batch_rejects_bad_input(gpu):
    n, ops, pidx, theta, terms = batch.hea_instance(3, 1, 1)
    with pytest.raises(ValueError):
        batch.Batch([(n, ops, pidx, theta, terms)], tile_qubits=13)
    bad = pidx.copy()
    bad[0] = len(ops) + 5
    with pytest.raises(ValueError):
        batch.Batch([(n, ops, bad, theta, terms)])


def test_variational_workload_shapes():
    insts = batch.hea_workload(count=64)
    qs = [i[0] for i in insts]
    assert min(qs) >= 10 and max(qs) <= 22
    for n, ops, pidx, theta, terms in insts:
        assert len(pidx) % (2 * n) == 0 and 2 <= len(pidx) // (2 * n) <= 10
        assert len(terms) == 2 * n - 1


def test_autotuner_times_candidates_and_caches(gpu, tmp_path, monkeypatch):
    monkeypatch.setenv("SPZ_AUTOTUNE_CACHE", str(tmp_path))
    insts = _instances()
    cands = [(6, 64, 1), (6, 128, 4)]
    best = batch.autotune(insts, candidates=cands, sample=8)
    assert (best["tile_qubits"], best["threads"], best["tiles_per_item"]) in cands
    assert len(best["candidates"]) == 2 and best["sample"] <= len(insts)
    again = batch.autotune(insts, candidates=[(5, 64, 2)])  # answered from the cache
    assert again == best
    b = batch.Batch(insts, tile_qubits=best["tile_qubits"], threads=best["threads"],
                    tiles_per_item=best["tiles_per_item"])
    e, g = b.run()
    e1, g1 = _single(insts[5])
    assert abs(e[5] - e1) < 1e-12 * max(1.0, abs(e1))


def test_batch_library_defaults_with_wide_items(gpu):
    """The library's default launch shape (tile, threads, tiles per item) with
    the 13- and 14-qubit instances as wide work items."""
    insts = _instances()
    b = batch.Batch(insts, wide_qubits=12)
    assert b.info()["wide_in_kernel"] == 2
    e, g = b.run()
    for i in (4, 5, 2):
        e1, g1 = _single(insts[i])
        assert abs(e[i] - e1) < 1e-12 * max(1.0, abs(e1))
        np.testing.assert_allclose(b.split(g)[i], g1, atol=1e-11, rtol=0)
