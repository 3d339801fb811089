"""Host-side checks that need no GPU: the C-ABI library loads and exports every
declared entry point, struct layouts match, the RNG streams agree bit for bit
with the oracle, and the fusion planner's decisions."""
import math
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import circuit, rng
from spinoza_gb300.circuit import QuantumCircuit, QuantumRegister
from spinoza_gb300.gates import Gate

HEADER = Path(__file__).resolve().parent.parent / "include" / "spinoza_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(spz_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol(native):
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(native, name), name
    assert {s[0] for s in nat.SIGNATURES} == set(names)


def test_version(native):
    assert native.spz_version().decode().startswith("spinoza_gb300")


def test_struct_layouts():
    import ctypes

    assert ctypes.sizeof(nat.spz_gate) == 40
    assert ctypes.sizeof(nat.spz_op) == 64
    assert ctypes.sizeof(nat.spz_pauli_term) == 24
    assert ctypes.sizeof(nat.spz_exec_stats) == 80


def test_rng_stream_matches_oracle():
    u = rng.uniforms(1234, 64, start=10)
    for i in range(64):
        assert u[i] == oracle.stream_uniform(1234, 10 + i)


def test_uniform_state_matches_oracle():
    re, im = rng.uniform_state(10, 77)
    ore, oim = oracle.uniform_state(10, 77)
    assert np.array_equal(re, ore) and np.array_equal(im, oim)


def test_uniform_amplitudes_regenerate_any_index():
    re, im = rng.uniform_state(12, 31)
    idx = np.array([0, 1, 7, 4095, 2048, 1234, 7], dtype=np.uint64)
    gre, gim = rng.uniform_amplitudes(31, idx)
    assert np.array_equal(gre, re[idx.astype(np.int64)]) and np.array_equal(gim, im[idx.astype(np.int64)])
    # an index far beyond any state held on the host (bit 40 set)
    big = np.array([(1 << 40) + 5], dtype=np.uint64)
    bre, _ = rng.uniform_amplitudes(31, big)
    assert bre[0] == 2.0 * oracle.stream_uniform(31, 2 * ((1 << 40) + 5)) - 1.0


def test_normal_state_is_normalised():
    re, im = rng.normal_state(12, 1)
    assert abs(np.sum(re * re + im * im) - 1.0) < 1e-12


# ------------------------------------------------------------------- planner
def qft_ops(n):
    qc = QuantumCircuit.__new__(QuantumCircuit)
    qc.transformations = []
    for j in range(n - 1, -1, -1):
        qc.h(j)
        for k in range(j - 1, -1, -1):
            qc.cp(math.pi / 2 ** (j - k), j, k)
    for i in range(n // 2):
        qc.swap(i, n - 1 - i)
    return circuit._ops_array(qc.transformations, lambda: 0.0)


def brickwork_ops(n, layers, seed=2):
    qc = QuantumCircuit.__new__(QuantumCircuit)
    qc.transformations = []
    ang = rng.uniforms(seed, 3 * n * layers) * 2 * math.pi
    k = 0
    for _ in range(layers):
        for q in range(n):
            qc.u(ang[k], ang[k + 1], ang[k + 2], q)
            k += 3
        for q in range(0, n - 1, 2):
            qc.cx(q, q + 1)
        for q in range(1, n - 1, 2):
            qc.cx(q, q + 1)
    return circuit._ops_array(qc.transformations, lambda: 0.0)


def test_planner_fuses_qft(native):
    ops = qft_ops(20)
    st = circuit.plan_stats(20, ops)
    unf = circuit.plan_stats(20, ops, fused=False)
    assert st["gates"] == unf["gates"] == 20 + 190 + 10
    assert unf["passes"] == 220
    assert st["passes"] <= 12, st
    assert st["bytes_moved"] < unf["bytes_moved"]


def test_planner_fuses_brickwork(native):
    n, layers = 30, 2
    ops = brickwork_ops(n, layers)
    st = circuit.plan_stats(n, ops)
    assert st["gates"] == layers * (n + n - 1)
    assert st["passes"] < st["gates"] / 4, st
    # the algorithmic bytes are the unfused minimum
    assert st["algorithmic_bytes"] == layers * (n * 32 + (n - 1) * 16) << n


def test_planner_marks_shuffle_runs(native):
    """SPZ_EXEC_SHUFFLE: runs of at least two consecutive ops on the five lowest
    tile qubits are marked (fast brickwork: the lazy rotations and CX there);
    none without the flag, none in tiles of fewer than 2^7 amplitudes."""
    n = 30
    ops = brickwork_ops(n, 4)
    counts = {}
    for flags in (nat.EXEC_FAST, nat.EXEC_FAST | nat.EXEC_SHUFFLE, nat.EXEC_SHUFFLE):
        st = nat.spz_exec_stats()
        nat.check(nat.lib().spz_plan_stats(n, nat.ptr(ops), len(ops), flags, nat.byref(st)))
        counts[flags] = (st.shuffle_gates, st.passes)
    assert counts[nat.EXEC_FAST][0] == 0
    assert counts[nat.EXEC_FAST | nat.EXEC_SHUFFLE][0] > 0
    assert counts[nat.EXEC_FAST | nat.EXEC_SHUFFLE][1] == counts[nat.EXEC_FAST][1]  # same passes
    # exact U is not run-eligible (its pair arithmetic does not split evenly over two lanes); CX is
    assert counts[nat.EXEC_SHUFFLE][0] > 0
    small = brickwork_ops(6, 4)
    st = nat.spz_exec_stats()
    nat.check(nat.lib().spz_plan_stats(6, nat.ptr(small), len(small), nat.EXEC_FAST | nat.EXEC_SHUFFLE,
                                       nat.byref(st)))
    assert st.shuffle_gates == 0


def test_plan_passes_full_tiles_and_fused_ops(native):
    """spz_plan_passes: one entry per counted pass; every tile pass of the
    30-qubit brickwork holds 2^10 amplitudes; a circuit on five qubits gets a
    single tile pass padded to 10 local qubits; in fast mode the fused lazy
    pairs leave fewer device ops than lowered ops."""
    n = 30
    ops = brickwork_ops(n, 20)
    for fast in (False, True):
        masks, pops = circuit.plan_passes(n, ops, fast=fast)
        st = circuit.plan_stats(n, ops, fast=fast)
        assert len(masks) == st["passes"] and (masks != 0).sum() == st["tile_passes"]
        assert all(bin(int(m)).count("1") == 10 and int(m) & 7 == 7 for m in masks if m)
    _, exact_ops = circuit.plan_passes(n, ops)
    _, fast_ops = circuit.plan_passes(n, ops, fast=True)
    assert exact_ops.sum() == len(ops)
    assert fast_ops.sum() < len(ops)  # 600 lazy rotations, most of them in fused pairs
    # the trailing fast passes keep three consecutive high qubits non-local (the
    # host-array execute downloads in their slab geometry)
    masks, _ = circuit.plan_passes(n, ops, fast=True)
    tail = int(masks[-1]) | int(masks[-2])
    assert any(((tail >> q) & 7) == 0 for q in range(15, 25))
    narrow = np.zeros(8, dtype=nat.OP_DTYPE)
    for i in range(8):
        narrow[i] = ((nat.H if i % 2 else nat.RY, 0, 0, 0, (0.3 * i, 0, 0)), i % 5, nat.CONTROLS_NONE, 0, 0)
    masks, pops = circuit.plan_passes(n, narrow)
    assert len(masks) == 1 and bin(int(masks[0])).count("1") == 10 and int(masks[0]) & 31 == 31
    assert pops[0] == 8
    # measurements: two passes each, no tile
    m = np.zeros(3, dtype=nat.OP_DTYPE)
    m[0] = ((nat.H, 0, 0, 0, (0, 0, 0)), 0, 0, 0, 0)
    m[1] = ((nat.M, 0, 0, 0, (0.5, 0, 0)), 1, 0, 0, 0)
    m[2] = ((nat.H, 0, 0, 0, (0, 0, 0)), 0, 0, 0, 0)
    masks, pops = circuit.plan_passes(4, m)
    assert list(pops) == [1, 0, 0, 1] and not masks.any()


def random_ops(n, ngates, seed):
    """Every gate kind with none / single / ones / mixed controls."""
    r = np.random.default_rng(seed)
    ops = np.zeros(ngates, dtype=nat.OP_DTYPE)
    kinds = [nat.H, nat.X, nat.Y, nat.Z, nat.P, nat.RX, nat.RY, nat.RZ, nat.U, nat.SWAP]
    for i in range(ngates):
        k = int(r.choice(kinds))
        q = r.permutation(n)
        nc = int(r.integers(0, 4))
        ctrls = [int(c) for c in q[2:2 + nc]]
        ck = [nat.CONTROLS_NONE, nat.CONTROLS_SINGLE, nat.CONTROLS_ONES, nat.CONTROLS_ONES][nc]
        zeros = 0
        if nc >= 2 and r.random() < 0.5:
            ck, zeros = nat.CONTROLS_MIXED, 1 << ctrls[0]
        ops[i] = ((k, int(q[0]), int(q[1]), 0, r.uniform(-math.pi, math.pi, 3)), int(q[0]), ck,
                  sum(1 << c for c in ctrls), zeros)
    return ops


@pytest.mark.parametrize("n", [5, 9, 13, 15])
@pytest.mark.parametrize("seed", range(4))
def test_planner_reordering_is_bit_exact(native, n, seed):
    """Replaying the fused schedule gate by gate through the oracle gives the
    sequential result bit for bit: the planner only swaps exactly-commuting gates."""
    ops = random_ops(n, 200, 1000 * n + seed)
    order, passes = circuit.plan_schedule(n, ops)
    assert sorted(order.tolist()) == list(range(len(ops)))
    assert np.all(np.diff(passes.astype(np.int64)) >= 0)
    init = rng.uniform_state(n, seed)
    a = [x.copy() for x in init]
    oracle.execute(ops, *a)
    b = [x.copy() for x in init]
    for i in order:
        oracle.execute(ops[i:i + 1], *b)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_planner_schedule_brickwork_and_qft_bit_exact(native):
    for n, ops in [(14, brickwork_ops(14, 3)), (14, qft_ops(14))]:
        order, _ = circuit.plan_schedule(n, ops)
        init = rng.uniform_state(n, 1)
        a = [x.copy() for x in init]
        oracle.execute(ops, *a)
        b = [x.copy() for x in init]
        for i in order:
            oracle.execute(ops[i:i + 1], *b)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_fast_lowering_cuts_fp64_instructions(native):
    """Fast mode: U as P RY P with lazy scaling and phases pushed through the CX
    ladders needs ~8 instead of 14 FP64 instructions per pair and gate."""
    ops = brickwork_ops(30, 20)
    exact = circuit.plan_stats(30, ops)
    fast = circuit.plan_stats(30, ops, fast=True)
    assert exact["fp64_ops"] == 600 * 14 * (1 << 29)
    assert fast["fp64_ops"] < 0.6 * exact["fp64_ops"]
    assert fast["gates"] == exact["gates"] and fast["algorithmic_bytes"] == exact["algorithmic_bytes"]
    q = circuit.plan_stats(20, qft_ops(20), fast=True)
    assert q["fp64_ops"] < circuit.plan_stats(20, qft_ops(20))["fp64_ops"]


def test_fast_pairs_fuse_lazy_rotations(native):
    """Fast mode fuses two lazy rotations on different tile qubits into one op
    over blocks of four amplitudes: 28 instead of 32 FP64 instructions per
    block, 2^n fewer per fused pair.  SPZ_FAST_PAIRS=0 (read once per process)
    turns it off; the planned passes are the same either way."""
    import subprocess
    import sys

    code = ("import json, sys; sys.path.insert(0, 'tests'); from test_host import brickwork_ops; "
            "from spinoza_gb300 import circuit; print(json.dumps(circuit.plan_stats(30, brickwork_ops(30, 20), "
            "fast=True)))")
    root = Path(__file__).resolve().parent.parent
    env = dict(__import__("os").environ, SPZ_FAST_PAIRS="0")
    res = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    import json

    off = json.loads(res.stdout.strip().splitlines()[-1])
    on = circuit.plan_stats(30, brickwork_ops(30, 20), fast=True)
    assert off["fp64_ops"] >= 600 * 8 * (1 << 29)  # unfused: 8 per pair and U, plus the final phase op
    saved = off["fp64_ops"] - on["fp64_ops"]
    assert saved > 0 and saved % (1 << 30) == 0
    assert saved // (1 << 30) >= 200  # most of the 300 possible pairs of U gates per 20 layers
    assert on["passes"] == off["passes"] and on["gates"] == off["gates"]


def test_planner_measurement_is_a_barrier(native):
    ops = np.zeros(3, dtype=nat.OP_DTYPE)
    ops[0] = ((nat.H, 0, 0, 0, (0, 0, 0)), 0, 0, 0, 0)
    ops[1] = ((nat.M, 0, 0, 0, (0.5, 0, 0)), 1, 0, 0, 0)
    ops[2] = ((nat.H, 0, 0, 0, (0, 0, 0)), 0, 0, 0, 0)
    st = circuit.plan_stats(4, ops)
    assert st["gates"] == 2 and st["passes"] == 1 + 2 + 1


def test_invalid_ops_are_rejected_on_the_host(native):
    ops = np.zeros(1, dtype=nat.OP_DTYPE)
    ops[0] = ((nat.H, 0, 0, 0, (0, 0, 0)), 7, 0, 0, 0)  # target 7 on 4 qubits
    with pytest.raises(ValueError):
        circuit.plan_stats(4, ops)
    ops[0] = ((nat.X, 0, 0, 0, (0, 0, 0)), 1, nat.CONTROLS_SINGLE, 1 << 1, 0)  # control == target
    with pytest.raises(ValueError):
        circuit.plan_stats(4, ops)
    ops[0] = ((nat.UNITARY, 0, 0, 0, (0, 0, 0)), 0, 0, 0, 0)
    with pytest.raises(NotImplementedError):
        circuit.plan_stats(4, ops)


def test_circuit_builders_mirror_reference(native):
    """circuit.rs: register shifts, Controls::from, new_with_control, inverse."""
    a, b = QuantumRegister(2), QuantumRegister(3)
    qc = QuantumCircuit.__new__(QuantumCircuit)
    qc.transformations = []
    QuantumCircuit.__init__  # registers are shifted by the constructor:
    bits = 0
    for r in (a, b):
        r.update_shift(bits)
        bits += len(r)
    assert a.qubits == [0, 1] and b.qubits == [2, 3, 4] and b.get_shift() == 2
    from spinoza_gb300.circuit import Controls

    c = Controls.single(0).new_with_control(3, 1)
    assert c.kind == Controls.ONES and c.controls == [1, 3]
    m = Controls.mixed([0], {0}).new_with_control(2, 1)
    assert m.kind == Controls.MIXED and m.controls == [1, 2] and m.zeros == {1}
    qc.h(0)
    qc.p(math.pi / 4, 1)
    qc.inverse()
    assert qc.transformations[0].gate == Gate.P(-math.pi / 4) and qc.transformations[1].gate == Gate.H


# ------------------------------------------------------- benchmark reference arm
def test_bench_arms_build_the_same_workload(native):
    """The reference arm builds its ops and byte count from the oracle's numpy
    restatements; they must equal the product-side ones bit for bit."""
    import bench

    a = bench.brickwork_ops(12, 3, source="product")
    b = bench.brickwork_ops(12, 3, source="oracle")
    assert a.dtype.itemsize == b.dtype.itemsize == 64
    assert a.tobytes() == b.tobytes()
    assert oracle.algorithmic_bytes(b, 12) == bench.algorithmic_bytes(a, 12)
    assert bench.workload_config(30, 20)["gates"] == len(bench.brickwork_ops(30, 20, source="oracle"))


def test_oracle_uniforms_match_the_c_stream():
    u = oracle.uniforms(99, 16, start=5)
    assert all(u[i] == oracle.stream_uniform(99, 5 + i) for i in range(16))


def test_reference_arm_does_not_load_the_product_library():
    """`bench.py --impl reference` must run the oracle only: neither the
    spinoza_gb300 package nor its shared library may be loaded."""
    import json
    import subprocess
    import sys

    root = Path(__file__).resolve().parent.parent
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--qubits', '12', '--layers', '4', "
            "'--steps', '2', '--warmup', '1']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'pkg': [m for m in sys.modules if m.startswith('spinoza_gb300')], "
            "'so': 'libspinoza_gb300' in maps}))")
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"] == __import__("bench").workload_config(12, 4)
    assert probe == {"pkg": [], "so": False}


def test_ctypes_struct_sizes_match_the_c_header(tmp_path):
    """Compile the header with gcc and compare sizeof of every struct with the
    ctypes mirrors the Python layer passes across the ABI."""
    import ctypes
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    names = {"spz_gate": nat.spz_gate, "spz_op": nat.spz_op, "spz_tracker": nat.spz_tracker,
             "spz_exec_stats": nat.spz_exec_stats, "spz_pauli_term": nat.spz_pauli_term,
             "spz_batch_instance": nat.spz_batch_instance, "spz_batch_config": nat.spz_batch_config,
             "spz_batch_stats": nat.spz_batch_stats}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "spinoza_gb300.h"\nint main(void) {\n' +
                   "".join(f'  printf("{k} %zu\\n", sizeof({k}));\n' for k in names) + "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run([gcc, "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {ln.split()[0]: int(ln.split()[1]) for ln in out.splitlines()}
    for k, ct in names.items():
        assert got[k] == ctypes.sizeof(ct), k
    assert nat.INSTANCE_DTYPE.itemsize == got["spz_batch_instance"]
