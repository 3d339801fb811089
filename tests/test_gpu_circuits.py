"""The fused circuit executor vs the oracle's sequential execute().

The planner only reorders gates where the swap is bit-exact, and each gate's
arithmetic inside a tile is the plain kernel's, so fused results are expected
to be bit-identical; the asserted bound is the 1e-12 parity bound plus an exact
check where the circuit allows it."""
import math

import numpy as np
import pytest

import oracle
from spinoza_gb300 import _native as nat
from spinoza_gb300 import circuit, rng
from spinoza_gb300.circuit import QuantumCircuit, QuantumRegister
from spinoza_gb300.core import State

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _run_gpu(n, ops, init, fused=True, tracker=(0, 0)):
    s = State.from_arrays(*init)
    qc = QuantumCircuit.from_state(s, fused=fused)
    qc.qubit_tracker.c.measured, qc.qubit_tracker.c.values = tracker
    qc.execute_ops(ops)
    return s.to_numpy(), (qc.qubit_tracker.c.measured, qc.qubit_tracker.c.values), qc.last_stats


def _run_oracle(ops, init, tracker=(0, 0)):
    re, im = init[0].copy(), init[1].copy()
    tr = oracle.execute(ops, re, im, *tracker)
    return (re, im), tr


def _builder():
    qc = QuantumCircuit.__new__(QuantumCircuit)
    qc.transformations = []
    qc._seed, qc._draw_index = 0, 0
    return qc


def qft_with_swaps(n):
    """QFT with swaps: for j = n-1..0: H(j), CP(pi/2^(j-k)) k < j; then SWAP(i, n-1-i)."""
    qc = _builder()
    for j in range(n - 1, -1, -1):
        qc.h(j)
        for k in range(j - 1, -1, -1):
            qc.cp(math.pi / 2 ** (j - k), j, k)
    for i in range(n // 2):
        qc.swap(i, n - 1 - i)
    return qc.ops()


def brickwork(n, layers, seed=2):
    """Brickwork: U(theta, phi, lambda) on every qubit, then CX even, CX odd."""
    qc = _builder()
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
    return qc.ops()


def random_circuit(n, ngates, seed):
    """Every gate kind, with none / single / ones / mixed controls."""
    r = np.random.default_rng(seed)
    ops = np.zeros(ngates, dtype=nat.OP_DTYPE)
    kinds = [nat.H, nat.X, nat.Y, nat.Z, nat.P, nat.RX, nat.RY, nat.RZ, nat.U, nat.SWAP]
    for i in range(ngates):
        k = int(r.choice(kinds))
        q = r.permutation(n)
        t, t2 = int(q[0]), int(q[1])
        nc = int(r.integers(0, 4))
        ctrls = [int(c) for c in q[2:2 + nc]]
        ck = [nat.CONTROLS_NONE, nat.CONTROLS_SINGLE, nat.CONTROLS_ONES, nat.CONTROLS_ONES][nc]
        zeros = 0
        if nc >= 2 and r.random() < 0.5:
            ck = nat.CONTROLS_MIXED
            zeros = 1 << ctrls[0]
        cm = sum(1 << c for c in ctrls)
        p = r.uniform(-math.pi, math.pi, 3)
        ops[i] = ((k, t, t2, 0, p), t, ck, cm, zeros)
    return ops


def _compare(a, b, exact=True):
    (gre, gim), (ore, oim) = a, b
    d = max(np.max(np.abs(gre - ore)), np.max(np.abs(gim - oim)))
    assert d <= TOL, d
    if exact:
        assert np.array_equal(gre, ore) and np.array_equal(gim, oim), d


def test_qft20_parity(gpu):
    """QFT with swaps on a seeded N(0,1) normalised 20-qubit state."""
    n = 20
    init = rng.normal_state(n, 1)
    ops = qft_with_swaps(n)
    g, _, st = _run_gpu(n, ops, init)
    o, _ = _run_oracle(ops, init)
    _compare(g, o)
    assert st.passes < 20 and st.gates == 220
    gu, _, stu = _run_gpu(n, ops, init, fused=False)
    _compare(gu, o)
    assert stu.passes == 220


@pytest.mark.parametrize("n,layers", [(12, 3), (17, 2)])
def test_brickwork_parity(gpu, n, layers):
    init = rng.uniform_state(n, 5)
    ops = brickwork(n, layers)
    g, _, st = _run_gpu(n, ops, init)
    o, _ = _run_oracle(ops, init)
    _compare(g, o)
    assert st.tile_passes >= 1


@pytest.mark.parametrize("n,seed", [(6, 1), (13, 2), (15, 3)])
def test_random_circuits_fused_equals_oracle(gpu, n, seed):
    init = rng.uniform_state(n, seed)
    ops = random_circuit(n, 300, seed)
    g, _, _ = _run_gpu(n, ops, init)
    o, _ = _run_oracle(ops, init)
    _compare(g, o)
    gu, _, _ = _run_gpu(n, ops, init, fused=False)
    _compare(gu, o)


def test_mid_circuit_measurement_and_classical_control(gpu):
    """circuit.rs:559-578: M records the outcome; a Single control on a measured
    qubit becomes a classical condition."""
    n = 8
    init = rng.normal_state(n, 3)
    qc = _builder()
    for q in range(n):
        qc.h(q)
    qc.measure(2)
    qc.cx(2, 5)      # classical: applies iff qubit 2 measured 1
    qc.crx(0.3, 2, 6)
    qc.ry(0.4, 2)
    qc.measure(7)
    qc.cx(7, 0)
    qc.measure(2)    # already measured: no-op
    ops = qc.ops()
    for u in (0.1, 0.9):
        ops["gate"]["p"][[n, n + 4], 0] = u  # the two fresh measurement draws
        g, gtr, _ = _run_gpu(n, ops, init)
        o, otr = _run_oracle(ops, init)
        assert gtr == otr
        # the collapse scale 1/sqrt(prob0) comes from a sum in a different order
        _compare(g, o, exact=False)


@pytest.mark.parametrize("mode", ["fused", "fast", "unfused"])
def test_measurements_on_device_with_conditioned_gates(gpu, mode):
    """Measurements inside the fused executor stay on the device: the outcome
    conditions later gates there (a Single control on a measured qubit,
    circuit.rs:570-578) and reaches the tracker at the end; the unfused mode
    measures on the host.  Every mode matches the oracle."""
    n = 11
    init = rng.normal_state(n, 21)
    qc = _builder()
    for q in range(n):
        qc.ry(0.3 + 0.1 * q, q)
    qc.measure(4)
    qc.cx(4, 9)        # conditioned X
    qc.crz(0.7, 4, 2)  # conditioned diagonal
    qc.ch(4, 0)        # conditioned pair gate on a low qubit
    for q in range(n - 1):
        qc.cx(q, q + 1)
    qc.measure(9)
    qc.cry(0.4, 9, 10)
    qc.u(0.1, 0.2, 0.3, 9)
    qc.measure(4)      # already measured: no-op
    ops = qc.ops()
    m = [i for i in range(len(ops)) if ops["gate"]["kind"][i] == nat.M]
    for draws in ((0.05, 0.95), (0.95, 0.05), (0.5, 0.5)):
        ops["gate"]["p"][m[0], 0], ops["gate"]["p"][m[1], 0] = draws
        s = State.from_arrays(*init)
        q2 = QuantumCircuit.from_state(s, fused=mode != "unfused", fast=mode == "fast")
        q2.execute_ops(ops)
        g = s.to_numpy()
        o, otr = _run_oracle(ops, init)
        assert (q2.qubit_tracker.c.measured, q2.qubit_tracker.c.values) == otr
        _compare(g, o, exact=False)


def test_reference_circuit_tests(gpu):
    """circuit.rs:725-822, 962-989, 1030-1061, 1234-1250 restated on the device."""
    # append: H on two one-qubit registers -> 0.5 everywhere
    qr0, qr1 = QuantumRegister(1), QuantumRegister(1)
    qc = QuantumCircuit(qr0, qr1)
    one = QuantumCircuit(QuantumRegister(1))
    one.h(0)
    qc.append(one, qr0)
    qc.append(one, qr1)
    qc.execute()
    re, im = qc.state.to_numpy()
    np.testing.assert_allclose(re, 0.5, atol=1e-4)
    np.testing.assert_allclose(im, 0.0, atol=1e-4)
    # inverse: [H(0), P(pi/4, 1)].inverse() == [P(-pi/4, 1), H(0)]
    a = QuantumCircuit(QuantumRegister(2))
    a.h(0)
    a.p(math.pi / 4, 1)
    a.inverse()
    a.execute()
    b = QuantumCircuit(QuantumRegister(2))
    b.p(-math.pi / 4, 1)
    b.h(0)
    b.execute()
    assert all(np.array_equal(x, y) for x, y in zip(a.state.to_numpy(), b.state.to_numpy()))
    # all_gates_as_transformations (N = 17): circuit == functional API
    from spinoza_gb300 import gates as G
    from spinoza_gb300.gates import Gate

    N, PI = 17, math.pi
    q = QuantumCircuit(QuantumRegister(N))
    for t in range(N):
        q.h(t)
    q.x(0); q.y(1); q.z(2); q.p(PI, 3); q.cp(PI, 3, 4); q.rx(PI, 5); q.ry(PI, 6); q.rz(PI, 7)
    q.u(PI, PI, PI, 8); q.cy(9, 10); q.crx(PI, 11, 12); q.cry(PI, 13, 14)
    q.execute()
    s = State(N)
    for t in range(N):
        G.apply(Gate.H, s, t)
    G.apply(Gate.X, s, 0); G.apply(Gate.Y, s, 1); G.apply(Gate.Z, s, 2); G.apply(Gate.P(PI), s, 3)
    G.c_apply(Gate.P(PI), s, 3, 4); G.apply(Gate.RX(PI), s, 5); G.apply(Gate.RY(PI), s, 6)
    G.apply(Gate.RZ(PI), s, 7); G.apply(Gate.U(PI, PI, PI), s, 8); G.c_apply(Gate.Y, s, 9, 10)
    G.c_apply(Gate.RX(PI), s, 11, 12); G.c_apply(Gate.RY(PI), s, 13, 14)
    assert all(np.array_equal(x, y) for x, y in zip(q.state.to_numpy(), s.to_numpy()))


def test_swap_all_qubits_circuit_equals_three_cx(gpu):
    """circuit.rs:891-929."""
    n = 9
    init = rng.uniform_state(n, 4)
    qc = _builder()
    for i in range(n >> 1):
        qc.swap(i, n - 1 - i)
    a, _, _ = _run_gpu(n, qc.ops(), init)
    qc = _builder()
    for i in range(n >> 1):
        j = n - 1 - i
        qc.cx(i, j); qc.cx(j, i); qc.cx(i, j)
    b, _, _ = _run_gpu(n, qc.ops(), init)
    _compare(a, b)


def test_iqft_device_entry_point(gpu):
    from spinoza_gb300.core import iqft

    n = 11
    init = rng.normal_state(n, 6)
    s = State.from_arrays(*init)
    t = list(range(n - 1, -1, -1))
    iqft(s, t)
    re, im = init[0].copy(), init[1].copy()
    oracle.iqft(re, im, t)
    _compare(s.to_numpy(), (re, im))


def test_plan_stats_agree_with_execution(gpu):
    n = 14
    ops = brickwork(n, 3)
    planned = circuit.plan_stats(n, ops)
    _, _, st = _run_gpu(n, ops, rng.uniform_state(n, 1))
    assert planned["passes"] == st.passes and planned["bytes_moved"] == st.bytes_moved


# ---------------------------------------------------------------- host state
def _host_pair(init, pinned):
    """Copies of init as host arrays: page-locked (torch pinned) or pageable."""
    if not pinned:
        return init[0].copy(), init[1].copy()
    import torch

    re = torch.empty(init[0].size, dtype=torch.float64, pin_memory=True).numpy()
    im = torch.empty(init[1].size, dtype=torch.float64, pin_memory=True).numpy()
    re[:] = init[0]
    im[:] = init[1]
    return re, im


def _last_gates_on_top(n):
    """A last pass with the top qubits local: its slabs are strided runs."""
    qc = _builder()
    for q in range(n):
        qc.ry(0.2 * (q + 1), q)
    for q in range(n - 1):
        qc.cx(q, q + 1)
    qc.h(n - 1)
    qc.rx(0.3, n - 2)
    qc.cx(n - 2, n - 1)
    return qc.ops()


def _first_gate_on_top(n):
    """A first pass whose local qubits include the top qubit (no slabbed upload)."""
    qc = _builder()
    qc.h(n - 1)
    qc.rx(0.7, n - 1)
    qc.cx(n - 1, 0)
    for q in range(n):
        qc.ry(0.1 * (q + 1), q)
    return qc.ops()


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("case", ["brickwork", "random", "top_first", "top_last", "empty", "unfused"])
def test_execute_host_equals_device_execute(gpu, pinned, case):
    """spz_circuit_execute_host (the reference's host State, mutated in place)
    gives exactly what upload + spz_circuit_execute + download gives."""
    n = 14
    init = rng.normal_state(n, 11)
    fused = case != "unfused"
    ops = {"brickwork": lambda: brickwork(n, 3), "random": lambda: random_circuit(n, 120, 5),
           "top_first": lambda: _first_gate_on_top(n), "top_last": lambda: _last_gates_on_top(n),
           "empty": lambda: np.zeros(0, dtype=nat.OP_DTYPE),
           "unfused": lambda: brickwork(n, 2)}[case]()
    want, _, _ = _run_gpu(n, ops, init, fused=fused)
    re, im = _host_pair(init, pinned)
    st = circuit.execute_host(ops, re, im, fused=fused)
    assert np.array_equal(re, want[0]) and np.array_equal(im, want[1])
    assert st.gates == (len(ops) if case != "empty" else 0)


def _below_top(n, layers):
    """Gates on qubits 0 .. n-4 only: every pass keeps the top three qubits
    non-local, so the whole run goes slab by slab (upload, passes, download)."""
    qc = _builder()
    ang = rng.uniforms(17, 3 * n * layers) * 2 * math.pi
    for layer in range(layers):
        for q in range(n - 3):
            qc.u(ang[3 * (layer * n + q)], ang[3 * (layer * n + q) + 1], ang[3 * (layer * n + q) + 2], q)
        for q in range(n - 4):
            qc.cx(q, q + 1)
        qc.cp(0.4, n - 1, 2)  # a control on a slab qubit: a per-tile predicate
    return qc.ops()


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
@pytest.mark.parametrize("case", ["prefix", "all_slabbed"])
def test_execute_host_slab_major_passes(gpu, case, fast):
    """Leading passes that keep the upload's slab qubits non-local run slab by
    slab after each slab's upload (and, when every pass does, each slab's
    download follows): results equal the device execute bit for bit."""
    n = 20 if case == "prefix" else 16
    ops = brickwork(n, 2) if case == "prefix" else _below_top(n, 3)
    init = rng.normal_state(n, 13)
    s = State.from_arrays(*init)
    qc = QuantumCircuit.from_state(s, fast=fast)
    qc.execute_ops(ops)
    want = s.to_numpy()
    for inplace in (True, False):
        re, im = _host_pair(init, True)
        out = None if inplace else _host_pair((np.zeros_like(init[0]), np.zeros_like(init[1])), True)
        st = circuit.execute_host(ops, re, im, out, fast=fast)
        got = (re, im) if inplace else out
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        assert st.gates == len(ops) and st.tile_passes >= 2


def _gap_brickwork(n, layers, gap=(15, 16, 17)):
    """Brickwork over every qubit but those in `gap`, which no gate touches:
    the trailing passes keep the gap non-local while the top qubits are local,
    so the download runs as a slab-major suffix in the gap's geometry (rows of
    2^15 amplitudes: 2^(n-18) of them per slab, as separate copies up to 64 and
    as one strided copy beyond)."""
    qs = [q for q in range(n) if q not in gap]
    qc = _builder()
    ang = rng.uniforms(23, 3 * len(qs) * layers) * 2 * math.pi
    k = 0
    for _ in range(layers):
        for q in qs:
            qc.u(ang[k], ang[k + 1], ang[k + 2], q)
            k += 3
        for a, b in zip(qs[0::2], qs[1::2]):
            qc.cx(a, b)
        for a, b in zip(qs[1::2], qs[2::2]):
            qc.cx(a, b)
    return qc.ops()


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
@pytest.mark.parametrize("case", ["gap20", "gap25", "brickwork"])
def test_execute_host_slab_major_suffix(gpu, case, fast):
    """Trailing passes that keep three consecutive qubits non-local run slab by
    slab with each slab's download right after its last pass: results equal
    the device execute bit for bit, in place and into separate arrays."""
    n = 25 if case == "gap25" else 20
    ops = _gap_brickwork(n, 3) if case != "brickwork" else brickwork(n, 2)
    init = rng.normal_state(n, 29)
    s = State.from_arrays(*init)
    QuantumCircuit.from_state(s, fast=fast).execute_ops(ops)
    want = s.to_numpy()
    for inplace in (True, False):
        re, im = _host_pair(init, True)
        out = None if inplace else _host_pair((np.zeros_like(init[0]), np.zeros_like(init[1])), True)
        st = circuit.execute_host(ops, re, im, out, fast=fast)
        got = (re, im) if inplace else out
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        if case != "brickwork":
            assert st.io_slab_passes >= 4, st.io_slab_passes


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
def test_execute_host_with_measurements(gpu, fast):
    """Measurements split the run into segments: the upload feeds the first,
    the download follows the last, and the tracker comes back."""
    n = 13
    init = rng.normal_state(n, 12)
    qc = _builder()
    qc.measure(n - 1)       # first segment empty: plain upload before the measurement
    for q in range(n):
        qc.u(0.3 + q, 0.2, 0.1 * q, q)
    qc.measure(3)
    qc.cx(3, 7)
    for q in range(n - 1):
        qc.cx(q, q + 1)
    ops = qc.ops()
    ops["gate"]["p"][0, 0] = 0.25
    ops["gate"]["p"][n + 1, 0] = 0.75
    s = State.from_arrays(*init)
    ref = QuantumCircuit.from_state(s, fast=fast)
    ref.execute_ops(ops)
    want = s.to_numpy()
    re, im = _host_pair(init, True)
    tr = circuit.QubitTracker()
    circuit.execute_host(ops, re, im, tracker=tr, fast=fast)
    assert (tr.c.measured, tr.c.values) == (ref.qubit_tracker.c.measured, ref.qubit_tracker.c.values)
    assert np.array_equal(re, want[0]) and np.array_equal(im, want[1])


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_execute_host_tiny_states(gpu, n):
    """States smaller than the 8 upload slabs are copied whole."""
    init = rng.normal_state(n, 30 + n)
    ops = random_circuit(n, 20, n) if n >= 4 else brickwork(n, 2)
    want, _, _ = _run_gpu(n, ops, init)
    re, im = _host_pair(init, True)
    circuit.execute_host(ops, re, im)
    assert np.array_equal(re, want[0]) and np.array_equal(im, want[1])


def test_execute_host_separate_output(gpu):
    """Input arrays stay untouched when an output pair is given."""
    n = 15
    init = rng.normal_state(n, 14)
    ops = brickwork(n, 2)
    want, _, _ = _run_gpu(n, ops, init, fused=True)
    re, im = _host_pair(init, True)
    ore, oim = _host_pair((np.zeros_like(init[0]), np.zeros_like(init[1])), True)
    circuit.execute_host(ops, re, im, (ore, oim))
    assert np.array_equal(re, init[0]) and np.array_equal(im, init[1])
    assert np.array_equal(ore, want[0]) and np.array_equal(oim, want[1])


def test_execute_host_reuses_a_state_and_checks_sizes(gpu):
    n = 12
    s = State(n)
    init = rng.normal_state(n, 13)
    ops = brickwork(n, 2)
    for _ in range(2):
        re, im = _host_pair(init, True)
        circuit.execute_host(ops, re, im, state=s)
    want, _, _ = _run_gpu(n, ops, init)
    assert np.array_equal(re, want[0]) and np.array_equal(im, want[1])
    with pytest.raises(ValueError):
        circuit.execute_host(ops, np.zeros(1 << (n + 1)), np.zeros(1 << (n + 1)), state=s)


# ---------------------------------------------------------------- programs
@pytest.mark.parametrize("mode", ["fused", "fast", "unfused"])
def test_program_replays_equal_execute(gpu, mode):
    """A compiled program (planned once, replayed as a CUDA graph) gives what
    spz_circuit_execute gives, run after run, on one state or another."""
    import torch

    n = 13
    ops = random_circuit(n, 150, 7)
    init = rng.normal_state(n, 41)
    fused, fast = mode != "unfused", mode == "fast"
    prog = circuit.Program(n, ops, fused=fused, fast=fast)
    s = State.from_arrays(*init)
    want = State.from_arrays(*init)
    ref = QuantumCircuit.from_state(want, fused=fused, fast=fast)
    for _ in range(3):  # capture, then two replays
        prog.run(s)
        ref.execute_ops(ops)
        s.synchronize()
        a, b = s.to_numpy(), want.to_numpy()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    other = State.from_arrays(*init)  # a different state: captured again
    prog.run(other)
    other.synchronize()
    o = other.to_numpy()
    first, _, _ = _run_gpu(n, ops, init, fused=fused)
    if not fast:
        assert np.array_equal(o[0], first[0]) and np.array_equal(o[1], first[1])
    st = prog.stats()
    assert st["gates"] == len(ops) and st["passes"] >= 1
    prog.close()
    _ = torch


def test_program_on_torch_stream_and_rejects_measurements(gpu):
    import torch

    n = 12
    ops = brickwork(n, 3)
    re = torch.zeros(1 << n, dtype=torch.float64, device="cuda")
    im = torch.zeros(1 << n, dtype=torch.float64, device="cuda")
    re[0] = 1.0
    s = State.from_torch(re, im)
    s.set_stream(torch.cuda.current_stream())
    prog = circuit.Program(n, ops)
    prog.run(s)
    torch.cuda.synchronize()
    e0 = np.zeros(1 << n)
    e0[0] = 1.0
    want, _, _ = _run_gpu(n, ops, (e0, np.zeros(1 << n)))
    assert np.array_equal(re.cpu().numpy(), want[0]) and np.array_equal(im.cpu().numpy(), want[1])
    qc = _builder()
    qc.h(0)
    qc.measure(0)
    with pytest.raises(NotImplementedError):
        circuit.Program(n, qc.ops())
    with pytest.raises(ValueError):
        prog.run(State(n + 1))
