"""Circuit builder and executor (spinoza/src/circuit.rs).

Builders append ``QuantumTransformation``s; ``execute`` drains them into one
flat op list and hands it to the device executor (spz_circuit_execute), which
fuses runs of gates into shared-memory tile passes.
"""
from __future__ import annotations

import math
from ctypes import byref
from typing import Iterable, List, Optional, Sequence, Set

import numpy as np

from . import _native as nat
from . import rng
from .core import State
from .gates import Gate, next_noise_draw

PI = math.pi


class QuantumRegister:
    """A list of qubit indices (circuit.rs:13-51)."""

    def __init__(self, size: int):
        if size <= 0:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "register size must be > 0 (circuit.rs:29)")
        self.qubits = list(range(size))

    def __getitem__(self, i: int) -> int:
        return self.qubits[i]

    def __len__(self) -> int:
        return len(self.qubits)

    def len(self) -> int:
        return len(self.qubits)

    def update_shift(self, shift: int) -> None:
        self.qubits = [q + shift for q in self.qubits]

    def get_shift(self) -> int:
        return self.qubits[0]


class Controls:
    """None / Single / Ones / Mixed (circuit.rs:53-109)."""

    NONE, SINGLE, ONES, MIXED = nat.CONTROLS_NONE, nat.CONTROLS_SINGLE, nat.CONTROLS_ONES, nat.CONTROLS_MIXED

    __slots__ = ("kind", "controls", "zeros")

    def __init__(self, kind: int, controls: Sequence[int] = (), zeros: Optional[Iterable[int]] = None):
        self.kind = kind
        self.controls = [int(c) for c in controls]
        self.zeros: Set[int] = set(int(z) for z in zeros) if zeros else set()

    @classmethod
    def none(cls) -> "Controls":
        return cls(cls.NONE)

    @classmethod
    def single(cls, c: int) -> "Controls":
        return cls(cls.SINGLE, [c])

    @classmethod
    def ones(cls, cs: Sequence[int]) -> "Controls":
        return cls(cls.ONES, cs)

    @classmethod
    def mixed(cls, controls: Sequence[int], zeros: Iterable[int]) -> "Controls":
        return cls(cls.MIXED, controls, zeros)

    @classmethod
    def from_(cls, controls: Sequence[int], zeros: Optional[Set[int]]) -> "Controls":  # circuit.rs:71-84
        if zeros:
            return cls.mixed(controls, zeros)
        if not controls:
            return cls.none()
        if len(controls) == 1:
            return cls.single(controls[0])
        return cls.ones(controls)

    def unpack(self):  # circuit.rs:86-93
        return list(self.controls), set(self.zeros)

    def new_with_control(self, control: int, shift: int) -> "Controls":  # circuit.rs:95-105
        controls, zeros = self.unpack()
        controls = [c + shift for c in controls] + [control]
        if not zeros:
            return Controls.from_(controls, None)
        return Controls.from_(controls, {z + shift for z in zeros})

    def __repr__(self) -> str:
        return f"Controls(kind={self.kind}, controls={self.controls}, zeros={sorted(self.zeros)})"


class QuantumTransformation:
    """gate + target + controls (circuit.rs:111-120)."""

    __slots__ = ("gate", "target", "controls")

    def __init__(self, gate: Gate, target: int, controls: Optional[Controls] = None):
        self.gate = gate
        self.target = int(target)
        self.controls = controls if controls is not None else Controls.none()


class QubitTracker:
    """Measured qubits and their values (circuit.rs:122-164)."""

    def __init__(self):
        self.c = nat.spz_tracker(0, 0)

    def is_qubit_measured(self, q: int) -> bool:
        return bool((self.c.measured >> q) & 1)

    def get_qubit_measured_val(self, q: int) -> Optional[int]:
        return int((self.c.values >> q) & 1) if self.is_qubit_measured(q) else None


def _ops_array(transformations: Sequence[QuantumTransformation], draws) -> np.ndarray:
    ops = np.zeros(len(transformations), dtype=nat.OP_DTYPE)
    for i, tr in enumerate(transformations):
        g = tr.gate
        if g.kind == nat.UNITARY:
            raise nat.Unsupported(nat.SPZ_ERR_UNSUPPORTED, "a dense Unitary is not an op; QuantumCircuit.execute "
                                                          "applies it between op runs")
        p = list(g.params)
        if g.kind == nat.M:
            p[0] = draws()
        elif g.kind == nat.BITFLIP and math.isnan(p[1]):
            p[1] = next_noise_draw()
        cmask = 0
        for c in tr.controls.controls:
            cmask |= 1 << c
        zmask = 0
        for z in tr.controls.zeros:
            zmask |= 1 << z
        ops[i] = ((g.kind, g.qubits[0], g.qubits[1], 0, p), tr.target, tr.controls.kind, cmask, zmask)
    return ops


class QuantumCircuit:
    """A circuit over one or more registers (circuit.rs:166-601).

    Keyword-only extensions: ``seed`` seeds the stream that resolves
    measurement outcomes inside execute(); ``fused=False`` runs one kernel per
    gate (the plain per-gate path)."""

    def __init__(self, *registers: QuantumRegister, seed: int = 0, fused: bool = True, fast: bool = False,
                 state: Optional[State] = None):
        bits = 0
        sizes = []
        for r in registers:  # circuit.rs:181-198
            r.update_shift(bits)
            sizes.append(len(r))
            bits += len(r)
        self.transformations: List[QuantumTransformation] = []
        self.quantum_registers_info = sizes
        self.num_qubits = state.n if state is not None else bits
        self._state = state  # allocated on the device on first use
        self.qubit_tracker = QubitTracker()
        self.fused = fused
        self.fast = fast
        self.last_stats = nat.spz_exec_stats()
        self._seed = int(seed)
        self._draw_index = 0

    @classmethod
    def from_state(cls, state: State, **kw) -> "QuantumCircuit":
        qc = cls(state=state, **kw)
        return qc

    @property
    def state(self) -> State:
        if self._state is None:
            self._state = State(self.num_qubits)
        return self._state

    @state.setter
    def state(self, s: State) -> None:
        self._state = s
        self.num_qubits = s.n

    def get_statevector(self) -> State:
        return self.state

    def inverse(self) -> None:  # circuit.rs:206-211
        self.transformations.reverse()
        for tr in self.transformations:
            tr.gate = tr.gate.inverse()

    def add(self, transformation: QuantumTransformation) -> None:
        self.transformations.append(transformation)

    def _add(self, gate: Gate, target: int, controls: Optional[Controls] = None) -> None:
        self.add(QuantumTransformation(gate, target, controls))

    # builders (circuit.rs:214-445)
    def measure(self, target: int) -> None: self._add(Gate.M, target)
    def swap(self, t0: int, t1: int) -> None: self._add(Gate.SWAP(t0, t1), 0)
    def x(self, target: int) -> None: self._add(Gate.X, target)
    def y(self, target: int) -> None: self._add(Gate.Y, target)
    def z(self, target: int) -> None: self._add(Gate.Z, target)
    def h(self, target: int) -> None: self._add(Gate.H, target)
    def p(self, angle: float, target: int) -> None: self._add(Gate.P(angle), target)
    def rx(self, angle: float, target: int) -> None: self._add(Gate.RX(angle), target)
    def ry(self, angle: float, target: int) -> None: self._add(Gate.RY(angle), target)
    def rz(self, angle: float, target: int) -> None: self._add(Gate.RZ(angle), target)
    def u(self, theta: float, phi: float, lam: float, target: int) -> None: self._add(Gate.U(theta, phi, lam), target)
    def cx(self, control: int, target: int) -> None: self._add(Gate.X, target, Controls.single(control))
    def ccx(self, c1: int, c2: int, target: int) -> None: self._add(Gate.X, target, Controls.ones([c1, c2]))
    def ch(self, control: int, target: int) -> None: self._add(Gate.H, target, Controls.single(control))
    def cy(self, control: int, target: int) -> None: self._add(Gate.Y, target, Controls.single(control))
    def cz(self, control: int, target: int) -> None: self._add(Gate.Z, target, Controls.single(control))
    def cp(self, angle: float, control: int, target: int) -> None: self._add(Gate.P(angle), target, Controls.single(control))
    def crx(self, angle: float, control: int, target: int) -> None: self._add(Gate.RX(angle), target, Controls.single(control))
    def cry(self, angle: float, control: int, target: int) -> None: self._add(Gate.RY(angle), target, Controls.single(control))
    def crz(self, angle: float, control: int, target: int) -> None: self._add(Gate.RZ(angle), target, Controls.single(control))

    def cu(self, theta: float, phi: float, lam: float, control: int, target: int) -> None:
        self._add(Gate.U(theta, phi, lam), target, Controls.single(control))

    def bit_flip_noise(self, prob: float, target: int) -> None:
        self._add(Gate.BitFlipNoise(prob), target)

    def iqft(self, targets: Sequence[int]) -> None:  # circuit.rs:438-445
        for j in range(len(targets) - 1, -1, -1):
            self.h(targets[j])
            for k in range(j - 1, -1, -1):
                self.cp(-PI / 2.0 ** (j - k), targets[j], targets[k])

    def append(self, circuit: "QuantumCircuit", reg: QuantumRegister) -> None:  # circuit.rs:448-460
        if len(reg) != sum(circuit.quantum_registers_info):
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "register size mismatch (circuit.rs:449)")
        for tr in circuit.transformations:
            self.add(QuantumTransformation(tr.gate, reg.get_shift() + tr.target, tr.controls))

    def c_append(self, circuit: "QuantumCircuit", c: int, reg: QuantumRegister) -> None:  # circuit.rs:463-477
        if reg.get_shift() <= c < reg.get_shift() + len(reg):
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "control inside the register (circuit.rs:464)")
        for tr in circuit.transformations:
            self.add(QuantumTransformation(tr.gate, reg.get_shift() + tr.target,
                                           tr.controls.new_with_control(c, reg.get_shift())))

    def mc_append(self, circuit: "QuantumCircuit", controls: Sequence[int], reg: QuantumRegister) -> None:
        """circuit.rs:480-511 (appends the circuit once per control, as the reference does)."""
        if len(set(controls)) != len(controls):
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "duplicate controls (circuit.rs:488)")
        lo, hi = reg.get_shift(), reg.get_shift() + len(reg)
        for c in controls:
            if lo <= c < hi:
                raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT,
                                          f"control {c} should not be in: Range(start: {lo} end: {hi})")
        for control in controls:
            for tr in circuit.transformations:
                self.add(QuantumTransformation(tr.gate, reg.get_shift() + tr.target,
                                               tr.controls.new_with_control(control, reg.get_shift())))

    # execution
    def _next_draw(self) -> float:
        u = float(rng.uniforms(self._seed, 1, self._draw_index)[0])
        self._draw_index += 1
        return u

    def ops(self) -> np.ndarray:
        """The pending transformations as a C-ABI op array (draws resolved)."""
        return _ops_array(self.transformations, self._next_draw)

    def execute(self) -> None:  # circuit.rs:552-600 (drains the transformations)
        trs = self.transformations
        self.transformations = []
        start = 0
        for i, tr in enumerate(trs + [None]):
            if tr is not None and tr.gate.kind != nat.UNITARY:
                continue
            if i > start:
                self.execute_ops(_ops_array(trs[start:i], self._next_draw))
            if tr is not None:  # circuit.rs:555-558: transform_u / c_transform_u
                from .unitaries import c_transform_u, transform_u

                if tr.controls.kind == Controls.NONE:
                    transform_u(self.state, tr.gate.matrix, tr.target)
                elif tr.controls.kind == Controls.SINGLE:
                    c_transform_u(self.state, tr.gate.matrix, tr.controls.controls[0], tr.target)
                else:
                    raise nat.Unsupported(nat.SPZ_ERR_UNSUPPORTED, "a Unitary takes at most one control")
            start = i + 1

    # dense unitaries (circuit.rs:514-545)
    def unitary(self, u, target: int) -> None:
        self._add(Gate.Unitary(u), target)

    def append_u(self, u, qr: QuantumRegister) -> None:
        if u.height != u.width or u.height != 1 << len(qr):
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "unitary size must be 2^len(register)")
        self.unitary(u, qr.get_shift())

    def c_unitary(self, u, c: int, t: int) -> None:
        self._add(Gate.Unitary(u), t, Controls.single(c))

    def c_append_u(self, u, c: int, qr: QuantumRegister) -> None:
        if u.height != u.width or u.height != 1 << len(qr):
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "unitary size must be 2^len(register)")
        self.c_unitary(u, c, qr.get_shift())

    def execute_ops(self, ops: np.ndarray) -> None:
        ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
        flags = _flags(self.fused, self.fast)
        nat.check(nat.lib().spz_circuit_execute(self.state.handle, nat.ptr(ops), len(ops),
                                                byref(self.qubit_tracker.c), flags, byref(self.last_stats)))


def execute_host(ops: np.ndarray, reals: np.ndarray, imags: np.ndarray, out: Optional[tuple] = None, *,
                 state: Optional[State] = None, tracker: Optional[QubitTracker] = None, fused: bool = True,
                 fast: bool = False) -> nat.spz_exec_stats:
    """QuantumCircuit::execute on a host state (spz_circuit_execute_host): runs
    `ops` on (reals, imags) and writes the result to `out` = (out_re, out_im),
    or in place when `out` is None (the reference's behaviour).  Contiguous
    float64 arrays of 2^n; page-locked arrays (e.g.
    ``torch.empty(..., pin_memory=True).numpy()``) get copies that overlap the
    leading and last passes.  `state` supplies the device memory (a new n-qubit
    handle when None)."""
    out_re, out_im = out if out is not None else (reals, imags)
    arrs = (reals, imags, out_re, out_im)
    if any(a.dtype != np.float64 or a.ndim != 1 or a.shape != reals.shape for a in arrs):
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "state arrays must be equal-length float64 vectors")
    if not all(a.flags.c_contiguous for a in arrs) or not (out_re.flags.writeable and out_im.flags.writeable):
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "state arrays must be contiguous (outputs writeable)")
    n = int(reals.size).bit_length() - 1
    if reals.size != 1 << n:
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "the state length must be a power of two")
    if state is None:
        state = State(n)
    elif state.n != n:
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "state size differs from the host arrays")
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    tr = tracker if tracker is not None else QubitTracker()
    st = nat.spz_exec_stats()
    nat.check(nat.lib().spz_circuit_execute_host(state.handle, nat.ptr(reals), nat.ptr(imags), nat.ptr(out_re),
                                                 nat.ptr(out_im), nat.ptr(ops), len(ops), byref(tr.c),
                                                 _flags(fused, fast), byref(st)))
    return st


class Program:
    """A circuit planned once and replayed as a CUDA graph (spz_program_*):
    ``Program(n, ops).run(state)`` applies `ops` to an n-qubit state with no
    planning or uploads per run.  No measurements; fused / fast as in
    QuantumCircuit.  Runs are asynchronous on the state's stream.
    `extra_flags` adds executor flags (EXEC_SHUFFLE)."""

    def __init__(self, n: int, ops: np.ndarray, fused: bool = True, fast: bool = False, extra_flags: int = 0):
        self.n = int(n)
        ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
        h = nat.c_void_p()
        flags = _flags(fused, fast) | int(extra_flags)
        nat.check(nat.lib().spz_program_create(self.n, nat.ptr(ops), len(ops), flags, byref(h)))
        self._h = h

    def run(self, state: State) -> None:
        nat.check(nat.lib().spz_program_run(self._h, state.handle))

    def stats(self) -> dict:
        st = nat.spz_exec_stats()
        nat.check(nat.lib().spz_program_stats(self._h, byref(st)))
        return {f: getattr(st, f) for f, _ in nat.spz_exec_stats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            nat.lib().spz_program_destroy(self._h)
            self._h = nat.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _flags(fused: bool, fast: bool) -> int:
    if fast:
        return nat.EXEC_FAST
    return nat.EXEC_DEFAULT if fused else nat.EXEC_UNFUSED


def plan_schedule(n: int, ops: np.ndarray, fused: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """(order, pass): the op indices in the order the executor applies them, and
    the pass (kernel launch) of each (host only, no GPU)."""
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    flags = nat.EXEC_DEFAULT if fused else nat.EXEC_UNFUSED
    cap = len(ops)
    order = np.zeros(cap, dtype=np.uint32)
    passes = np.zeros(cap, dtype=np.uint32)
    count = nat.c_size_t()
    nat.check(nat.lib().spz_plan_schedule(int(n), nat.ptr(ops), len(ops), flags, nat.ptr(order), nat.ptr(passes),
                                          cap, byref(count)))
    return order[: count.value], passes[: count.value]


def plan_passes(n: int, ops: np.ndarray, fused: bool = True, fast: bool = False,
                extra_flags: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """(local_mask, pass_ops): per pass the executor would launch, the fused
    tile pass's local qubits as a bit mask (0 for a plain one-gate pass or a
    measurement's passes) and the device ops it applies (host only, no GPU)."""
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    flags = _flags(fused, fast) | int(extra_flags)
    count = nat.c_size_t()
    nat.check(nat.lib().spz_plan_passes(int(n), nat.ptr(ops), len(ops), flags, None, None, 0, byref(count)))
    masks = np.zeros(count.value, dtype=np.uint64)
    pass_ops = np.zeros(count.value, dtype=np.uint32)
    nat.check(nat.lib().spz_plan_passes(int(n), nat.ptr(ops), len(ops), flags, nat.ptr(masks), nat.ptr(pass_ops),
                                        count.value, byref(count)))
    return masks, pass_ops


def plan_stats(n: int, ops: np.ndarray, fused: bool = True, fast: bool = False) -> dict:
    """How the executor would fuse `ops` on n qubits (host only, no GPU)."""
    st = nat.spz_exec_stats()
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    flags = _flags(fused, fast)
    nat.check(nat.lib().spz_plan_stats(int(n), nat.ptr(ops), len(ops), flags, byref(st)))
    return {f: getattr(st, f) for f, _ in nat.spz_exec_stats._fields_}


# ------------------------------------------------------------ executor tuning
# (tile qubits, threads per block) of the fused passes.  Measured on the
# 30-qubit brickwork (fast mode, share of the DFMA rate): 2^10 x 64 0.86,
# 2^10 x 128 0.78, 2^9 x 64 0.80 (the executor's defaults are 2^10 x 64).
EXECUTOR_CANDIDATES = [(10, 64), (10, 32), (9, 64), (9, 32), (8, 64)]


def _executor_signature(n: int, ops: np.ndarray) -> str:
    """Gate class x target class histogram of a circuit: the key its tuning is
    cached under (dense / diagonal / measurement; 0, 1 or more controls;
    target in the three low qubits, in a default tile, or above)."""
    import hashlib

    diag = {nat.Z, nat.P, nat.RZ}
    hist = {}
    for op in np.ascontiguousarray(ops, dtype=nat.OP_DTYPE):
        kind = int(op["gate"]["kind"])
        kc = "m" if kind == nat.M else ("d" if kind in diag else "x")
        nc = bin(int(op["controls"])).count("1") if int(op["controls_kind"]) != nat.CONTROLS_NONE else 0
        t = int(op["target"])
        tc = "low" if t < 3 else ("tile" if t < 10 else "high")
        key = f"{kc}{min(nc, 2)}{tc}"
        hist[key] = hist.get(key, 0) + 1
    text = ",".join(f"{k}:{hist[k]}" for k in sorted(hist))
    return hashlib.sha256(f"{n}|{text}".encode()).hexdigest()[:16]


def autotune_executor(state: State, ops: np.ndarray, fast: bool = False, candidates=EXECUTOR_CANDIDATES,
                      reps: int = 2, use_cache: bool = True) -> dict:
    """Pick the fused passes' tile geometry for running `ops` on `state`'s qubit
    count: each candidate is timed (device time of the passes, mean of `reps`
    runs from |0...0>; the state is overwritten), the fastest is set on the
    state, and the choice is cached per GPU name, qubit count, mode and the
    circuit's gate-class signature (SPZ_AUTOTUNE_CACHE or
    ~/.cache/spinoza_gb300/executor_autotune.json)."""
    import json
    import os
    from pathlib import Path

    import torch

    key = f"{torch.cuda.get_device_name()}|n={state.n}|fast={int(fast)}|{_executor_signature(state.n, ops)}"
    base = os.environ.get("SPZ_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "spinoza_gb300")
    path = Path(base) / "executor_autotune.json"
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = cache[key]
        state.set_tile(best["tile_qubits"], best["threads"])
        return best
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    flags = (nat.EXEC_FAST if fast else nat.EXEC_DEFAULT) | nat.EXEC_TIME_PASSES
    results = []
    for k, t in candidates:
        state.set_tile(k, t)
        ms = 0.0
        for r in range(reps + 1):  # the first run warms up
            state.reset_zero()
            tr, st = nat.spz_tracker(0, 0), nat.spz_exec_stats()
            nat.check(nat.lib().spz_circuit_execute(state.handle, nat.ptr(ops), len(ops), byref(tr), flags, byref(st)))
            if r:
                ms += st.tile_ms + st.plain_ms
        results.append({"tile_qubits": k, "threads": t, "ms": ms / reps})
    best = dict(min(results, key=lambda r: r["ms"]), candidates=results)
    state.set_tile(best["tile_qubits"], best["threads"])
    if use_cache:
        cache[key] = best
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best
