"""Drop-in mirror of the ``spynoza`` Python module (spynoza/src/lib.rs:1-421).

Same classes and functions (lib.rs:408-421): ``QuantumCircuit``,
``QuantumRegister``, ``PyState``, ``PyQuantumTransformation``, ``run``,
``show_table``, ``qubit_expectation_value``, ``xyz_expectation_value``,
``get_samples``.  The state lives on the GPU; ``state_vector`` returns a device
snapshot (the reference deep-copies into a host ``PyState``, lib.rs:205-211),
whose amplitudes are fetched once, on first index.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as nat
from . import circuit as _c
from . import core as _core
from .gates import Gate


class PyState:
    """Snapshot of a state (lib.rs:34-58): len, [i] -> (re, im), str."""

    def __init__(self, state: _core.State):
        self.data = state
        self._host: Optional[Tuple[np.ndarray, np.ndarray]] = None

    def _arrays(self) -> Tuple[np.ndarray, np.ndarray]:
        if self._host is None:
            self._host = self.data.to_numpy()
        return self._host

    def __len__(self) -> int:
        return len(self.data)

    def __getitem__(self, i: int) -> Tuple[float, float]:
        re, im = self._arrays()
        return float(re[i]), float(im[i])

    def __str__(self) -> str:
        re, im = self._arrays()
        return "".join(f"{a} + i{b}\n" for a, b in zip(re, im))


class QuantumRegister(_c.QuantumRegister):
    """lib.rs:64-89."""

    def __init__(self, size: int):
        self.qubits = list(range(size))


class PyQuantumTransformation:
    """Read-only view of a transformation (lib.rs:91-170)."""

    _NAMES = {nat.H: "h", nat.X: "x", nat.Y: "y", nat.Z: "z", nat.P: "p", nat.RX: "rx", nat.RY: "ry",
              nat.RZ: "rz", nat.U: "u"}

    def __init__(self, tr: _c.QuantumTransformation):
        if tr.controls.kind == _c.Controls.MIXED:
            raise nat.Unsupported(nat.SPZ_ERR_UNSUPPORTED, "Mixed controls have no Python view (lib.rs:146)")
        self.target = tr.target
        self.controls: Optional[List[int]] = list(tr.controls.controls) if tr.controls.controls else None
        if tr.gate.kind not in self._NAMES:
            raise nat.Unsupported(nat.SPZ_ERR_UNSUPPORTED, f"no Python view of {tr.gate!r} (lib.rs:160)")
        self.name = self._NAMES[tr.gate.kind]
        if tr.gate.kind in (nat.P, nat.RX, nat.RY, nat.RZ):
            self.arg: Optional[Tuple[float, float, float]] = (tr.gate.params[0], 0.0, 0.0)
        elif tr.gate.kind == nat.U:
            self.arg = tuple(tr.gate.params)
        else:
            self.arg = None

    def __str__(self) -> str:
        s = f"name: {self.name}\ntarget: {self.target}\n"
        s += f"arg: ({self.arg[0]}, {self.arg[1]}, {self.arg[2]})\n" if self.arg else "arg: None\n"
        s += f"controls: [{','.join(map(str, self.controls))}]" if self.controls else "controls: None"
        return s


class QuantumCircuit:
    """lib.rs:177-375.

    Takes registers as positional arguments (lib.rs:185-197).  A list of
    registers is also accepted and unpacked: the reference's own examples pass
    one (``QuantumCircuit([q])``, spynoza/examples/circuits.py), which its
    constructor would reject."""

    def __init__(self, *registers: QuantumRegister, seed: int = 0, fused: bool = True):
        regs: List[QuantumRegister] = []
        for r in registers:
            regs.extend(r if isinstance(r, (list, tuple)) else [r])
        self.qc = _c.QuantumCircuit(*regs, seed=seed, fused=fused)

    @property
    def num_qubits(self) -> int:
        return self.qc.state.n

    @property
    def register_sizes(self) -> List[int]:
        return list(self.qc.quantum_registers_info)

    @property
    def state_vector(self) -> PyState:
        return PyState(self.qc.state.clone())

    @property
    def transformations(self) -> List[PyQuantumTransformation]:
        return [PyQuantumTransformation(t) for t in self.qc.transformations]

    def inverse(self) -> None: self.qc.inverse()
    def h(self, target: int) -> None: self.qc.h(target)
    def x(self, target: int) -> None: self.qc.x(target)
    def y(self, target: int) -> None: self.qc.y(target)
    def z(self, target: int) -> None: self.qc.z(target)
    def p(self, angle: float, target: int) -> None: self.qc.p(angle, target)
    def rx(self, angle: float, target: int) -> None: self.qc.rx(angle, target)
    def ry(self, angle: float, target: int) -> None: self.qc.ry(angle, target)
    def rz(self, angle: float, target: int) -> None: self.qc.rz(angle, target)
    def u(self, theta: float, phi: float, lam: float, target: int) -> None: self.qc.u(theta, phi, lam, target)
    def ch(self, control: int, target: int) -> None: self.qc.ch(control, target)
    def cx(self, control: int, target: int) -> None: self.qc.cx(control, target)
    def ccx(self, c0: int, c1: int, target: int) -> None: self.qc.ccx(c0, c1, target)
    def cy(self, control: int, target: int) -> None: self.qc.cy(control, target)
    def cu(self, theta: float, phi: float, lam: float, control: int, target: int) -> None: self.qc.cu(theta, phi, lam, control, target)
    def cp(self, angle: float, control: int, target: int) -> None: self.qc.cp(angle, control, target)
    def crx(self, angle: float, control: int, target: int) -> None: self.qc.crx(angle, control, target)
    def cry(self, angle: float, control: int, target: int) -> None: self.qc.cry(angle, control, target)
    def crz(self, angle: float, control: int, target: int) -> None: self.qc.crz(angle, control, target)
    def measure(self, target: int) -> None: self.qc.measure(target)
    def swap(self, t0: int, t1: int) -> None: self.qc.swap(t0, t1)
    def iqft(self, targets: Sequence[int]) -> None: self.qc.iqft(list(targets))
    def bit_flip_noise(self, prob: float, target: int) -> None: self.qc.bit_flip_noise(prob, target)
    def add(self, q_transformation: _c.QuantumTransformation) -> None: self.qc.add(q_transformation)

    def append(self, circuit: "QuantumCircuit", quantum_register: QuantumRegister) -> None:
        self.qc.append(circuit.qc, quantum_register)

    def c_append(self, circuit: "QuantumCircuit", c: int, quantum_register: QuantumRegister) -> None:
        self.qc.c_append(circuit.qc, c, quantum_register)

    def mc_append(self, circuit: "QuantumCircuit", cs: Sequence[int], quantum_register: QuantumRegister) -> None:
        self.qc.mc_append(circuit.qc, list(cs), quantum_register)

    def execute(self) -> None:
        self.qc.execute()


def xyz_expectation_value(observable: str, state: PyState, targets: Sequence[int]) -> List[float]:
    """lib.rs:383-386."""
    return _core.xyz_expectation_value(observable, state.data, targets)


def qubit_expectation_value(state: PyState, target: int) -> float:
    """lib.rs:388-391."""
    return _core.qubit_expectation_value(state.data, target)


def get_samples(state: PyState, reservoir_size: int, num_tests: int, seed: int = 0) -> Dict[int, int]:
    """lib.rs:393-400: histogram of `reservoir_size` samples of |psi|^2."""
    return _core.reservoir_sampling(state.data, reservoir_size, num_tests, seed).get_outcome_count()


def run(qc: QuantumCircuit) -> PyState:
    """lib.rs:402-406."""
    qc.execute()
    return qc.state_vector


def show_table(s: PyState) -> str:
    """Plain-text amplitude table (the reference's to_table draws a coloured terminal table)."""
    re, im = s._arrays()
    n = max(1, int(len(re)).bit_length() - 1)
    lines = [f"{'outcome':>10} {'bits':>{n}} {'amplitude':>40} {'probability':>12}"]
    for i, (a, b) in enumerate(zip(re, im)):
        lines.append(f"{i:>10} {i:0{n}b} {a:>19.12g} {b:+19.12g}i {a * a + b * b:>12.6g}")
    return "\n".join(lines)


__all__ = ["PyState", "QuantumRegister", "PyQuantumTransformation", "QuantumCircuit", "run", "show_table",
           "qubit_expectation_value", "xyz_expectation_value", "get_samples", "Gate"]
