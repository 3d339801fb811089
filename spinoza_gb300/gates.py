"""Gates and gate application (spinoza/src/gates.rs).

``Gate`` mirrors the Rust enum (gates.rs:45-74): ``Gate.H``, ``Gate.M``,
``Gate.X``, ``Gate.Y``, ``Gate.Z`` are values; ``Gate.P(theta)``,
``Gate.RX/RY/RZ(theta)``, ``Gate.SWAP(t0, t1)``, ``Gate.U(theta, phi, lam)``
and ``Gate.BitFlipNoise(prob)`` build the payload variants.
"""
from __future__ import annotations

import cmath
import math
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _native as nat
from .core import State

_NAMES = {nat.H: "H", nat.M: "M", nat.X: "X", nat.Y: "Y", nat.Z: "Z", nat.P: "P", nat.RX: "RX",
          nat.RY: "RY", nat.RZ: "RZ", nat.SWAP: "SWAP", nat.U: "U", nat.UNITARY: "Unitary",
          nat.BITFLIP: "BitFlipNoise"}


class Gate:
    __slots__ = ("kind", "params", "qubits", "matrix")

    def __init__(self, kind: int, params: Sequence[float] = (), qubits: Sequence[int] = (), matrix=None):
        self.kind = int(kind)
        p = [float(v) for v in params] + [0.0] * (3 - len(params))
        self.params = tuple(p[:3])
        q = [int(v) for v in qubits] + [0] * (2 - len(qubits))
        self.qubits = tuple(q[:2])
        self.matrix = matrix  # Unitary payload (gates.rs:67)

    @staticmethod
    def Unitary(u) -> "Gate":
        """A dense unitary (spinoza_gb300.unitaries.Unitary) acting on qubits target .. target+m-1."""
        return Gate(nat.UNITARY, matrix=u)

    # payload variants
    @staticmethod
    def P(theta: float) -> "Gate":
        return Gate(nat.P, (theta,))

    @staticmethod
    def RX(theta: float) -> "Gate":
        return Gate(nat.RX, (theta,))

    @staticmethod
    def RY(theta: float) -> "Gate":
        return Gate(nat.RY, (theta,))

    @staticmethod
    def RZ(theta: float) -> "Gate":
        return Gate(nat.RZ, (theta,))

    @staticmethod
    def U(theta: float, phi: float, lam: float) -> "Gate":
        return Gate(nat.U, (theta, phi, lam))

    @staticmethod
    def SWAP(t0: int, t1: int) -> "Gate":
        return Gate(nat.SWAP, (), (t0, t1))

    @staticmethod
    def BitFlipNoise(prob: float, draw: Optional[float] = None) -> "Gate":
        """X with probability `prob` (gates.rs:1365-1374).  `draw` is the uniform
        compared against prob (X iff draw <= prob); None draws it at apply time
        from the seeded noise stream."""
        return Gate(nat.BITFLIP, (prob, math.nan if draw is None else draw))

    def __repr__(self) -> str:
        name = _NAMES.get(self.kind, "?")
        if self.kind in (nat.P, nat.RX, nat.RY, nat.RZ, nat.BITFLIP):
            return f"{name}({self.params[0]})"
        if self.kind == nat.U:
            return f"U{self.params}"
        if self.kind == nat.SWAP:
            return f"SWAP{self.qubits}"
        return name

    def __eq__(self, other) -> bool:
        return isinstance(other, Gate) and (self.kind, self.params, self.qubits) == (other.kind, other.params, other.qubits)

    def __hash__(self) -> int:
        return hash((self.kind, self.params, self.qubits))

    def inverse(self) -> "Gate":
        """gates.rs:78-94: angles negate; U(t, p, l)^-1 = U(-t, -l, -p); M/BitFlipNoise panic."""
        k = self.kind
        if k in (nat.H, nat.X, nat.Y, nat.Z, nat.SWAP):
            return self
        if k in (nat.P, nat.RX, nat.RY, nat.RZ):
            return Gate(k, (-self.params[0],))
        if k == nat.U:
            t, p, l = self.params
            return Gate(nat.U, (-t, -l, -p))
        if k == nat.UNITARY:  # gates.rs:87-90: conjugate transpose
            from .unitaries import Unitary

            u = Unitary(self.matrix.reals.copy(), self.matrix.imags.copy(), self.matrix.height, self.matrix.width)
            u.conj_t()
            return Gate.Unitary(u)
        raise nat.Unsupported(nat.SPZ_ERR_UNSUPPORTED, f"{self!r} has no inverse (gates.rs:86)")

    def to_matrix(self) -> np.ndarray:
        """2x2 complex matrix (gates.rs:97-191)."""
        k, (a, b, c) = self.kind, self.params
        s2 = 1.0 / math.sqrt(2.0)
        if k == nat.H:
            return np.array([[s2, s2], [s2, -s2]], dtype=complex)
        if k == nat.X:
            return np.array([[0, 1], [1, 0]], dtype=complex)
        if k == nat.Y:
            return np.array([[0, -1j], [1j, 0]], dtype=complex)
        if k == nat.Z:
            return np.array([[1, 0], [0, -1]], dtype=complex)
        if k == nat.P:
            return np.array([[1, 0], [0, cmath.exp(1j * a)]], dtype=complex)
        if k == nat.RX:
            t = a / 2
            return np.array([[math.cos(t), -1j * math.sin(t)], [-1j * math.sin(t), math.cos(t)]], dtype=complex)
        if k == nat.RY:
            t = a / 2
            return np.array([[math.cos(t), -math.sin(t)], [math.sin(t), math.cos(t)]], dtype=complex)
        if k == nat.RZ:
            t = a / 2
            return np.array([[complex(math.cos(t), -math.sin(t)), 0], [0, complex(math.cos(t), math.sin(t))]])
        if k == nat.U:
            t = a / 2
            return np.array([[math.cos(t), -cmath.exp(1j * c) * math.sin(t)],
                             [cmath.exp(1j * b) * math.sin(t), cmath.exp(1j * (b + c)) * math.cos(t)]])
        raise nat.Unsupported(nat.SPZ_ERR_UNSUPPORTED, f"{self!r} has no 2x2 matrix")

    def c_struct(self) -> nat.spz_gate:
        return nat.make_gate(self.kind, self.params, *self.qubits)


Gate.H = Gate(nat.H)
Gate.M = Gate(nat.M)
Gate.X = Gate(nat.X)
Gate.Y = Gate(nat.Y)
Gate.Z = Gate(nat.Z)

_flip_stream = [0, 0]  # (seed, next index) of the BitFlipNoise draws


def seed_noise(seed: int) -> None:
    """Seed the stream that resolves BitFlipNoise draws made through apply()."""
    _flip_stream[0], _flip_stream[1] = int(seed), 0


def next_noise_draw() -> float:
    from . import rng

    u = float(rng.uniforms(_flip_stream[0], 1, _flip_stream[1])[0])
    _flip_stream[1] += 1
    return u


def _resolve(gate: Gate) -> nat.spz_gate:
    g = gate.c_struct()
    if gate.kind == nat.BITFLIP and math.isnan(gate.params[1]):
        g.p[1] = next_noise_draw()
    return g


def apply(gate: Gate, state: State, target: int) -> None:
    """Uncontrolled gate on `target` (gates.rs:215-232)."""
    if gate.kind == nat.UNITARY:
        from .unitaries import transform_u

        transform_u(state, gate.matrix, target)
        return
    g = _resolve(gate)
    nat.check(nat.lib().spz_apply(state.handle, nat.byref(g), int(target)))


def c_apply(gate: Gate, state: State, control: int, target: int) -> None:
    """Gate on `target` where `control` reads 1 (gates.rs:257-269)."""
    if gate.kind == nat.UNITARY:
        from .unitaries import c_transform_u

        c_transform_u(state, gate.matrix, control, target)
        return
    g = gate.c_struct()
    nat.check(nat.lib().spz_c_apply(state.handle, nat.byref(g), int(control), int(target)))


def cc_apply(gate: Gate, state: State, control0: int, control1: int, target: int) -> None:
    """Two controls, single target (gates.rs:272-277)."""
    g = gate.c_struct()
    nat.check(nat.lib().spz_cc_apply(state.handle, nat.byref(g), int(control0), int(control1), int(target)))


def mc_apply(gate: Gate, state: State, controls: Sequence[int], zeros: Optional[Iterable[int]], target: int) -> None:
    """Gate on `target` where every control reads 1, except `zeros`, which must read 0 (gates.rs:290-320)."""
    g = gate.c_struct()
    c = np.ascontiguousarray(np.array([int(v) for v in controls], dtype=np.uint32))
    z = np.ascontiguousarray(np.array(sorted(int(v) for v in zeros) if zeros else [], dtype=np.uint32))
    nat.check(nat.lib().spz_mc_apply(state.handle, nat.byref(g), nat.ptr(c), len(c), nat.ptr(z), len(z), int(target)))
