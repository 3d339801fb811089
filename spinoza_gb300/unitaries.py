"""Dense unitaries (spinoza/src/unitaries.rs) and their application
(transform_u / c_transform_u, spinoza/src/gates.rs:1427-1487).

``Unitary`` keeps the reference's row-major SoA layout (reals, imags, height,
width).  Applying one runs on the GPU (spz_apply_unitary); building and
multiplying matrices is host work, as in the reference.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat
from .core import State
from .gates import Gate


class Unitary:
    """A 2^m x 2^m complex matrix in row-major SoA form (unitaries.rs:9-17)."""

    def __init__(self, reals, imags, height: int, width: int):
        self.reals = np.ascontiguousarray(reals, dtype=np.float64).reshape(-1)
        self.imags = np.ascontiguousarray(imags, dtype=np.float64).reshape(-1)
        self.height, self.width = int(height), int(width)
        if self.reals.size != self.height * self.width or self.imags.size != self.reals.size:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "matrix data does not match its shape")

    @classmethod
    def from_matrix(cls, m: np.ndarray) -> "Unitary":
        m = np.asarray(m, dtype=complex)
        return cls(m.real, m.imag, m.shape[0], m.shape[1])

    def matrix(self) -> np.ndarray:
        return (self.reals + 1j * self.imags).reshape(self.height, self.width)

    @classmethod
    def from_single_qubit_gate(cls, state_or_n, gate: Gate, target: int) -> "Unitary":
        """The full 2^n x 2^n matrix of a 1-qubit gate on `target` (unitaries.rs:36-70)."""
        n = state_or_n.n if isinstance(state_or_n, State) else int(state_or_n)
        g = gate.to_matrix()
        eye = np.eye(1 << target, dtype=complex)
        full = np.kron(np.kron(np.eye(1 << (n - target - 1), dtype=complex), g), eye)
        return cls.from_matrix(full)

    def conj_t(self) -> None:
        """In-place conjugate transpose (unitaries.rs:72-85)."""
        m = self.matrix().conj().T
        self.reals, self.imags = np.ascontiguousarray(m.real).reshape(-1), np.ascontiguousarray(m.imag).reshape(-1)
        self.height, self.width = self.width, self.height

    def multiply(self, other: "Unitary") -> "Unitary":
        """self x other (unitaries.rs:87-129)."""
        if self.width != other.height:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "inner dimensions differ")
        return Unitary.from_matrix(self.matrix() @ other.matrix())

    @property
    def qubits(self) -> int:
        m = int(self.height).bit_length() - 1
        if self.height != self.width or self.height != 1 << m:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "unitary must be square of size 2^m")
        return m

    def __str__(self) -> str:
        m = self.matrix()
        return "".join(" ".join(f"{z.real}+i{z.imag}" for z in row) + " \n" for row in m)


def transform_u(state: State, u: Unitary, target: int) -> None:
    """Apply `u` to qubits target .. target+m-1 (gates.rs:1427-1452)."""
    nat.check(nat.lib().spz_apply_unitary(state.handle, nat.ptr(u.reals), nat.ptr(u.imags), u.qubits, int(target), -1))


def c_transform_u(state: State, u: Unitary, control: int, target: int) -> None:
    """Controlled form (gates.rs:1455-1487); the control lies outside the block."""
    nat.check(nat.lib().spz_apply_unitary(state.handle, nat.ptr(u.reals), nat.ptr(u.imags), u.qubits, int(target),
                                          int(control)))


def apply_unitary(state: State, unitary: Unitary) -> State:
    """A new state = unitary x state, the matrix spanning the whole state (unitaries.rs:132-160)."""
    if unitary.height != len(state) or unitary.width != len(state):
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "matrix size must equal the state length")
    out = state.clone()
    transform_u(out, unitary, 0)
    return out
