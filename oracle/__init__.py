"""ORACLE — test infrastructure only.

ctypes wrapper around oracle/_build/liboracle.so, the CPU restatement of the
reference's (QuState/spinoza v0.5.1) gate-application path.  Used only by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm, as
the checker.  The product (spinoza_gb300/) never imports this package.

Each function operates on numpy arrays (reals, imags) in place, like the
reference's functions on `&mut State`.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_char, c_double, c_int, c_uint8, c_uint32, c_uint64, c_void_p
from pathlib import Path
from typing import Iterable, Optional, Sequence

import numpy as np

from . import build as _build

H, M, X, Y, Z, P, RX, RY, RZ, SWAP, U, UNITARY, BITFLIP = range(13)


class Gate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("q0", c_uint32), ("q1", c_uint32), ("pad", c_uint32),
                ("p", c_double * 3)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        v, d = c_void_p, c_double
        sig = {
            "orc_apply": [c_int, v, v, POINTER(Gate), c_int],
            "orc_c_apply": [c_int, v, v, POINTER(Gate), c_int, c_int],
            "orc_cc_apply": [c_int, v, v, POINTER(Gate), c_int, c_int, c_int],
            "orc_mc_apply": [c_int, v, v, POINTER(Gate), c_uint64, c_uint64, c_int],
            "orc_execute": [c_int, v, v, v, c_uint64, POINTER(c_uint64), POINTER(c_uint64)],
            "orc_measure_qubit": [c_int, v, v, c_int, c_int, c_int, d, POINTER(c_uint8), POINTER(d)],
            "orc_prob0": [c_int, v, v, c_int],
            "orc_qubit_expectation_value": [c_int, v, v, c_int],
            "orc_xyz_expectation_value": [c_int, v, v, c_char, v, c_uint32, v],
            "orc_pauli_expectation": [c_int, v, v, v, c_uint64, POINTER(d)],
            "orc_iqft": [c_int, v, v, v, c_uint32],
            "orc_sample": [c_int, v, v, v, c_uint64, v],
            "orc_apply_unitary": [c_int, v, v, v, v, c_int, c_int, c_int],
            "orc_stream_u64": [c_uint64, c_uint64],
            "orc_stream_uniform": [c_uint64, c_uint64],
            "orc_fill_uniform": [c_int, v, v, c_uint64],
            "orc_num_threads": [],
        }
        res = {"orc_prob0": d, "orc_qubit_expectation_value": d, "orc_stream_u64": c_uint64,
               "orc_stream_uniform": d, "orc_fill_uniform": None, "orc_num_threads": c_int}
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res.get(name, c_int)
        _lib = L
    return _lib


def _p(a: np.ndarray) -> c_void_p:
    assert a.flags.c_contiguous
    return c_void_p(a.ctypes.data)


def _n(re: np.ndarray) -> int:
    n = int(re.size).bit_length() - 1
    assert re.size == 1 << n and re.dtype == np.float64
    return n


class OracleError(RuntimeError):
    pass


def _check(rc: int) -> None:
    if rc != 0:
        raise OracleError(f"oracle status {rc}")


def gate(kind: int, params: Sequence[float] = (), q0: int = 0, q1: int = 0) -> Gate:
    g = Gate()
    g.kind, g.q0, g.q1 = kind, q0, q1
    for i, val in enumerate(params):
        g.p[i] = float(val)
    return g


def zero_state(n: int) -> tuple[np.ndarray, np.ndarray]:
    """State::new(n) (core.rs:32-42)."""
    re = np.zeros(1 << n)
    re[0] = 1.0
    return re, np.zeros(1 << n)


def apply(g: Gate, re: np.ndarray, im: np.ndarray, target: int) -> None:
    _check(lib().orc_apply(_n(re), _p(re), _p(im), byref(g), target))


def c_apply(g: Gate, re, im, control: int, target: int) -> None:
    _check(lib().orc_c_apply(_n(re), _p(re), _p(im), byref(g), control, target))


def cc_apply(g: Gate, re, im, c0: int, c1: int, target: int) -> None:
    _check(lib().orc_cc_apply(_n(re), _p(re), _p(im), byref(g), c0, c1, target))


def mc_apply(g: Gate, re, im, controls: Iterable[int], zeros: Optional[Iterable[int]], target: int) -> None:
    cm = 0
    for c in controls:
        cm |= 1 << c
    zm = 0
    for z in zeros or ():
        zm |= 1 << z
    _check(lib().orc_mc_apply(_n(re), _p(re), _p(im), byref(g), cm, zm, target))


def execute(ops: np.ndarray, re, im, measured: int = 0, values: int = 0) -> tuple[int, int]:
    """QuantumCircuit::execute on an op array with the product's spz_op layout."""
    m, v = c_uint64(measured), c_uint64(values)
    ops = np.ascontiguousarray(ops)
    _check(lib().orc_execute(_n(re), _p(re), _p(im), _p(ops), len(ops), byref(m), byref(v)))
    return m.value, v.value


def measure_qubit(re, im, target: int, reset: bool, forced: Optional[int] = None, u: float = 0.0) -> tuple[int, float]:
    out, p0 = c_uint8(), c_double()
    _check(lib().orc_measure_qubit(_n(re), _p(re), _p(im), target, int(reset), -1 if forced is None else forced,
                                   u, byref(out), byref(p0)))
    return out.value, p0.value


def prob0(re, im, target: int) -> float:
    return lib().orc_prob0(_n(re), _p(re), _p(im), target)


def qubit_expectation_value(re, im, target: int) -> float:
    return lib().orc_qubit_expectation_value(_n(re), _p(re), _p(im), target)


def xyz_expectation_value(obs: str, re, im, targets: Sequence[int]) -> list[float]:
    t = np.ascontiguousarray(np.array(targets, dtype=np.uint32))
    out = np.empty(len(t))
    _check(lib().orc_xyz_expectation_value(_n(re), _p(re), _p(im), obs.encode(), _p(t), len(t), _p(out)))
    return out.tolist()


def pauli_expectation(re, im, terms: np.ndarray) -> float:
    terms = np.ascontiguousarray(terms)
    out = c_double()
    _check(lib().orc_pauli_expectation(_n(re), _p(re), _p(im), _p(terms), len(terms), byref(out)))
    return out.value


def iqft(re, im, targets: Sequence[int]) -> None:
    t = np.ascontiguousarray(np.array(targets, dtype=np.uint32))
    _check(lib().orc_iqft(_n(re), _p(re), _p(im), _p(t), len(t)))


def apply_unitary(re, im, matrix: np.ndarray, target: int, control: int = -1) -> None:
    mr = np.ascontiguousarray(matrix.real, dtype=np.float64)
    mi = np.ascontiguousarray(matrix.imag, dtype=np.float64)
    m = int(matrix.shape[0]).bit_length() - 1
    _check(lib().orc_apply_unitary(_n(re), _p(re), _p(im), _p(mr), _p(mi), m, target, control))


def sample(re, im, u: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(u.size, dtype=np.uint64)
    _check(lib().orc_sample(_n(re), _p(re), _p(im), _p(u), u.size, _p(out)))
    return out


def uniform_state(n: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    re, im = np.empty(1 << n), np.empty(1 << n)
    lib().orc_fill_uniform(n, _p(re), _p(im), seed)
    return re, im


def stream_uniform(seed: int, i: int) -> float:
    return lib().orc_stream_uniform(seed, i)


def num_threads() -> int:
    return lib().orc_num_threads()


# --------------------------------------------------------------------------
# numpy restatements used where the product library must not be loaded (the
# benchmark's reference arm): the op record layout, the seeded uniform stream
# and the per-gate algorithmic byte counts.

GATE_DTYPE = np.dtype([("kind", "<i4"), ("q0", "<u4"), ("q1", "<u4"), ("pad_", "<u4"), ("p", "<f8", (3,))])
# Same 64-byte record as `struct Op` in spz_oracle.cpp (the flat form of the
# reference's QuantumTransformation, circuit.rs:113-120).
OP_DTYPE = np.dtype([("gate", GATE_DTYPE), ("target", "<u4"), ("controls_kind", "<i4"),
                     ("controls", "<u8"), ("zeros", "<u8")])
CONTROLS_NONE, CONTROLS_SINGLE, CONTROLS_ONES, CONTROLS_MIXED = range(4)

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniforms(seed: int, count: int, start: int = 0) -> np.ndarray:
    """Uniforms [start, start + count) of the seeded splitmix64 stream, the same
    values as orc_stream_uniform (53 random bits each)."""
    with np.errstate(over="ignore"):
        key = _mix64(np.array([seed], dtype=np.uint64) + _GOLDEN)[0]
        idx = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        return (_mix64(key + idx * _GOLDEN) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def algorithmic_bytes(ops: np.ndarray, n: int) -> int:
    """Sum over the ops of the bytes one unfused pass of that gate must read and
    write on 2^n FP64 SoA amplitudes: every amplitude (32 N) for a gate that
    mixes or rephases both halves, half of them (16 N) for Z, P and SWAP, and
    2^-k of that under k controls.  Measurements are not counted."""
    N = 1 << n
    total = 0
    for op in ops:
        kind = int(op["gate"]["kind"])
        nc = bin(int(op["controls"])).count("1") if int(op["controls_kind"]) != CONTROLS_NONE else 0
        if kind == M:
            continue
        full = 16 * N if kind in (Z, P, SWAP) else 32 * N
        total += full >> nc
    return total


_ = Path
