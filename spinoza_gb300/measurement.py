"""Single-qubit projective measurement (spinoza/src/measurement.rs:12-92)."""
from __future__ import annotations

from ctypes import byref, c_double, c_uint8
from typing import Optional

from . import _native as nat
from . import rng
from .core import State

_stream = [0, 0]  # (seed, next index) of the measurement draws


def seed_measurements(seed: int) -> None:
    """Seed the stream from which unforced measurement outcomes are drawn."""
    _stream[0], _stream[1] = int(seed), 0


def next_draw() -> float:
    u = float(rng.uniforms(_stream[0], 1, _stream[1])[0])
    _stream[1] += 1
    return u


def measure_qubit(state: State, target: int, reset: bool, v: Optional[int] = None,
                  u: Optional[float] = None) -> int:
    """Measure `target`; collapse and renormalise; with `reset`, flip a 1 back to 0.

    v forces the outcome (0 or 1), as in the reference.  Otherwise the outcome
    is 1 iff u < 1 - prob0 (Binomial(1, 1 - prob0)); u defaults to the next
    value of the seeded measurement stream."""
    if v is not None and v not in (0, 1):
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "v must be 0 or 1 (measurement.rs:32)")
    forced = -1 if v is None else int(v)
    draw = (next_draw() if u is None else float(u)) if v is None else 0.0
    out = c_uint8()
    p0 = c_double()
    nat.check(nat.lib().spz_measure_qubit(state.handle, int(target), int(bool(reset)), forced, draw,
                                          byref(out), byref(p0)))
    return int(out.value)


def prob0(state: State, target: int) -> float:
    out = c_double()
    nat.check(nat.lib().spz_prob0(state.handle, int(target), byref(out)))
    return out.value
