"""Seeded, counter-based random streams (splitmix64), shared by the host API,
the benchmarks and the tests so that every synthetic input is reproducible.

u64(seed, i) = mix(mix(seed + G) + (i + 1) * G) with G = 0x9E3779B97F4A7C15 and
mix the splitmix64 finaliser; uniform(seed, i) = (u64 >> 11) * 2^-53 in [0, 1).
The device fill kernel (spz_state_fill_random) uses the same stream.
"""
from __future__ import annotations

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def u64(seed: int, start: int, count: int) -> np.ndarray:
    """count consecutive 64-bit values of stream `seed`, from index `start`."""
    with np.errstate(over="ignore"):
        key = _mix(np.array([seed], dtype=np.uint64) + GOLDEN)[0]
        idx = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        return _mix(key + idx * GOLDEN)


def u64_at(seed: int, idx: np.ndarray) -> np.ndarray:
    """The 64-bit values of stream `seed` at arbitrary counter positions `idx`."""
    with np.errstate(over="ignore"):
        key = _mix(np.array([seed], dtype=np.uint64) + GOLDEN)[0]
        return _mix(key + (np.asarray(idx, dtype=np.uint64) + np.uint64(1)) * GOLDEN)


def uniform_amplitudes(seed: int, idx: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Amplitudes `idx` of uniform_state(n, seed) for any n, without the rest of the state."""
    i2 = np.asarray(idx, dtype=np.uint64) * np.uint64(2)
    ure = (u64_at(seed, i2) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    uim = (u64_at(seed, i2 + np.uint64(1)) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return 2.0 * ure - 1.0, 2.0 * uim - 1.0


def uniforms(seed: int, count: int, start: int = 0) -> np.ndarray:
    """count uniforms in [0, 1) with 53 random bits each."""
    return (u64(seed, start, count) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def uniform_state(n: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """reals/imags i.i.d. uniform in [-1, 1): re[i] = 2u(2i) - 1, im[i] = 2u(2i+1) - 1 (exact)."""
    u = uniforms(seed, 2 << n)
    return 2.0 * u[0::2] - 1.0, 2.0 * u[1::2] - 1.0


def normal_state(n: int, seed: int, normalise: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """reals/imags i.i.d. N(0,1) by Box-Muller on (u(2i), u(2i+1)), optionally normalised."""
    u = uniforms(seed, 2 << n)
    r = np.sqrt(-2.0 * np.log1p(-u[0::2]))
    ang = 2.0 * np.pi * u[1::2]
    re, im = r * np.cos(ang), r * np.sin(ang)
    if normalise:
        s = 1.0 / np.sqrt(np.sum(re * re + im * im))
        re, im = re * s, im * s
    return re, im
