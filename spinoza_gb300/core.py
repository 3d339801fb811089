"""Device-resident state and the reductions of spinoza/src/core.rs.

``State`` mirrors ``State { reals, imags, n }`` (core.rs:18-51), but its two
FP64 arrays live in HBM behind a C-ABI handle.  ``reals`` / ``imags`` return
host (numpy) copies, as the reference's public ``Vec<f64>`` fields are read.
"""
from __future__ import annotations

import ctypes
from collections import Counter
from ctypes import byref, c_double, c_uint32, c_uint64, c_void_p
from typing import Iterable, Sequence

import numpy as np

from . import _native as nat
from . import rng


class State:
    """Quantum state of n qubits, 2^n FP64 amplitudes in SoA layout on the GPU.

    State(n) is |0...0> (core.rs:32-42; n must be > 0).
    """

    __slots__ = ("_h", "n", "_keep", "__weakref__")

    def __init__(self, n: int, *, _handle: c_void_p | None = None, _keep=None):
        if _handle is None:
            if n <= 0:
                raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "n must be > 0 (core.rs:33)")
            h = c_void_p()
            nat.check(nat.lib().spz_state_create(int(n), byref(h)))
            _handle = h
        self._h = _handle
        self.n = int(n)
        self._keep = _keep

    # -- construction --------------------------------------------------------
    @classmethod
    def from_arrays(cls, reals: np.ndarray, imags: np.ndarray) -> "State":
        reals = np.ascontiguousarray(reals, dtype=np.float64)
        imags = np.ascontiguousarray(imags, dtype=np.float64)
        if reals.shape != imags.shape or reals.ndim != 1:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "reals and imags must be 1-D of equal length")
        n = int(reals.size).bit_length() - 1
        if reals.size != 1 << n or n == 0:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "length must be 2^n with n > 0")
        s = cls(n)
        s.upload(reals, imags)
        return s

    @classmethod
    def from_torch(cls, reals, imags) -> "State":
        """Wrap two CUDA float64 torch tensors (no copy; they are kept alive).

        Work is issued on torch's current stream at the time of wrapping."""
        import torch

        if reals.dtype != torch.float64 or imags.dtype != torch.float64 or not reals.is_cuda:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "need CUDA float64 tensors")
        if not (reals.is_contiguous() and imags.is_contiguous()) or reals.numel() != imags.numel():
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "need contiguous tensors of equal size")
        n = int(reals.numel()).bit_length() - 1
        h = c_void_p()
        nat.check(nat.lib().spz_state_wrap(n, c_void_p(reals.data_ptr()), c_void_p(imags.data_ptr()), byref(h)))
        s = cls(n, _handle=h, _keep=(reals, imags))
        s.set_stream(torch.cuda.current_stream())
        return s

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                nat.lib().spz_state_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    # -- reference surface -------------------------------------------------
    def __len__(self) -> int:
        return 1 << self.n

    def len(self) -> int:  # State::len (core.rs:46-50)
        return 1 << self.n

    @property
    def handle(self) -> c_void_p:
        return self._h

    @property
    def reals(self) -> np.ndarray:
        return self.to_numpy()[0]

    @property
    def imags(self) -> np.ndarray:
        return self.to_numpy()[1]

    def to_numpy(self) -> tuple[np.ndarray, np.ndarray]:
        re = np.empty(1 << self.n, dtype=np.float64)
        im = np.empty(1 << self.n, dtype=np.float64)
        nat.check(nat.lib().spz_state_download(self._h, nat.ptr(re), nat.ptr(im)))
        return re, im

    def upload(self, reals: np.ndarray, imags: np.ndarray) -> None:
        reals = np.ascontiguousarray(reals, dtype=np.float64)
        imags = np.ascontiguousarray(imags, dtype=np.float64)
        if reals.size != 1 << self.n or imags.size != 1 << self.n:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "array length must be 2^n")
        nat.check(nat.lib().spz_state_upload(self._h, nat.ptr(reals), nat.ptr(imags)))

    def reset_zero(self) -> None:
        nat.check(nat.lib().spz_state_reset_zero(self._h))

    def clone(self) -> "State":  # State: Clone (core.rs:18)
        s = State(self.n)
        nat.check(nat.lib().spz_state_copy(s._h, self._h))
        return s

    def copy_from(self, other: "State") -> None:
        nat.check(nat.lib().spz_state_copy(self._h, other._h))

    def fill_random(self, seed: int, dist: str = "normal", normalise: bool = True) -> None:
        """Seeded synthetic state on the device ('uniform' in [-1,1) or 'normal')."""
        d = {"uniform": 0, "normal": 1}[dist]
        nat.check(nat.lib().spz_state_fill_random(self._h, c_uint64(seed), d, int(normalise)))

    def synchronize(self) -> None:
        nat.check(nat.lib().spz_state_synchronize(self._h))

    def set_lazy(self, enable: bool = True) -> None:
        """Opt-in lazy per-gate arithmetic (spz_state_set_lazy): uncontrolled H,
        RX, RY and RZ applied with half the FP64 work, a pending factor folded in
        before any read; equal to the exact mode up to rounding.  States
        wrapped around torch tensors must be settle()d before the tensors are
        read directly."""
        nat.check(nat.lib().spz_state_set_lazy(self._h, int(bool(enable))))

    def settle(self) -> None:
        """Fold the lazy mode's pending factor into the arrays now."""
        nat.check(nat.lib().spz_state_settle(self._h))

    def set_tile(self, tile_qubits: int = 0, threads: int = 0) -> None:
        """Tile geometry of this state's fused passes (spz_state_set_tile):
        2^tile_qubits amplitudes (4..10) and 32 or 64 threads; 0 = defaults.
        See spinoza_gb300.circuit.autotune_executor."""
        nat.check(nat.lib().spz_state_set_tile(self._h, int(tile_qubits), int(threads)))

    def set_stream(self, stream) -> None:
        """Issue this state's work on `stream`: a torch.cuda.Stream, a raw
        cudaStream_t as int, or None for the handle's own stream.  torch's
        default stream (handle 0) maps to cudaStreamLegacy."""
        if stream is None:
            nat.check(nat.lib().spz_state_set_stream(self._h, None))
            return
        raw = int(getattr(stream, "cuda_stream", stream))
        nat.check(nat.lib().spz_state_set_stream(self._h, c_void_p(raw if raw else nat.CUDA_STREAM_LEGACY)))

    def device_arrays(self) -> tuple[int, int]:
        r, i = c_void_p(), c_void_p()
        nat.check(nat.lib().spz_state_device_arrays(self._h, byref(r), byref(i)))
        return r.value, i.value

    def norm_sqr(self) -> float:
        out = c_double()
        nat.check(nat.lib().spz_norm_sqr(self._h, byref(out)))
        return out.value

    def __str__(self) -> str:  # impl Display (core.rs:53-63)
        re, im = self.to_numpy()
        return "".join(f"{r} + i{i}\n" for r, i in zip(re, im))


def _u32(values: Iterable[int]) -> np.ndarray:
    return np.ascontiguousarray(np.fromiter((int(v) for v in values), dtype=np.uint32))


def iqft(state: State, targets: Sequence[int]) -> None:
    """Inverse QFT on `targets` (core.rs:184-191)."""
    t = _u32(targets)
    nat.check(nat.lib().spz_iqft(state.handle, nat.ptr(t), len(t)))


def qubit_expectation_value(state: State, target: int) -> float:
    """<Z_target> = 2 prob0 - 1 (core.rs:198-219)."""
    out = c_double()
    nat.check(nat.lib().spz_qubit_expectation_value(state.handle, int(target), byref(out)))
    return out.value


def xyz_expectation_value(observable: str, state: State, targets: Sequence[int]) -> list[float]:
    """Re<psi|O_t|psi> for O in 'x', 'y', 'z' and each target (core.rs:222-264)."""
    if observable not in ("x", "y", "z"):
        raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, f"observable {observable} not supported")
    t = _u32(targets)
    out = np.empty(len(t), dtype=np.float64)
    nat.check(nat.lib().spz_xyz_expectation_value(state.handle, observable.encode(), nat.ptr(t), len(t),
                                                   nat.ptr(out)))
    return out.tolist()


def pauli_terms(terms: Sequence[tuple[float, int, int]]) -> np.ndarray:
    """Pack (coeff, x_mask, z_mask) triples into the C-ABI term array."""
    a = np.zeros(len(terms), dtype=nat.TERM_DTYPE)
    for i, (c, x, z) in enumerate(terms):
        a[i] = (float(c), int(x), int(z))
    return a


def ising_hamiltonian(a: Sequence[float], b: Sequence[float]) -> np.ndarray:
    """H = sum_i a_i Z_i Z_{i+1} + sum_i b_i X_i  (len(a) = n - 1, len(b) = n)."""
    terms = [(a[i], 0, (1 << i) | (1 << (i + 1))) for i in range(len(a))]
    terms += [(b[i], 1 << i, 0) for i in range(len(b))]
    return pauli_terms(terms)


def pauli_expectation(state: State, terms) -> float:
    """<psi|H|psi> for H = sum of Pauli strings (coeff, x_mask, z_mask)."""
    arr = terms if isinstance(terms, np.ndarray) else pauli_terms(terms)
    arr = np.ascontiguousarray(arr, dtype=nat.TERM_DTYPE)
    out = c_double()
    nat.check(nat.lib().spz_pauli_expectation(state.handle, nat.ptr(arr), len(arr), byref(out)))
    return out.value


def sample(state: State, u: np.ndarray) -> np.ndarray:
    """Basis-state outcomes for uniforms u in [0,1) (library's fixed blocked CDF order)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(u.size, dtype=np.uint64)
    nat.check(nat.lib().spz_sample(state.handle, nat.ptr(u), u.size, nat.ptr(out)))
    return out


class Reservoir:
    """Sampling result with the reference's interface (core.rs:65-129).

    The reference fills a reservoir of k entries by weighted reservoir sampling
    over `num_tests` uniform candidates (unseeded).  Each entry is then a draw
    from |psi_i|^2 (for num_tests large); here the k entries are drawn exactly
    from |psi_i|^2 by the device inverse-CDF sampler, from a seeded stream."""

    def __init__(self, k: int):
        self.entries = np.zeros(int(k), dtype=np.uint64)

    def sampling(self, state: State, num_tests: int, seed: int = 0) -> None:
        if len(self.entries):
            self.entries = sample(state, rng.uniforms(seed, len(self.entries)))

    def get_outcome_count(self) -> dict[int, int]:
        return dict(Counter(int(e) for e in self.entries))


def reservoir_sampling(state: State, reservoir_size: int, num_tests: int, seed: int = 0) -> Reservoir:
    """core.rs:125-129."""
    r = Reservoir(reservoir_size)
    r.sampling(state, num_tests, seed)
    return r


def fp64_fma_rate() -> float:
    """Measured FP64 FMA issue rate of the current GPU (FMA/s)."""
    out = c_double()
    nat.check(nat.lib().spz_probe_fp64_fma_rate(byref(out)))
    return out.value


_ = (ctypes, c_uint32)
