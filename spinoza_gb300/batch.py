"""Batched variational instances: forward <H> and adjoint gradients of many
independent circuits of uneven qubit counts in one persistent, graph-replayed
launch (spz_batch_*).  No reference counterpart (new form).

``hea_workload`` builds the seeded variational workload
(4096 hardware-efficient ansatz instances, qubits uniform in 10..22, depth
uniform in 2..10, RY/RZ layers + CZ ring, observable sum a_i Z_i Z_{i+1} + b_i X_i).
``autotune`` times candidate launch shapes (tile qubits x threads per CTA) and
caches the fastest per GPU and batch signature.
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import time
from ctypes import byref, c_void_p
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _native as nat
from . import rng
from .adjoint import hardware_efficient_ansatz
from .core import ising_hamiltonian

Instance = Tuple[int, np.ndarray, np.ndarray, np.ndarray, np.ndarray]  # (n, ops, param_index, theta, terms)


def hea_instance(n: int, depth: int, seed: int) -> Instance:
    """One instance: the RY/RZ/CZ-ring ansatz with angles U[-pi, pi] and the
    observable sum a_i Z_i Z_{i+1} + b_i X_i with a, b ~ N(0,1), all from `seed`."""
    ops, pidx = hardware_efficient_ansatz(n, depth)
    theta = (rng.uniforms(seed, len(pidx)) * 2.0 - 1.0) * math.pi
    u = rng.uniforms(seed + 1_000_003, 4 * n)
    a = np.sqrt(-2.0 * np.log1p(-u[: n - 1])) * np.cos(2.0 * math.pi * u[n: 2 * n - 1])
    b = np.sqrt(-2.0 * np.log1p(-u[2 * n: 3 * n])) * np.cos(2.0 * math.pi * u[3 * n: 4 * n])
    return n, ops, pidx, theta, ising_hamiltonian(a, b)


def hea_workload(count: int = 4096, qmin: int = 10, qmax: int = 22, dmin: int = 2, dmax: int = 10,
                      base_seed: int = 8) -> List[Instance]:
    """Qubits uniform in qmin..qmax and depth uniform in dmin..dmax from stream
    `base_seed`; instance k draws its angles and observable from seed base_seed + k."""
    u = rng.uniforms(base_seed, 2 * count)
    qs = qmin + np.floor(u[:count] * (qmax - qmin + 1)).astype(int)
    ds = dmin + np.floor(u[count:] * (dmax - dmin + 1)).astype(int)
    return [hea_instance(int(qs[k]), int(ds[k]), base_seed + k) for k in range(count)]


def pack(instances: Sequence[Instance]):
    """Concatenate instances into the flat arrays of the C ABI."""
    inst = np.zeros(len(instances), dtype=nat.INSTANCE_DTYPE)
    ops_l, pidx_l, theta_l, terms_l = [], [], [], []
    o = p = t = 0
    for i, (n, ops, pidx, theta, terms) in enumerate(instances):
        inst[i] = (n, len(ops), len(pidx), len(terms), o, p, t)
        ops_l.append(ops); pidx_l.append(np.asarray(pidx, dtype=np.uint32))
        theta_l.append(np.asarray(theta, dtype=np.float64)); terms_l.append(terms)
        o += len(ops); p += len(pidx); t += len(terms)
    cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros(0, dtype=dt), dtype=dt)
    return (inst, cat(ops_l, nat.OP_DTYPE), cat(pidx_l, np.uint32), cat(theta_l, np.float64),
            cat(terms_l, nat.TERM_DTYPE))


class Batch:
    """A planned, device-resident batch; run(theta) -> (energies, grads)."""

    def __init__(self, instances: Sequence[Instance], tile_qubits: int = 0, threads: int = 0, wide_qubits: int = 0,
                 fast: bool = False, tiles_per_item: int = 0, wide_apart: bool = False):
        """tile_qubits / threads: launch shape of the persistent kernel;
        wide_qubits: instances of at least this many qubits are spread over
        many CTAs as work items of tiles_per_item tiles (0: the library's
        defaults, 31: never); fast: those run one at a time across the GPU with
        the fast adjoint (equal to the exact one up to rounding); wide_apart:
        they run one at a time across the GPU in the exact mode."""
        self.inst, self.ops, self.pidx, self.theta, self.terms = pack(instances)
        cfg = nat.spz_batch_config(int(tile_qubits), int(threads), int(wide_qubits),
                                   (nat.EXEC_FAST if fast else nat.EXEC_DEFAULT) |
                                   (nat.BATCH_WIDE_APART if wide_apart else 0), int(tiles_per_item))
        h = c_void_p()
        nat.check(nat.lib().spz_batch_create(nat.ptr(self.inst), len(self.inst), nat.ptr(self.ops),
                                             nat.ptr(self.pidx), nat.ptr(self.terms), byref(cfg), byref(h)))
        self._h = h
        self.energies = np.zeros(len(self.inst))
        self.grads = np.zeros(len(self.theta))

    def run(self, theta: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
        th = self.theta if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
        if th.size != self.theta.size:
            raise nat.InvalidArgument(nat.SPZ_ERR_INVALID_ARGUMENT, "theta has the wrong length")
        nat.check(nat.lib().spz_batch_run(self._h, nat.ptr(th), nat.ptr(self.energies), nat.ptr(self.grads)))
        return self.energies.copy(), self.grads.copy()

    def info(self) -> dict:
        st = nat.spz_batch_stats()
        nat.check(nat.lib().spz_batch_info(self._h, byref(st)))
        return {f: getattr(st, f) for f, _ in nat.spz_batch_stats._fields_}

    def split(self, values: np.ndarray) -> List[np.ndarray]:
        """Per-instance views of a flat parameter-indexed array."""
        return [values[int(r["param_offset"]): int(r["param_offset"]) + int(r["nparams"])] for r in self.inst]

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            nat.lib().spz_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# (tile qubits, threads per CTA, tiles per work item of a wide instance)
# On the 4096-instance, 10-22-qubit batch (one GB300, one box): 2^9 x 64 x 64
# 25.65 s, x 16 25.71 s, 2^9 x 128 26.9 s, 2^10 x 128 26.7 s, 2^11 x 128
# 28.2 s, 2^8 x 64 26.9 s (wide instances as work items in the launch).
CANDIDATES = [(9, 64, 64), (9, 64, 16), (9, 128, 64), (10, 64, 64), (10, 128, 16), (11, 128, 16), (8, 64, 64)]


def _signature(instances: Sequence[Instance]) -> str:
    h = hashlib.sha256()
    for n, ops, pidx, _, terms in instances:
        h.update(np.array([n, len(ops), len(pidx), len(terms)], dtype=np.int64).tobytes())
    return h.hexdigest()[:16]


def _cache_path() -> Path:
    base = os.environ.get("SPZ_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "spinoza_gb300")
    return Path(base) / "batch_autotune.json"


def autotune(instances: Sequence[Instance], candidates=CANDIDATES, reps: int = 1, use_cache: bool = True,
             sample: int = 512) -> dict:
    """Pick (tile_qubits, threads, tiles_per_item) for this batch by timing
    each candidate on a stratified sample of `sample` instances (every size and
    depth represented); the choice is cached per GPU name and batch signature
    (SPZ_AUTOTUNE_CACHE or ~/.cache/spinoza_gb300/batch_autotune.json)."""
    import torch

    key = f"{torch.cuda.get_device_name()}|{_signature(instances)}"
    path = _cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        return cache[key]
    order = sorted(range(len(instances)), key=lambda i: (instances[i][0], len(instances[i][1])))
    step = max(1, len(order) // max(1, sample))
    subset = [instances[i] for i in order[::step]]
    results = []
    for k, t, tpi in candidates:
        try:
            b = Batch(subset, tile_qubits=k, threads=t, tiles_per_item=tpi)
        except nat.SpzError:
            continue
        b.run()  # graph capture + warm-up
        t0 = time.perf_counter()
        for _ in range(reps):
            b.run()
        dt = (time.perf_counter() - t0) / reps
        results.append({"tile_qubits": k, "threads": t, "tiles_per_item": tpi, "seconds": dt})
        b.close()
    best = min(results, key=lambda r: r["seconds"])
    best = dict(best, candidates=results, sample=len(subset))
    if use_cache:
        cache[key] = best
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best
