"""ctypes binding of the spinoza_gb300 C ABI (include/spinoza_gb300.h).

The library is the product's only compute path: if it is missing or fails to
load, importing the compute API raises — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, byref, c_char, c_char_p, c_double, c_int, c_int32, c_size_t, c_uint8, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_native" / "libspinoza_gb300.so"

# enum spz_status
SPZ_OK = 0
SPZ_ERR_INVALID_ARGUMENT = 1
SPZ_ERR_UNSUPPORTED = 2
SPZ_ERR_OUT_OF_MEMORY = 3
SPZ_ERR_CUDA = 4
SPZ_ERR_NULL = 5
SPZ_ERR_TIMEOUT = 6

# enum spz_gate_kind (same order as the Rust `Gate` enum, gates.rs:45-74)
H, M, X, Y, Z, P, RX, RY, RZ, SWAP, U, UNITARY, BITFLIP = range(13)

# enum spz_controls_kind (circuit.rs:55-69)
CONTROLS_NONE, CONTROLS_SINGLE, CONTROLS_ONES, CONTROLS_MIXED = range(4)

CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy: the legacy default stream (torch's stream handle 0)

EXEC_DEFAULT = 0
EXEC_UNFUSED = 1
EXEC_TIME_PASSES = 4
EXEC_FAST = 8
BATCH_WIDE_APART = 16
EXEC_TMA = 32
EXEC_TMA_PREFETCH = 64
EXEC_SHUFFLE = 128
MAX_QUBITS = 34


class SpzError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status (the reference panics)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[spz status {code}] {message}")
        self.code = code


class InvalidArgument(SpzError, ValueError):
    pass


class Unsupported(SpzError, NotImplementedError):
    pass


class spz_gate(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("q0", c_uint32), ("q1", c_uint32), ("pad_", c_uint32), ("p", c_double * 3)]


class spz_op(ctypes.Structure):
    _fields_ = [("gate", spz_gate), ("target", c_uint32), ("controls_kind", c_int32),
                ("controls", c_uint64), ("zeros", c_uint64)]


class spz_tracker(ctypes.Structure):
    _fields_ = [("measured", c_uint64), ("values", c_uint64)]


class spz_exec_stats(ctypes.Structure):
    _fields_ = [("gates", c_uint64), ("passes", c_uint64), ("tile_passes", c_uint64),
                ("bytes_moved", c_uint64), ("algorithmic_bytes", c_uint64), ("fp64_ops", c_uint64),
                ("tile_ms", c_double), ("plain_ms", c_double), ("shuffle_gates", c_uint64),
                ("io_slab_passes", c_uint64)]


class spz_pauli_term(ctypes.Structure):
    _fields_ = [("coeff", c_double), ("x_mask", c_uint64), ("z_mask", c_uint64)]


class spz_batch_instance(ctypes.Structure):
    _fields_ = [("n", c_uint32), ("nops", c_uint32), ("nparams", c_uint32), ("nterms", c_uint32),
                ("op_offset", c_uint64), ("param_offset", c_uint64), ("term_offset", c_uint64)]


class spz_batch_config(ctypes.Structure):
    _fields_ = [("tile_qubits", c_int32), ("threads", c_int32), ("wide_qubits", c_int32), ("flags", c_int32),
                ("tiles_per_item", c_int32)]


class spz_batch_stats(ctypes.Structure):
    _fields_ = [("instances", c_uint64), ("resident_instances", c_uint64), ("forward_passes", c_uint64),
                ("hamiltonian_passes", c_uint64), ("backward_passes", c_uint64), ("ctas", c_uint64),
                ("workspace_bytes", c_uint64), ("tile_qubits", c_int32), ("threads", c_int32),
                ("wide_in_kernel", c_uint64), ("work_items", c_uint64), ("wide_separate", c_uint64),
                ("wide_workspace_bytes", c_uint64), ("tiles_per_item", c_int32), ("pad_", c_int32)]


INSTANCE_DTYPE = np.dtype([("n", "<u4"), ("nops", "<u4"), ("nparams", "<u4"), ("nterms", "<u4"),
                           ("op_offset", "<u8"), ("param_offset", "<u8"), ("term_offset", "<u8")])


# numpy mirrors of the structs (for building large op lists without Python loops)
GATE_DTYPE = np.dtype([("kind", "<i4"), ("q0", "<u4"), ("q1", "<u4"), ("pad_", "<u4"), ("p", "<f8", (3,))])
OP_DTYPE = np.dtype([("gate", GATE_DTYPE), ("target", "<u4"), ("controls_kind", "<i4"),
                     ("controls", "<u8"), ("zeros", "<u8")])
TERM_DTYPE = np.dtype([("coeff", "<f8"), ("x_mask", "<u8"), ("z_mask", "<u8")])
assert OP_DTYPE.itemsize == ctypes.sizeof(spz_op) == 64
assert TERM_DTYPE.itemsize == ctypes.sizeof(spz_pauli_term) == 24

_lib = None

# (name, restype, argtypes) of every entry point declared in include/spinoza_gb300.h
SIGNATURES = [
    ("spz_last_error", c_char_p, []),
    ("spz_version", c_char_p, []),
    ("spz_state_create", c_int, [c_uint32, POINTER(c_void_p)]),
    ("spz_state_wrap", c_int, [c_uint32, c_void_p, c_void_p, POINTER(c_void_p)]),
    ("spz_state_destroy", c_int, [c_void_p]),
    ("spz_state_set_stream", c_int, [c_void_p, c_void_p]),
    ("spz_state_synchronize", c_int, [c_void_p]),
    ("spz_state_num_qubits", c_int, [c_void_p, POINTER(c_uint32)]),
    ("spz_state_device_arrays", c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p)]),
    ("spz_state_upload", c_int, [c_void_p, c_void_p, c_void_p]),
    ("spz_state_download", c_int, [c_void_p, c_void_p, c_void_p]),
    ("spz_state_reset_zero", c_int, [c_void_p]),
    ("spz_state_copy", c_int, [c_void_p, c_void_p]),
    ("spz_state_fill_random", c_int, [c_void_p, c_uint64, c_int, c_int]),
    ("spz_state_set_lazy", c_int, [c_void_p, c_int]),
    ("spz_state_settle", c_int, [c_void_p]),
    ("spz_state_set_tile", c_int, [c_void_p, c_int, c_int]),
    ("spz_apply", c_int, [c_void_p, POINTER(spz_gate), c_uint32]),
    ("spz_c_apply", c_int, [c_void_p, POINTER(spz_gate), c_uint32, c_uint32]),
    ("spz_cc_apply", c_int, [c_void_p, POINTER(spz_gate), c_uint32, c_uint32, c_uint32]),
    ("spz_mc_apply", c_int, [c_void_p, POINTER(spz_gate), c_void_p, c_uint32, c_void_p, c_uint32, c_uint32]),
    ("spz_apply_unitary", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_int32]),
    ("spz_circuit_execute", c_int, [c_void_p, c_void_p, c_size_t, POINTER(spz_tracker), c_uint32,
                                    POINTER(spz_exec_stats)]),
    ("spz_circuit_execute_host", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                                         POINTER(spz_tracker), c_uint32, POINTER(spz_exec_stats)]),
    ("spz_program_create", c_int, [c_uint32, c_void_p, c_size_t, c_uint32, POINTER(c_void_p)]),
    ("spz_program_run", c_int, [c_void_p, c_void_p]),
    ("spz_program_stats", c_int, [c_void_p, POINTER(spz_exec_stats)]),
    ("spz_program_destroy", c_int, [c_void_p]),
    ("spz_plan_stats", c_int, [c_uint32, c_void_p, c_size_t, c_uint32, POINTER(spz_exec_stats)]),
    ("spz_plan_passes", c_int, [c_uint32, c_void_p, c_size_t, c_uint32, c_void_p, c_void_p, c_size_t,
                                POINTER(c_size_t)]),
    ("spz_plan_schedule", c_int, [c_uint32, c_void_p, c_size_t, c_uint32, c_void_p, c_void_p, c_size_t,
                                  POINTER(c_size_t)]),
    ("spz_iqft", c_int, [c_void_p, c_void_p, c_uint32]),
    ("spz_measure_qubit", c_int, [c_void_p, c_uint32, c_int, c_int, c_double, POINTER(c_uint8), POINTER(c_double)]),
    ("spz_prob0", c_int, [c_void_p, c_uint32, POINTER(c_double)]),
    ("spz_qubit_expectation_value", c_int, [c_void_p, c_uint32, POINTER(c_double)]),
    ("spz_xyz_expectation_value", c_int, [c_void_p, c_char, c_void_p, c_uint32, c_void_p]),
    ("spz_xyz_expectation_value_noalloc", c_int, [c_void_p, c_void_p, c_uint32, c_char, c_void_p, c_uint32,
                                                  c_void_p, c_void_p]),
    ("spz_pauli_expectation", c_int, [c_void_p, c_void_p, c_size_t, POINTER(c_double)]),
    ("spz_norm_sqr", c_int, [c_void_p, POINTER(c_double)]),
    ("spz_sample", c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    ("spz_adjoint_gradient", c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_size_t,
                                     c_uint32, POINTER(c_double), c_void_p]),
    ("spz_batch_create", c_int, [c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, POINTER(spz_batch_config),
                                 POINTER(c_void_p)]),
    ("spz_batch_run", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("spz_batch_info", c_int, [c_void_p, POINTER(spz_batch_stats)]),
    ("spz_batch_destroy", c_int, [c_void_p]),
    ("spz_probe_fp64_fma_rate", c_int, [POINTER(c_double)]),
]


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load the library (once) and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"spinoza_gb300 native library not found at {p}; build it with "
            "`python -c 'import spinoza_gb300.build as b; b.build()'` (needs nvcc)")
    lib = ctypes.CDLL(str(p))
    for name, restype, argtypes in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _lib = lib
    return lib


def lib() -> ctypes.CDLL:
    return _lib if _lib is not None else load()


def check(code: int) -> None:
    """Turn a status code into an exception (mirrors the reference's panics)."""
    if code == SPZ_OK:
        return
    msg = lib().spz_last_error().decode(errors="replace")
    if code == SPZ_ERR_INVALID_ARGUMENT:
        raise InvalidArgument(code, msg)
    if code == SPZ_ERR_UNSUPPORTED:
        raise Unsupported(code, msg)
    raise SpzError(code, msg)


def make_gate(kind: int, params=(0.0, 0.0, 0.0), q0: int = 0, q1: int = 0) -> spz_gate:
    g = spz_gate()
    g.kind = kind
    g.q0 = q0
    g.q1 = q1
    for i, v in enumerate(params):
        g.p[i] = float(v)
    return g


def ptr(a: np.ndarray) -> c_void_p:
    return c_void_p(a.ctypes.data)


__all__ = [n for n in dir() if not n.startswith("_")]
_ = (byref,)  # re-exported helper for callers
