"""spinoza_gb300 — GB300-native FP64 state-vector engine, a drop-in for the
gate-application path of Spinoza (QuState/spinoza).

Module map (reference module -> here):
  spinoza::core         -> spinoza_gb300.core   (State, iqft, expectations, sampling)
  spinoza::gates        -> spinoza_gb300.gates  (Gate, apply, c_apply, cc_apply, mc_apply)
  spinoza::circuit      -> spinoza_gb300.circuit (QuantumRegister, QuantumCircuit, ...)
  spinoza::measurement  -> spinoza_gb300.measurement (measure_qubit)
  spynoza (PyO3)        -> spinoza_gb300.spynoza
  (new) adjoint differentiation -> spinoza_gb300.adjoint
  (new) batched variational runs -> spinoza_gb300.batch

All compute runs in the CUDA library ``_native/libspinoza_gb300.so`` (sm_103a),
reached through the C ABI in include/spinoza_gb300.h.
"""
from . import _native
from .build import build, library_path

__version__ = "0.1.0"


def load():
    """Load the native library (raises if it has not been built)."""
    return _native.load()


__all__ = ["build", "library_path", "load", "__version__"]
