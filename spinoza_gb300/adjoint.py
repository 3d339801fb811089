"""Adjoint differentiation of <psi(theta)|H|psi(theta)> on the GPU.

No reference counterpart: a new form built on the gate path.  The C ABI's
spz_adjoint_gradient runs the forward circuit (fused executor), forms
lam = H psi, and sweeps backwards un-applying each gate on psi and lam while
reducing <lam|dG|psi> for every parameterised gate, with two extra state
vectors of device memory.

``AdjointExpectation`` wraps it as a torch.autograd.Function: the forward pass
returns E(theta) as a 0-d float64 tensor and keeps dE/dtheta for backward.
"""
from __future__ import annotations

import math
from ctypes import byref, c_double
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _native as nat
from .core import State, pauli_terms


def hardware_efficient_ansatz(n: int, layers: int) -> Tuple[np.ndarray, np.ndarray]:
    """layers x (RY(theta) on every qubit, RZ(theta) on every qubit, CZ ring).

    Returns (ops, param_index): ops is the C-ABI op array with zero angles;
    param_index[j] is the op whose angle is parameter j (2 n layers of them)."""
    rows, params = [], []
    for _ in range(layers):
        for kind in (nat.RY, nat.RZ):
            for q in range(n):
                params.append(len(rows))
                rows.append(((kind, 0, 0, 0, (0.0, 0.0, 0.0)), q, nat.CONTROLS_NONE, 0, 0))
        if n > 1:
            pairs = [(i, (i + 1) % n) for i in range(n)] if n > 2 else [(0, 1)]
            for c, t in pairs:
                rows.append(((nat.Z, 0, 0, 0, (0.0, 0.0, 0.0)), t, nat.CONTROLS_SINGLE, 1 << c, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    return ops, np.array(params, dtype=np.uint32)


def set_params(ops: np.ndarray, param_index: np.ndarray, theta) -> np.ndarray:
    out = ops.copy()
    out["gate"]["p"][param_index.astype(np.int64), 0] = np.asarray(theta, dtype=np.float64)
    return out


def adjoint_gradient(state: State, ops: np.ndarray, param_index: np.ndarray, terms,
                     fast: bool = False) -> Tuple[float, np.ndarray]:
    """Apply `ops` to `state` (left holding psi(theta)) and return (E, dE/dtheta).
    fast=True: fast-mode forward and a lazily scaled backward sweep (about half
    the FP64 work; equal to the exact gradients up to rounding)."""
    ops = np.ascontiguousarray(ops, dtype=nat.OP_DTYPE)
    pidx = np.ascontiguousarray(param_index, dtype=np.uint32)
    arr = terms if isinstance(terms, np.ndarray) else pauli_terms(terms)
    arr = np.ascontiguousarray(arr, dtype=nat.TERM_DTYPE)
    grad = np.zeros(len(pidx), dtype=np.float64)
    e = c_double()
    flags = nat.EXEC_FAST if fast else nat.EXEC_DEFAULT
    nat.check(nat.lib().spz_adjoint_gradient(state.handle, nat.ptr(ops), len(ops), nat.ptr(pidx), len(pidx),
                                             nat.ptr(arr), len(arr), flags, byref(e), nat.ptr(grad)))
    return e.value, grad


def expectation(state: State, ops: np.ndarray, terms) -> float:
    """Forward only: apply `ops` with the fused executor and return <psi|H|psi>."""
    from .circuit import QuantumCircuit
    from .core import pauli_expectation

    QuantumCircuit.from_state(state).execute_ops(ops)
    return pauli_expectation(state, terms)


def _torch_function():
    import torch

    class AdjointExpectation(torch.autograd.Function):
        """E(theta) = <0|U(theta)^dagger H U(theta)|0>; backward by adjoint differentiation."""

        @staticmethod
        def forward(ctx, theta, n: int, ops: np.ndarray, param_index: np.ndarray, terms: np.ndarray,
                    fast: bool = False):
            th = theta.detach().to("cpu", torch.float64).numpy()
            s = State(n)
            e, g = adjoint_gradient(s, set_params(ops, param_index, th), param_index, terms, fast=fast)
            ctx.save_for_backward(torch.from_numpy(g).to(theta.device))
            return torch.tensor(e, dtype=torch.float64, device=theta.device)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None, None, None, None

    return AdjointExpectation


_fn = None


def energy(theta, n: int, ops: np.ndarray, param_index: np.ndarray, terms,
           fast: bool = False) -> "torch.Tensor":  # noqa: F821
    """Differentiable E(theta) as a torch scalar (float64); fast=True uses the
    fast adjoint (equal to the exact gradients up to rounding)."""
    global _fn
    if _fn is None:
        _fn = _torch_function()
    arr = terms if isinstance(terms, np.ndarray) else pauli_terms(terms)
    return _fn.apply(theta, n, ops, param_index, arr, fast)


_ = (math, Optional, Sequence)
