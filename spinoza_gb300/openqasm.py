"""OpenQASM 2.0 front-end: a program -> QuantumCircuit (spinoza/src/openqasm.rs:13-172).

The reference hands the source to the third-party `qasm` crate (1.0.0) and
maps h, x, y, z, rx, ry, rz, u, cp and cx onto the circuit builders; this is
a self-contained parser for the same statements, plus the standard qelib1
gates the builders can express (s, sdg, t, tdg, p/u1, u2, u3, cz, cy, ch,
crx, cry, crz, cu/cu3, ccx, swap), `measure`, `barrier` and `creg`.
Angles are arithmetic expressions over numbers and `pi`.  Registers are laid
out in declaration order (the reference iterates a HashMap, so its order for
several registers is unspecified).
"""
from __future__ import annotations

import ast
import math
import operator
import re
from pathlib import Path
from typing import Dict, List, Tuple

from . import _native as nat
from .circuit import QuantumCircuit, QuantumRegister


class QasmError(ValueError):
    pass


_BIN = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
        ast.Pow: operator.pow}
_UN = {ast.UAdd: operator.pos, ast.USub: operator.neg}
_FUN = {"sin": math.sin, "cos": math.cos, "tan": math.tan, "exp": math.exp, "ln": math.log, "sqrt": math.sqrt}


def eval_angle(expr: str) -> float:
    """Evaluate an OpenQASM parameter expression (numbers, pi, + - * / ^, functions)."""
    try:
        tree = ast.parse(expr.replace("^", "**"), mode="eval")
    except SyntaxError as e:
        raise QasmError(f"bad parameter expression {expr!r}") from e

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return float(node.value)
        if isinstance(node, ast.Name) and node.id == "pi":
            return math.pi
        if isinstance(node, ast.BinOp) and type(node.op) in _BIN:
            return _BIN[type(node.op)](ev(node.left), ev(node.right))
        if isinstance(node, ast.UnaryOp) and type(node.op) in _UN:
            return _UN[type(node.op)](ev(node.operand))
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id in _FUN and len(node.args) == 1:
            return _FUN[node.func.id](ev(node.args[0]))
        raise QasmError(f"unsupported parameter expression {expr!r}")

    return ev(tree)


_STMT = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_]*)\s*(?:\((.*)\))?\s*(.*)$", re.S)
_ARG = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_]*)\s*(?:\[\s*(\d+)\s*\])?\s*$")

# name -> (number of params, number of qubits, builder)
_GATES = {
    "h": (0, 1, lambda qc, p, q: qc.h(q[0])),
    "x": (0, 1, lambda qc, p, q: qc.x(q[0])),
    "y": (0, 1, lambda qc, p, q: qc.y(q[0])),
    "z": (0, 1, lambda qc, p, q: qc.z(q[0])),
    "s": (0, 1, lambda qc, p, q: qc.p(math.pi / 2, q[0])),
    "sdg": (0, 1, lambda qc, p, q: qc.p(-math.pi / 2, q[0])),
    "t": (0, 1, lambda qc, p, q: qc.p(math.pi / 4, q[0])),
    "tdg": (0, 1, lambda qc, p, q: qc.p(-math.pi / 4, q[0])),
    "rx": (1, 1, lambda qc, p, q: qc.rx(p[0], q[0])),
    "ry": (1, 1, lambda qc, p, q: qc.ry(p[0], q[0])),
    "rz": (1, 1, lambda qc, p, q: qc.rz(p[0], q[0])),
    "p": (1, 1, lambda qc, p, q: qc.p(p[0], q[0])),
    "u1": (1, 1, lambda qc, p, q: qc.p(p[0], q[0])),
    "u2": (2, 1, lambda qc, p, q: qc.u(math.pi / 2, p[0], p[1], q[0])),
    "u": (3, 1, lambda qc, p, q: qc.u(p[0], p[1], p[2], q[0])),
    "u3": (3, 1, lambda qc, p, q: qc.u(p[0], p[1], p[2], q[0])),
    "cx": (0, 2, lambda qc, p, q: qc.cx(q[0], q[1])),
    "cy": (0, 2, lambda qc, p, q: qc.cy(q[0], q[1])),
    "cz": (0, 2, lambda qc, p, q: qc.cz(q[0], q[1])),
    "ch": (0, 2, lambda qc, p, q: qc.ch(q[0], q[1])),
    "cp": (1, 2, lambda qc, p, q: qc.cp(p[0], q[0], q[1])),
    "cu1": (1, 2, lambda qc, p, q: qc.cp(p[0], q[0], q[1])),
    "crx": (1, 2, lambda qc, p, q: qc.crx(p[0], q[0], q[1])),
    "cry": (1, 2, lambda qc, p, q: qc.cry(p[0], q[0], q[1])),
    "crz": (1, 2, lambda qc, p, q: qc.crz(p[0], q[0], q[1])),
    "cu": (3, 2, lambda qc, p, q: qc.cu(p[0], p[1], p[2], q[0], q[1])),
    "cu3": (3, 2, lambda qc, p, q: qc.cu(p[0], p[1], p[2], q[0], q[1])),
    "ccx": (0, 3, lambda qc, p, q: qc.ccx(q[0], q[1], q[2])),
    "swap": (0, 2, lambda qc, p, q: qc.swap(q[0], q[1])),
}


def _statements(source: str) -> List[str]:
    source = re.sub(r"//[^\n]*", "", source)
    return [s.strip() for s in source.split(";") if s.strip()]


def _split_top(s: str) -> List[str]:
    out, depth, cur = [], 0, []
    for ch in s:
        if ch == "," and depth == 0:
            out.append("".join(cur))
            cur = []
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur.append(ch)
    if cur:
        out.append("".join(cur))
    return [x.strip() for x in out if x.strip()]


def loads(source: str, **circuit_kwargs) -> QuantumCircuit:
    """Parse an OpenQASM 2.0 program (openqasm.rs:26-33 `loads`)."""
    stmts = _statements(source)
    if not stmts or not re.match(r"^OPENQASM\s+2(\.\d+)?$", stmts[0]):
        raise QasmError("program must start with 'OPENQASM 2.0;'")
    qregs: Dict[str, int] = {}
    order: List[str] = []
    for s in stmts[1:]:
        m = re.match(r"^qreg\s+([A-Za-z_][A-Za-z0-9_]*)\s*\[\s*(\d+)\s*\]$", s)
        if m:
            if m.group(1) in qregs:
                raise QasmError(f"register {m.group(1)} declared twice")
            qregs[m.group(1)] = int(m.group(2))
            order.append(m.group(1))
    if not order:
        raise QasmError("no qreg declared")
    regs = {name: QuantumRegister(qregs[name]) for name in order}
    qc = QuantumCircuit(*[regs[name] for name in order], **circuit_kwargs)

    def qubits(arg: str) -> List[int]:
        m = _ARG.match(arg)
        if not m or m.group(1) not in regs:
            raise QasmError(f"unknown quantum argument {arg!r}")
        r = regs[m.group(1)]
        if m.group(2) is None:
            return list(r.qubits)
        i = int(m.group(2))
        if i >= len(r):
            raise QasmError(f"index out of range in {arg!r}")
        return [r[i]]

    for s in stmts[1:]:
        head = s.split(None, 1)[0]
        if head in ("qreg", "creg", "include", "barrier"):
            continue
        if head == "measure":
            m = re.match(r"^measure\s+(.+?)\s*->\s*(.+)$", s)
            if not m:
                raise QasmError(f"bad measure statement {s!r}")
            for q in qubits(m.group(1)):
                qc.measure(q)
            continue
        m = _STMT.match(s)
        if not m or m.group(1) not in _GATES:
            raise QasmError(f"unsupported statement {s!r}")
        name, params_s, args_s = m.group(1), m.group(2), m.group(3)
        nparam, nq, build = _GATES[name]
        params = [eval_angle(p) for p in _split_top(params_s)] if params_s is not None else []
        if len(params) != nparam:
            raise QasmError(f"{name} takes {nparam} parameters, got {len(params)}")
        args = [qubits(a) for a in _split_top(args_s)]
        if len(args) != nq:
            raise QasmError(f"{name} takes {nq} qubit arguments, got {len(args)}")
        width = max(len(a) for a in args)
        for a in args:  # register broadcast: every argument is one qubit or the same length
            if len(a) not in (1, width):
                raise QasmError(f"mismatched register sizes in {s!r}")
        for i in range(width):
            build(qc, params, [a[0] if len(a) == 1 else a[i] for a in args])
    return qc


def load(path) -> QuantumCircuit:
    """Parse an OpenQASM 2.0 file (openqasm.rs:13-24 `load`)."""
    return loads(Path(path).read_text())


_ = (nat, Tuple)
