"""Build recipe of the oracle (test infrastructure only).

Compiles ``oracle/spz_oracle.cpp`` — the CPU restatement of the reference's
gate-application path — into ``oracle/_build/liboracle.so`` with g++.
``-ffp-contract=off`` keeps every a*b+c unfused, as Rust does; std::fma is
called exactly where the reference calls mul_add.  OpenMP parallelises the
pair loops from 15 qubits up (the reference's rayon threshold).

The reference itself (Rust, crates not vendored) cannot be compiled here, so
there is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "spz_oracle.cpp"
OUT = HERE / "_build" / "liboracle.so"


def build(verbose: bool = False) -> Path:
    cxx = shutil.which("g++") or "g++"
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           str(SRC), "-o", str(OUT)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
