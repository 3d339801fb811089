"""Build the spinoza_gb300 CUDA library in-tree.

Compiles every ``csrc/*.cu`` for sm_103a (GB300) with nvcc, in parallel, and
links ``_native/libspinoza_gb300.so``.  Device code is built with
``--fmad=false`` so that no multiply-add is contracted behind the kernels'
back: every FMA in the library is an explicit ``fma.rn.f64``, placed exactly
where the reference's arithmetic has one.  Host code is built with
``-ffp-contract=off`` for the same reason (GCC contracts by default on Arm).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_native"
BUILD_DIR = PKG / "_build"
LIB_NAME = "libspinoza_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the spinoza_gb300 CUDA library cannot be built")


def nvcc_flags() -> list[str]:
    return ARCH + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "--fmad=false",
        "-Xcompiler",
        "-fPIC,-O2,-ffp-contract=off",
        "-I" + str(PKG.parent / "include"),
    ]


def library_path() -> Path:
    return OUT_DIR / LIB_NAME


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link the library; returns its path.  Incremental."""
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "spinoza_gb300.h"]
    objects = []
    jobs = []
    for src in sources:
        obj = BUILD_DIR / (src.stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *nvcc_flags(), "-c", str(src), "-o", str(obj)])

    def run(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr.strip():
            print(res.stderr, file=sys.stderr)

    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(workers) as ex:
            list(ex.map(run, jobs))
    lib = library_path()
    if force or jobs or _stale(lib, objects):
        run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objects)])
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
