"""Build recipe of the GB300 MLEM library (no cmake, no torch extension).

Compiles every CUDA translation unit in ``csrc/`` for sm_103a in parallel and
links ``lib/libmlem_gb300.so`` (C ABI of ``include/mlem.h``) and the command
line drop-in ``bin/mlem_gb300``.  Objects go to ``<repo>/_build/mlem``.
Rebuilds only what changed (source, headers or flags).
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = ROOT / "_build" / "mlem"
LIB = PKG / "lib" / "libmlem_gb300.so"
CLI = PKG / "bin" / "mlem_gb300"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-O2",
                     "-I", str(ROOT / "include")]
# the Siddon generator must not contract a*b+c into FMA on the device either,
# so the host and device generators give bit-identical matrices
PER_FILE = {"siddon.cu": ["-fmad=false"]}
UNITS = ["spmv.cu", "spmv_tma.cu", "spmv_fused.cu", "spmv_d16.cu", "spmv_ilv.cu", "merge.cu", "transpose.cu", "siddon.cu", "batch.cu", "runtime.cu",
         "server.cu", "io.cu", "layout.cu", "symmetry.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return "nvcc"


def _digest(unit: str, flags: list[str]) -> str:
    h = hashlib.sha256()
    h.update(" ".join(flags).encode())
    for p in sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "mlem.h", CSRC / unit]:
        h.update(p.read_bytes())
    return h.hexdigest()


def _compile(unit: str, verbose: bool) -> Path:
    flags = NVCC_FLAGS + PER_FILE.get(unit, [])
    obj = OBJ / (unit + ".o")
    stamp = OBJ / (unit + ".sha")
    d = _digest(unit, flags)
    if obj.exists() and stamp.exists() and stamp.read_text() == d:
        return obj
    cmd = [nvcc()] + flags + ["-c", str(CSRC / unit), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    stamp.write_text(d)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles and links the library and the CLI; returns the library path."""
    OBJ.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    CLI.parent.mkdir(parents=True, exist_ok=True)
    jobs = jobs or min(len(UNITS), max(2, os.cpu_count() or 2))
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda u: _compile(u, verbose), UNITS))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + \
              ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = CSRC / "cli_main.cpp"
    if not CLI.exists() or CLI.stat().st_mtime < max(LIB.stat().st_mtime, cli_src.stat().st_mtime):
        cmd = ["g++", "-O2", "-std=c++17", "-o", str(CLI), str(cli_src), "-L", str(LIB.parent),
               "-lmlem_gb300", "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
