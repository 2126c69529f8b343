"""Compiles the reference's own sources into oracle/_ref/libmlemref.so and
oracle/_ref/mlemref_kernels.cubin.

Test infrastructure: the library pins the oracle (mlem_oracle.c) against the
reference itself.  It needs the reference checkout (the directory named by
the MLEM_REFERENCE environment variable, else a checkout named `reference`
beside this repository) and x86 g++ (sptrans.h includes immintrin.h); it is built
only where the reference is present and never shipped or imported by the
product.  Sources compiled directly from where they lie:
  kernel.cu                                   (as C++, CUDA built-ins emulated
                                               by ref_shim/cuda_runtime.h)
  sptrans.h                                   (included by ref_glue.cpp)
  helper_files_common/csr4matrix.cpp, scannerconfig.cpp, vector3d.cpp
                                              (boost::iterator_facade stand-in
                                               in ref_shim/, -include unistd.h)
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = Path(os.environ["MLEM_REFERENCE"]) if os.environ.get("MLEM_REFERENCE") else HERE.parent.parent / "reference"
OUT = HERE / "_ref" / "libmlemref.so"


def available() -> bool:
    return (REF / "kernel.cu").exists() and (REF / "sptrans.h").exists()


def build() -> Path | None:
    if not available():
        return None
    OUT.parent.mkdir(parents=True, exist_ok=True)
    glue = HERE / "ref_glue.cpp"
    deps = [glue] + list((HERE / "ref_shim").rglob("*.h*"))
    if OUT.exists() and OUT.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return OUT
    hc = REF / "helper_files_common"
    cmd = ["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w",
           "-I", str(HERE / "ref_shim"), "-I", str(REF), "-I", str(hc), "-include", "unistd.h",
           "-x", "c++", str(REF / "kernel.cu"), "-x", "none",
           str(glue), str(hc / "csr4matrix.cpp"), str(hc / "scannerconfig.cpp"), str(hc / "vector3d.cpp"),
           "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return OUT


CUBIN = HERE / "_ref" / "mlemref_kernels.cubin"


def build_cubin() -> Path | None:
    """The reference's kernel.cu, unmodified, compiled for sm_103a as a cubin.

    Device code only, so it also loads on a GPU host of another CPU
    architecture (ref_cuda.py launches its kernels through the driver API)."""
    if not available():
        return None
    CUBIN.parent.mkdir(parents=True, exist_ok=True)
    src = [REF / "kernel.cu", REF / "kernel.cuh"]
    if CUBIN.exists() and CUBIN.stat().st_mtime >= max(p.stat().st_mtime for p in src):
        return CUBIN
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-I", str(REF),
           str(REF / "kernel.cu"), "-o", str(CUBIN)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference cubin build failed:\n{r.stdout}\n{r.stderr}")
    return CUBIN


if __name__ == "__main__":
    print(build(), build_cubin())
