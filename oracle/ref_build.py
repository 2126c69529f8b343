"""Compiles the reference's own sources into oracle/_ref/libmlemref.so.

Test infrastructure: the library pins the oracle (mlem_oracle.c) against the
reference itself.  It needs the reference checkout at REF (default
/root/reference) and x86 g++ (sptrans.h includes immintrin.h); it is built
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
REF = Path(os.environ.get("MLEM_REFERENCE", "/root/reference"))
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


if __name__ == "__main__":
    print(build())
