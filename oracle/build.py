"""Builds the oracle (test infrastructure) into oracle/lib/liboracle.so.

Plain C, gcc, OpenMP, no FMA contraction.  Portable (x86_64 and aarch64).
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "mlem_oracle.c"
LIB = HERE / "lib" / "liboracle.so"


def build() -> Path:
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", str(LIB), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build())
