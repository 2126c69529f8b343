"""Builds the oracle (test infrastructure) into oracle/lib/liboracle.so.

Plain C, gcc, OpenMP, no FMA contraction.  Portable (x86_64 and aarch64).
Sources: mlem_oracle.c (the restated MLEM path) and siddon_oracle.c (the
CPU generator of the synthetic matrices).
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRCS = [HERE / "mlem_oracle.c", HERE / "siddon_oracle.c"]
LIB = HERE / "lib" / "liboracle.so"


def build() -> Path:
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if LIB.exists() and all(LIB.stat().st_mtime >= s.stat().st_mtime for s in SRCS + [Path(__file__)]):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", str(tmp), *map(str, SRCS), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build())
