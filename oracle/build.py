"""Build the CPU oracle (test infrastructure; never linked into the product).

Compiles fibmd_oracle.c with gcc, OpenMP for the timed CPU baseline, and
-ffp-contract=off so binary64 expressions round in the reference's written
order. Output: oracle/liboracle_fibmd.so (git-ignored).
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "fibmd_oracle.c"
LIB = HERE / "liboracle_fibmd.so"


def build(force: bool = False) -> Path:
    deps = [SRC, HERE / "fibmd_oracle.h", HERE.parent / "include" / "fibmd_gpu.h", Path(__file__)]
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-o", str(tmp), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
