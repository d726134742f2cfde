"""Build libfibmd_gpu.so (CUDA for sm_103a + the C++ host layer) in-tree.

Each translation unit is compiled in parallel with nvcc; the shared library
lands next to this file. The host side is compiled with -ffp-contract=off so
the binary64 decisions that mirror the reference (radii, cell counts, the
2-body table) round exactly as written.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
HOST = HERE / "host"
BUILD = HERE / "_build"
LIB = HERE / "libfibmd_gpu.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfibmd_gpu.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(HOST.glob("*.cpp"))


def _compile(nvcc: str, src: Path, obj: Path) -> tuple[Path, str]:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
              f"-I{HERE.parent / 'include'}"]
    if src.suffix == ".cu":
        cmd = [nvcc, ARCH, "-lineinfo", "-Xptxas", "-warn-spills", *common, "-c", str(src),
               "-o", str(obj)]
    else:
        cmd = [nvcc, "-x", "c++", *common, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = sources()
    headers = list(CSRC.glob("*.cuh")) + list(HOST.glob("*.h")) + \
        list((HERE.parent / "include").glob("*.h"))
    newest = max(p.stat().st_mtime for p in srcs + headers + [Path(__file__)])
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, nvcc, s, BUILD / (s.stem + ".o")) for s in srcs]
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if verbose and log.strip():
                print(log, file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
