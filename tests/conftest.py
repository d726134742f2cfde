"""Shared fixtures. `gpu` marks tests that need a CUDA GPU (GB300)."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gpu_lib():
    """libfibmd_gpu.so, built in-tree if it is missing or stale."""
    from fib_md_gb300 import build as fbuild
    from fib_md_gb300 import _abi

    fbuild.build()
    return _abi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle_ffi

    return oracle_ffi.lib()
