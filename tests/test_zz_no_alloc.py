"""The allocation-free force entry point against the context-based one.

fibmd_gpu_force_noalloc serves hosts that cannot ask the driver for device
memory when they need a force (pool-managed device memory, embedding
runtimes that forbid allocation after start-up, fixed device footprints on a
shared GPU): all of its scratch lives in one fixed array inside the library.
This file is collected last so that a failure here stops a run only after
every other test has run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle_ffi as of

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-10  # the parity tolerance of the binary64 force tests


def _configuration(seed):
    o, _, _ = of.crystal((4, 4, 4), 1, -1001)
    nsg = o.p.Nsg
    rs = np.random.default_rng(seed)
    o.X[:nsg] += rs.normal(scale=0.08e-10, size=(nsg, 3))
    top = int(np.argmax(o.X[:nsg, 2]))
    o.X[nsg] = o.X[top] + np.array([0.3e-10, 0.2e-10, 1.7e-10])
    return o


def _context_force(o):
    import fib_md_gb300 as fm

    g = fm.FibMD(o.p)
    try:
        g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
        g.set_impact(1)
        g.si_nlist()
        return g.si_force()
    finally:
        g.close()


def _noalloc_force(lib, o):
    import torch

    import fib_md_gb300 as fm

    p = fm.md.as_params(o.p)
    X = torch.tensor(np.ascontiguousarray(o.X.T), dtype=torch.float64, device="cuda")  # (3,N)
    t = torch.tensor(np.asarray(o.atype, dtype=np.int32), device="cuda")
    F = torch.zeros((3, o.N), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.fibmd_gpu_force_noalloc(C.byref(p), C.c_void_p(X.data_ptr()),
                                     C.c_void_p(t.data_ptr()), 1, C.c_void_p(F.data_ptr()),
                                     None)
    if rc:
        buf = C.create_string_buffer(512)
        lib.fibmd_gpu_last_error(None, buf, 512)
        raise AssertionError(f"fibmd_gpu_force_noalloc returned {rc}: {buf.value.decode()}")
    return F.cpu().numpy().T


def test_noalloc_force_matches_context_force(gpu_lib):
    # two calls in a row on different configurations: the second must not
    # see the first's lists or counters in the shared scratch array; each
    # result is also held to the oracle's si_force at the per-atom bar
    for seed in (3, 4):
        o = _configuration(seed)
        F_ref = _context_force(o)
        F = _noalloc_force(gpu_lib, o)
        err = of.per_atom_err(F, F_ref)
        assert err < FORCE_RTOL, (seed, err)
        o.set_impact(1)
        o.si_nlist()
        assert of.per_atom_err(F, o.si_force()) < FORCE_RTOL, seed


def test_noalloc_rejects_oversize(gpu_lib):
    import fib_md_gb300 as fm

    o = _configuration(3)
    p = fm.md.as_params(o.p)
    p.Natm = 100000
    rc = gpu_lib.fibmd_gpu_force_noalloc(C.byref(p), C.c_void_p(1), C.c_void_p(1), 1,
                                         C.c_void_p(1), None)
    assert rc == 1
    buf = C.create_string_buffer(512)
    gpu_lib.fibmd_gpu_last_error(None, buf, 512)
    assert b"limit is 8192" in buf.value
