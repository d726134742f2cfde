"""The C-ABI library loads, exports every declared entry point, and its
host-side logic agrees with the oracle's restatement (no GPU calls)."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

import oracle_ffi as of

ROOT = Path(__file__).resolve().parents[1]


def _declared(header: Path) -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(fibmd_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(gpu_lib):
    headers = sorted((ROOT / "include").glob("*.h"))
    assert headers
    names = [n for h in headers for n in _declared(h)]
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_params_layout_and_defaults(gpu_lib):
    from fib_md_gb300 import _abi, params_default

    assert gpu_lib.fibmd_gpu_params_size() == C.sizeof(_abi.Params)
    # the oracle harness's own mirror of the struct: the same fields in order
    assert [(n, C.sizeof(t)) for n, t in of.Params._fields_] == \
        [(n, C.sizeof(t)) for n, t in _abi.Params._fields_]
    assert C.sizeof(of.Params) == C.sizeof(_abi.Params)
    a = params_default()
    b = of.params_default()
    for name, _ in _abi.Params._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            assert list(va) == list(vb), name
        else:
            assert va == vb, name


def test_create_without_device_reports_error(gpu_lib):
    """On a machine without a usable device, create fails with a message
    instead of aborting (the product has no CPU fallback)."""
    import fib_md_gb300 as fm

    try:
        import torch

        if torch.cuda.is_available():
            return
    except Exception:
        pass
    s = fm.crystal_system((2, 2, 2), 1, -5)
    try:
        fm.FibMD(s.params)
    except fm.FibmdError as e:
        assert e.code == 2 and "CUDA" in str(e)
    else:
        raise AssertionError("create succeeded without a device")


def test_ran1_host_matches_oracle(gpu_lib):
    from fib_md_gb300 import Ran1

    for seed in (-1, -12345, -987654):
        a, b = Ran1(seed), of.OrcRng(seed)
        va = [a() for _ in range(5000)]
        vb = [b() for _ in range(5000)]
        assert va == vb


def test_initial_state_matches_oracle(gpu_lib):
    import fib_md_gb300 as fm

    for nc, nlj, seed in [((4, 4, 4), 1, -1001), ((3, 5, 2), 7, -77)]:
        s = fm.crystal_system(nc, nlj, seed)
        o, rng, Xr = of.crystal(nc, nlj, seed)
        assert s.params.Natm == o.N
        assert list(s.params.Lb) == list(o.p.Lb)
        assert np.array_equal(s.X, o.X)
        assert np.array_equal(s.Xi, o.Xi)
        assert np.array_equal(s.V, o.V)
        assert np.array_equal(s.mass, o.mass)
        assert np.array_equal(s.atype, o.atype)
        assert np.array_equal(s.xsides, o.xsides)
        assert np.array_equal(s.Xrand, Xr)
        # knock draws the same start point and velocity
        i, x, v = fm.knock(s.params, s.rng, 1, 500.0, 7.0, 30.0, s.Xrand)
        o.knock(rng, 1, 500.0, 7.0, 30.0, Xr)
        assert i == s.params.Nsg + 1
        assert np.array_equal(x, o.X[i - 1]) and np.array_equal(v, o.V[i - 1])


def test_read_siga(gpu_lib, tmp_path):
    import fib_md_gb300 as fm

    src = (ROOT / "tests" / "golden" / "siga_slab8.in").read_text()
    f = tmp_path / "siga.in"
    f.write_text(src)
    p, s = fm.read_siga(str(f))
    assert (s.amorcrys, s.whichic, s.startimpact) == (0, 4, 0)
    assert s.eV == 500.0 and list(s.Nc) == [8, 8, 8] and list(s.Npc) == [1, 1, 1]
    assert p.Nlj == 1 and s.Nt == 2000
    assert p.Ts_i == 2.0e-17 and p.Ts_r == 2.0e-16 and p.Ttar1 == 300.0
    assert (p.ntlist_i, p.ntlist_r, p.atlist_i, p.atlist_r) == (50, 20, 50, 20)
    assert (p.dslist_i, p.dslist_r, p.atm_out_i, p.atm_out_r, p.res_out) == (500, 500, 50, 500, -5000)
    assert list(p.outz) == [1.3, 3.5, 7.5, 9.8] and list(p.atomz) == [4.5, 6.5]
    assert (p.ionz, p.knockz, p.sidewidth, p.dti) == (5.5, 1.25, 1.5, 1e-12)
    assert (s.Nrand, s.fwhm, s.phiz, s.phixy) == (10000, 2.0, 0.0, 0.0)
    assert p.Nsg == 4096 and p.Natm == 4097
    assert abs(p.Lb[0] - 8 * 5.431073e-10) == 0 and abs(p.Lb[2] - 80 * 5.431073e-10) < 1e-25
    # a truncated file is rejected with the missing value named
    f.write_text("\n".join(src.splitlines()[:20]))
    try:
        fm.read_siga(str(f))
    except fm.FibmdError as e:
        assert "cannot read" in str(e)
    else:
        raise AssertionError("truncated siga.in accepted")
