"""The reference's dump files written by the host layer: writeatoms'
extended-xyz frames and snapshot (src/out.f90:62-100) in their fixed-width
Fortran layout, and writerestart's unformatted records (src/out.f90:34-58)
with gfortran's 4-byte length markers."""
from __future__ import annotations

import struct

import numpy as np
import pytest


def test_xyz_frames_layout(gpu_lib, tmp_path):
    import fib_md_gb300 as fm

    xyz = np.array([[1.5, -2.25, 10.0], [123.456789, 0.0, 7.77777], [5.0, 6.0, 7.0]])
    atype = np.array([1, 3, 2], dtype=np.int32)
    ke = np.array([0.0234567, 1234.5, 0.0])
    path, snap = tmp_path / "mdrun2.xyz", tmp_path / "3dmol2.xyz"
    with fm.XyzWriter(path, snap) as w:
        w.write(2.5e-13, xyz, atype, ke)
        w.write(3.0e-12, xyz * 2, atype, ke)
    lines = path.read_text().splitlines()
    assert len(lines) == 2 * 5
    # (I9) and (1A12,F12.5,3A12,2A8,3A16...): the title stops at 'KE (eV)'
    assert lines[0] == "        3"
    assert lines[1] == ("Time (ps) =      0.25000       x (A)       y (A)       z (A)"
                        "    type   proc#         KE (eV)")
    # (3F12.4,A8,I8,1ES14.3)
    assert lines[2] == "      1.5000     -2.2500     10.0000      Si       0     2.346E-02"
    assert lines[3] == "    123.4568      0.0000      7.7778      Ga       0     1.234E+03"
    assert lines[4] == "      5.0000      6.0000      7.0000      Ge       0     0.000E+00"
    assert lines[6].startswith("Time (ps) =      3.00000")
    # the snapshot holds the last frame: (I9), (5A12,F12.5), (A8,3F10.4)
    s = snap.read_text().splitlines()
    assert s[0] == "        3"
    assert s[1] == "        type       x (A)       y (A)       z (A)Time (ps) =      3.00000"
    assert s[2] == "      Si    3.0000   -4.5000   20.0000"
    assert len(s) == 5


def test_restart_records(gpu_lib, tmp_path):
    import fib_md_gb300 as fm

    rs = np.random.default_rng(1)
    n = 7
    X, V = rs.normal(size=(n, 3)), rs.normal(size=(n, 3))
    m = rs.uniform(1, 2, n)
    t = np.array([1, 1, 1, 2, 1, 3, 3], dtype=np.int32)
    p = tmp_path / "restart.in_old"
    fm.write_restart(p, 1234, 5.5e-12, X, V, m, t, 42)
    raw = p.read_bytes()
    # three records, each framed by its byte count
    assert len(raw) == (4 + 12 + 4) + (4 + 60 * n + 4) + (4 + 4 + 4)
    assert struct.unpack_from("<i", raw, 0)[0] == 12
    assert struct.unpack_from("<id", raw, 4) == (1234, 5.5e-12)
    assert struct.unpack_from("<i", raw, 20)[0] == 60 * n
    assert np.array_equal(np.frombuffer(raw, "<f8", 3 * n, 24).reshape(3, n).T, X)
    lt, rt, X2, V2, m2, t2, imp = fm.read_restart(p, n)
    assert (lt, rt, imp) == (1234, 5.5e-12, 42)
    assert np.array_equal(X2, X) and np.array_equal(V2, V) and np.array_equal(m2, m)
    assert np.array_equal(t2, t)
    with pytest.raises(fm.FibmdError):
        fm.read_restart(p, n + 1)
