"""writeatoms' columns packed on the device (fibmd_gpu_xyz_frame) against
the same columns computed on the host from the downloaded state."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_xyz_frame_matches_downloaded_state(gpu_lib, tmp_path):
    import fib_md_gb300 as fm

    sl = fm.spec_slab((4, 4, 3), seed=3, ion_eV=500.0, polar_deg=5.0, ion_height=3e-10)
    g = fm.FibMD(sl.params)
    g.upload(sl.X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(sl.params.Natm, np.int32))
    g.set_tags(sl.tags)
    g.set_impact(1)
    g.si_nlist()
    g.si_force()
    lt, t, _, _ = g.steps(2, 30, 0, 0.0, 300.0)
    X, V, _ = g.download()
    xyz, ke = g.xyz_frame()
    g.close()
    assert np.array_equal(xyz, X * 1e10)
    ke_host = 0.5 * sl.mass * np.sum(V * V, axis=1) * 6.252e18
    assert np.allclose(ke, ke_host, rtol=1e-14, atol=0.0)
    with fm.XyzWriter(tmp_path / "f.xyz") as w:
        w.write(t, xyz, sl.atype, ke)
    lines = (tmp_path / "f.xyz").read_text().splitlines()
    assert len(lines) == sl.params.Natm + 2 and lines[-1].split()[3] == "Ga"
