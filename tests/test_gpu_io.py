"""writeatoms' columns packed on the device (fibmd_gpu_xyz_frame) against
the same columns from the oracle's spec-mode run of the same steps and from
the downloaded state."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_xyz_frame_matches_downloaded_state(gpu_lib, tmp_path):
    import fib_md_gb300 as fm
    import oracle_ffi as of

    p = fm.params_default()
    p.list_skin = 0.6e-10
    sl = fm.spec_slab((4, 4, 3), seed=3, ion_eV=500.0, polar_deg=5.0, ion_height=3e-10,
                      params=p)
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
    # the oracle's spec mode from the same seeded slab, the same 30 steps
    q = of.params_default()
    q.list_skin = 0.6e-10
    so = of.spec_slab((4, 4, 3), 3, 500.0, 5.0, ion_height=3e-10, params=q)
    o = of.spec_oracle(so)
    for _ in range(30):
        o.spec_step()
    assert abs(o.spec_scalars()["time"] - t) <= 1e-12 * t
    assert np.abs(xyz - o.X * 1e10).max() < 1e-8  # Angstrom
    ke_o = 0.5 * so["mass"] * np.sum(o.V * o.V, axis=1) * 6.252e18
    assert np.allclose(ke, ke_o, rtol=1e-8, atol=1e-12 * ke_o.max())
    o.close()
    with fm.XyzWriter(tmp_path / "f.xyz") as w:
        w.write(t, xyz, sl.atype, ke)
    lines = (tmp_path / "f.xyz").read_text().splitlines()
    assert len(lines) == sl.params.Natm + 2 and lines[-1].split()[3] == "Ga"
