"""Device-side dose loop: successive impacts injected and run on the GPU
without host round trips must move exactly as the same impacts driven from
the host (set_tags / set_atom / steps)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(d, graph=True):
    import fib_md_gb300 as fm

    sl = d.slab
    g = fm.FibMD(sl.params)
    g.upload(sl.X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(sl.params.Natm, np.int32))
    g.set_tags(sl.tags)
    g.set_impact(len(d.ion_atoms))
    g.set_option("graph", 1 if graph else 0)
    g.si_nlist()
    g.si_force()
    return g


def _dose_slab(n=3):
    import fib_md_gb300 as fm

    p = fm.params_default()
    p.precision = 0
    return fm.dose_slab((4, 4, 3), n, seed=21, ion_eV=300.0, ion_height=3e-10, params=p)


def test_dose_matches_host_driven_impacts(gpu_lib):
    d = _dose_slab(3)
    steps = 60
    g = _ctx(d)
    rm, ir, t, st = g.dose(d.ion_atoms[:2], d.X0[:2], d.V0[:2], steps)
    assert list(st) == [steps, 2 * steps]
    Xd, Vd, _ = g.download()
    g.close()

    h = _ctx(d)
    tags = d.slab.tags.copy()
    lt, tm = 0, 0.0
    for k in range(2):
        a = int(d.ion_atoms[k])
        tags[a - 1] = 0
        h.set_tags(tags)
        h.set_atom(a, d.X0[k], d.V0[k])
        h.si_nlist()  # the new ion joins the lists
        lt, tm, _, _ = h.steps(2, steps, lt, tm, 300.0)
    Xh, Vh, _ = h.download()
    h.close()
    assert abs(t[-1] - tm) <= 1e-12 * tm
    Lb = np.array(d.slab.params.Lb[:])
    dX = Xd - Xh
    dX[:, :2] -= Lb[:2] * np.rint(dX[:, :2] / Lb[:2])
    assert np.abs(dX).max() < 1e-18
    # the third ion was never injected
    last = int(d.ion_atoms[2]) - 1
    assert np.array_equal(Xd[last], d.X0[2]) and np.all(Vd[last] == 0.0)
    # the injected ions hit the surface and are moving
    assert np.all(np.abs(Vd[d.ion_atoms[:2] - 1]).max(axis=1) > 0)


def test_dose_relaxation_and_records(gpu_lib):
    d = _dose_slab(2)
    g = _ctx(d)
    relax = 20e-15
    rm, ir, t, st = g.dose(d.ion_atoms, d.X0, d.V0, 40, relax)
    assert st[0] > 40 and st[1] - st[0] > 40
    g.close()
    assert np.all(np.diff(t) > relax) and t[0] > relax
    assert np.all(np.diff(rm) >= 0) and np.all(rm >= 0) and np.all(ir >= 0)


def test_dose_matches_oracle(gpu_lib):
    """The device dose (binary64) against the oracle running the same
    impacts (inject, cascade steps, relaxation until its end time): the
    same times, positions within 1e-8 A, the same atoms removed."""
    import oracle_ffi as of

    d = _dose_slab(2)
    steps, relax = 60, 15e-15
    g = _ctx(d)
    rm, ir, t, st = g.dose(d.ion_atoms, d.X0, d.V0, steps, relax)
    Xd, _, _ = g.download()
    tags_d = g.get_tags()
    g.close()
    sl = d.slab
    slab = dict(params=sl.params, X=sl.X, V=sl.V, Xi=sl.Xi, mass=sl.mass, atype=sl.atype,
                tags=sl.tags)
    o = of.spec_oracle(slab, impact=len(d.ion_atoms))
    t_o = o.spec_dose(d.ion_atoms, d.X0, d.V0, steps, relax)
    assert np.allclose(t, t_o, rtol=1e-12, atol=0)
    Lb = np.array(sl.params.Lb[:])
    dX = Xd - o.X
    dX[:, :2] -= Lb[:2] * np.rint(dX[:, :2] / Lb[:2])
    assert np.abs(dX).max() < 1e-18
    assert np.array_equal(tags_d, o.spec_tags())
    sc = o.spec_scalars()
    assert rm[-1] == sc["removed"] and ir[-1] == sc["ions_removed"]
    o.close()
