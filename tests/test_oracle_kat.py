"""Known answers that pin the CPU oracle (no GPU).

The reference ships no tests or fixtures and cannot be compiled here, so the
oracle is pinned by answers that follow from the reference's own formulas
and published algorithms: the minimal-standard generator's check value, the
perfect-diamond energy, Newton's third law, F = -dU/dX, and the list rules.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_ffi as of


def test_ran1_minimal_standard_check_value(oracle_lib):
    # Park & Miller (1988): x_10000 = 1043618065 from x_0 = 1. ran1 with
    # seed -1 takes 40 steps to fill its shuffle table, then one per call.
    r = of.OrcRng(-1)
    for _ in range(10000 - 40):
        r()
    assert r.idum == 1043618065


def test_ran1_range_and_shuffle(oracle_lib):
    r = of.OrcRng(-4242)
    v = np.array([r() for _ in range(20000)])
    assert v.min() > 0.0 and v.max() < 1.0
    assert abs(v.mean() - 0.5) < 0.01


def _bulk(nc=(4, 4, 4)):
    o, _, _ = of.crystal(nc, 0, -1001, periodic_z=True)
    return o


def test_perfect_diamond_energy_per_atom(oracle_lib):
    """Each bulk atom has 4 bonds at a*sqrt(3)/4; the angle term vanishes at
    cos = -1/3, so u(i) = 4 * 0.5*eps*A*(B u^-4 - 1) exp(1/(u - a))."""
    o = _bulk()
    p = o.p
    o.si_nlist()
    U, u = o.si_potential()
    nsg = p.Nsg
    ur = 5.431073e-10 * np.sqrt(3.0) / 4.0 / p.sigmaSi
    expect = 4 * 0.5 * p.epsSi * p.A * (p.B * ur ** -4 - 1.0) * np.exp(1.0 / (ur - p.al))
    assert np.allclose(u[:nsg], expect, rtol=1e-9, atol=0)
    # the Stillinger-Weber pair minimum at 2^(1/6) sigma is -eps
    assert abs(expect / p.epsSi + 2.0) < 1e-6
    F = o.si_force()
    assert np.abs(F[:nsg]).max() < 1e-18  # N; bonds are ~1e-9 N


def test_bulk_list_sizes(oracle_lib):
    o = _bulk()
    o.si_nlist()
    info = o.list_info()
    nsg = o.p.Nsg
    assert info["nbr_cnt_full"] == 16 * nsg  # first and second shells inside rc
    assert info["Nbrs"] == 92 * nsg          # connected triplets per atom
    # with Nlj = 0 the reference's MLlj is 0, so its ion-list warning fires
    assert info["overflow"] & 3 == 0 and info["cell_oob"] == 0


def _perturbed_slab(nc=(4, 4, 4), sigma_A=0.08, seed=7, fire_ion=True):
    o, rng, Xr = of.crystal(nc, 1, -1001)
    rs = np.random.default_rng(seed)
    nsg = o.p.Nsg
    o.X[:nsg] += rs.normal(scale=sigma_A * 1e-10, size=(nsg, 3))
    if fire_ion:
        # a fired Ga 1.6 A above a surface atom
        top = np.argmax(o.X[:nsg, 2])
        o.X[nsg] = o.X[top] + np.array([0.3e-10, 0.2e-10, 1.6e-10])
        o.set_impact(1)
    return o


def test_newton_third_law(oracle_lib):
    o = _perturbed_slab()
    o.si_nlist()
    F = o.si_force()
    assert np.abs(F.sum(axis=0)).max() <= 1e-12 * np.abs(F).sum()


def _fd_force(o, i, h=2e-15):
    g = np.zeros(3)
    for d in range(3):
        X = o.X.copy(order="F")
        X[i, d] += h
        Up, _ = o.si_potential(X)
        X[i, d] -= 2 * h
        Um, _ = o.si_potential(X)
        g[d] = -(Up - Um) / (2 * h)
    return g


def test_force_is_minus_energy_gradient(oracle_lib):
    """si_force's 3-body and Moliere terms are the analytic gradient of
    si_potential; the 2-body force comes from the interpolated table, which
    agrees with the analytic derivative to the interpolation error."""
    o = _perturbed_slab()
    o.si_nlist()
    F = o.si_force()
    scale = np.abs(F).max()
    nsg = o.p.Nsg
    for i in [0, 17, 100, nsg - 1, nsg]:  # nsg = the fired ion (Moliere)
        g = _fd_force(o, i)
        assert np.abs(g - F[i]).max() < 2e-6 * scale, (i, g, F[i])


def test_table_matches_analytic_derivative(oracle_lib):
    o = _bulk((2, 2, 2))
    p = o.p
    tab, uabs = o.table()
    du = uabs[2] - uabs[1]

    def dphi(u):
        ex = np.exp(1.0 / (u - p.al))
        return -p.A * ex * ((p.B * u ** -4 - 1.0) / (u - p.al) ** 2 + 4 * p.B * u ** -5)

    i = np.arange(2000, 4300)
    assert np.allclose(tab[i] * du * du, dphi(uabs[i]), rtol=1e-12)
    rs = np.random.default_rng(3)
    for ue in rs.uniform(1.0, 1.79, size=200):
        v = o.itable2bd(ue)
        # 3-point interpolation on du = 4.1e-4: error ~1e-8 relative
        assert abs(v - dphi(ue)) < 1e-7 * max(1.0, abs(dphi(ue)))
    # entries at and beyond 0.999*a are zero
    assert np.all(tab[uabs >= 0.999 * p.al] == 0.0)


def _bruteforce_pairs(o, kind):
    X = o.X
    N = o.N
    Lb = np.array(o.p.Lb[:])
    iLb = 1.0 / Lb
    g = o.geometry()
    out = []
    for i in range(N):
        d = X[i] - X
        n = np.where(d * iLb >= 0, np.floor(d * iLb + 0.5), -np.floor(-d * iLb + 0.5))
        xx = d - n * Lb
        r2 = (xx[:, 0] * xx[:, 0] + xx[:, 1] * xx[:, 1]) + xx[:, 2] * xx[:, 2]
        ion = np.maximum(o.atype[i], o.atype) >= 3
        if kind == 0:
            sel = (~ion) & (r2 < g["rc"] * g["rc"])
        else:
            sel = ion & (r2 < g["rclj"] * g["rclj"])
        sel[i] = False
        for j in np.nonzero(sel)[0]:
            if j > i:
                out.append((i + 1, j + 1))
    return np.array(sorted(out), dtype=np.int32).reshape(-1, 2)


def test_sw_list_matches_bruteforce(oracle_lib):
    """Cells are at least rc wide, so the 27-cell stencil finds every SW pair
    inside rc: the half list equals an all-pairs search."""
    o = _perturbed_slab()
    o.si_nlist()
    assert np.array_equal(o.pairs(0), _bruteforce_pairs(o, 0))


def test_moliere_stencil_quirk(oracle_lib):
    """The Moliere list radius (5.76 A) exceeds the cell width (>= 4.15 A),
    yet the reference scans only the 27 adjacent cells: every listed pair is
    a true pair, and the pairs it misses lie in non-adjacent cells."""
    o = _perturbed_slab((6, 6, 4))
    o.si_nlist()
    got = {tuple(x) for x in o.pairs(1)}
    full = {tuple(x) for x in _bruteforce_pairs(o, 1)}
    assert got <= full
    g = o.geometry()
    Lb = np.array(o.p.Lb[:])
    h = Lb / np.array(g["Nc"])
    for (i, j) in full - got:
        ci = np.floor(o.X[i - 1] / h).astype(int)
        cj = np.floor(o.X[j - 1] / h).astype(int)
        dc = np.abs(ci - cj)
        dc = np.minimum(dc, np.array(g["Nc"]) - dc)
        assert dc.max() >= 2


def test_triplets_are_connected_triples(oracle_lib):
    o = _perturbed_slab()
    o.si_nlist()
    half = o.pairs(0)
    nb = {}
    for i, j in half:
        nb.setdefault(i, set()).add(j)
        nb.setdefault(j, set()).add(i)
    expect = set()
    for c, s in nb.items():
        s = sorted(s)
        for a in range(len(s)):
            for b in range(a + 1, len(s)):
                expect.add(tuple(sorted((c, s[a], s[b]))))
    got = o.triplets()
    assert len(got) == len(expect)
    assert {tuple(t) for t in got} == expect


def test_ti_exit_increments_lt(oracle_lib):
    """TI(1) increments lt before testing time > impact*dti
    (timeint.f90:138-147)."""
    o = _perturbed_slab((2, 2, 2), fire_ion=False)
    o.si_nlist()
    o.F[:] = o.si_force()
    o.set_impact(1)
    o.set_fast(True, False)
    n, lt, t, T = o.TI(1, 0, 2.0e-12, 0, 300.0)  # time already past dti
    assert n == 0 and lt == 1


def test_parking_bands(oracle_lib):
    """frzsptrdatms moves atoms in outz(1..2) to atomz(1), outz(3..4) to
    atomz(2), and stops atoms near atomz/ionz."""
    from oracle_ffi import lib as _lib  # noqa: F401

    o = _perturbed_slab((2, 2, 2), fire_ion=False)
    p = o.p
    L3 = p.Lb[2]
    o.X[0, 2] = 2.0 * L3 / 10
    o.X[1, 2] = 8.0 * L3 / 10
    o.X[2, 2] = 4.6 * L3 / 10
    o.V[:3] = 1000.0
    import ctypes as C
    of.lib().orc_frzsptrdatms.argtypes = [C.c_void_p]
    of.lib().orc_frzsptrdatms(o.h)
    assert o.X[0, 2] == p.atomz[0] * L3 / 10.0
    assert o.X[1, 2] == p.atomz[1] * L3 / 10.0
    assert np.all(o.V[:3] == 0.0)
