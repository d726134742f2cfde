"""Batched ensemble: replicas of different boxes advanced in one context
must move as the same replicas run one by one (same algorithm; only the
order of the force sums differs): positions within 1e-6 A after 120 steps
of 300-1500 eV cascades."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPLICAS = [((4, 4, 3), 31, 800.0, 10.0), ((5, 4, 3), 32, 400.0, 25.0), ((3, 5, 3), 33, 1500.0, 0.0)]


def _slabs(precision):
    import fib_md_gb300 as fm

    p = fm.params_default()
    p.precision = precision
    return [fm.spec_slab(c, seed, eV, th, params=p, ion_height=4e-10)
            for c, seed, eV, th in REPLICAS]


def _single(sl, steps):
    import fib_md_gb300 as fm

    g = fm.FibMD(sl.params)
    g.upload(sl.X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(sl.params.Natm, np.int32))
    g.set_tags(sl.tags)
    g.set_impact(1)
    g.si_nlist()
    g.si_force()
    lt, t, _, _ = g.steps(2, steps, 0, 0.0, 300.0)
    X, V, _ = g.download()
    g.close()
    return X, V, t


def _batch(slabs, steps, rule=None):
    import fib_md_gb300 as fm

    reps = [(s.params.Natm, s.params.Nsg, list(s.params.Lb), s.params.remove_z) for s in slabs]
    b = fm.FibMDBatch(slabs[0].params, reps)
    if rule is not None:
        b.set_option("rebuild_rule", rule)
    X = b.pad([s.X for s in slabs])
    V = b.pad([s.V for s in slabs])
    Xi = b.pad([s.Xi for s in slabs])
    mass = b.pad([s.mass for s in slabs], fill=1.0)
    atype = b.pad([s.atype for s in slabs], fill=1, dtype=np.int32)
    tags = b.pad([s.tags for s in slabs], fill=0, dtype=np.uint32)
    b.upload(X, V, None, Xi, mass, atype, np.zeros(b.N, np.int32))
    b.set_tags(tags)
    b.si_nlist()
    b.si_force()
    b.steps(2, steps, 0, 0.0, 300.0)
    Xb, Vb, _ = b.download()
    t, _, _ = b.scalars()
    return b, Xb, Vb, t, X


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_single_replicas(gpu_lib, precision):
    slabs = _slabs(precision)
    steps = 120
    b, Xb, Vb, tb, X0 = _batch(slabs, steps)
    for r, sl in enumerate(slabs):
        X, V, t = _single(sl, steps)
        rows = b.rows(r)
        # the same arithmetic except the order of the binary64 force sums,
        # whose last-bit differences the cascade amplifies a little
        assert abs(tb[r] - t) <= 1e-10 * t, (r, tb[r], t)
        Lb = np.array(sl.params.Lb[:])
        d = Xb[rows] - X
        d[:, :2] -= Lb[:2] * np.rint(d[:, :2] / Lb[:2])
        assert np.abs(d).max() < 1e-16, (r, np.abs(d).max())
        assert np.abs(Vb[rows] - V).max() <= 1e-7 * np.abs(V).max()
    # replicas advance with their own variable step
    assert len(set(np.round(tb / tb.max(), 12))) > 1
    # padding slots never move
    pad = np.ones(b.N, dtype=bool)
    for r in range(b.nrep):
        pad[b.rows(r)] = False
    assert pad.any() and np.array_equal(Xb[pad], X0[pad])
    b.close()


def test_batch_layout(gpu_lib):
    slabs = _slabs(0)
    import fib_md_gb300 as fm

    reps = [(s.params.Natm, s.params.Nsg, list(s.params.Lb), s.params.remove_z) for s in slabs]
    b = fm.FibMDBatch(slabs[0].params, reps)
    assert b.nrep == 3 and np.all(b.offsets[:-1] % 256 == 0)
    assert np.all(np.diff(b.offsets)[:3] >= b.natm)
    b.close()


def test_impact_stats_on_device(gpu_lib):
    """fibmd_gpu_impact_stats on the final states of a batch after its
    cascades against the oracle's atom-by-atom restatement
    (oracle_ffi.impact_stats) and the host function impact_statistics."""
    import fib_md_gb300 as fm
    import oracle_ffi as of

    slabs = _slabs(1)
    b, Xb, Vb, tb, X0 = _batch(slabs, 300)
    sp, dc, dp = b.impact_stats([s.surface_z for s in slabs])
    for r, s in enumerate(slabs):
        Xr = Xb[b.rows(r)]
        os_, od, odisp = of.impact_stats(Xr, s.Xi, s.atype, list(s.params.Lb), s.surface_z,
                                         s.params.remove_z)
        assert sp[r] == os_ and dc[r] == odisp, (r, sp[r], os_, dc[r], odisp)
        assert (np.isnan(dp[r]) and np.isnan(od)) or abs(dp[r] - od) <= 1e-20
        hs, hd, hdisp = fm.impact_statistics(Xr, s.Xi, s.atype, list(s.params.Lb),
                                             s.surface_z, s.params.remove_z)
        assert (hs, hdisp) == (os_, odisp)
    assert dc.sum() > 0
    b.close()


@pytest.mark.parametrize("rule", [1, 0])
def test_batch_lists_hold_every_pair(gpu_lib, rule):
    """After 150 steps of the three cascades in one batch, whose replicas
    rebuild their SW lists separately (under the pair rule those whose two
    largest displacements reach the skin and those halfway there; under
    the half-skin rule those that moved half the skin and those that moved
    a quarter), every replica's list still holds each pair of its atoms
    inside the SW cutoff 0.999*a*sigma at the current positions (minimum
    image in x and y), and no pair across replicas."""
    slabs = _slabs(1)
    b, Xb, Vb, tb, X0 = _batch(slabs, 150, rule)
    listed = {tuple(p) for p in b.get_pairs(0)}
    tags = b.get_tags()
    lo = [int(b.offsets[r]) for r in range(b.nrep)]
    hi = [int(b.offsets[r] + b.natm[r]) for r in range(b.nrep)]
    for (i, j) in listed:
        ri = next(r for r in range(b.nrep) if lo[r] < i <= hi[r])
        assert lo[ri] < j <= hi[ri], (i, j)
    for r, sl in enumerate(slabs):
        p = sl.params
        rc = 0.999 * p.al * max(p.sigmaSi, p.sigmaGe)
        Lb = np.array(p.Lb[:])
        nsg = p.Nsg
        X = Xb[b.rows(r)][:nsg]
        live = (tags[b.rows(r)][:nsg] & 4) == 0
        need = 0
        for a in range(nsg):
            if not live[a]:
                continue
            d = X[a + 1:] - X[a]
            d[:, :2] -= Lb[:2] * np.rint(d[:, :2] / Lb[:2])
            close = np.nonzero((np.einsum("ij,ij->i", d, d) < rc * rc) & live[a + 1:])[0]
            for c in close:
                need += 1
                assert (lo[r] + a + 1, lo[r] + a + 2 + c) in listed, (r, a, c)
        assert need > nsg  # about 2 bonds per atom in a diamond lattice
    b.close()


def test_batch_pair_rule_fewer_rebuilds(gpu_lib):
    """The same 150 steps of the three cascades under both rules: the same
    motion (binary64: positions within 1e-6 A, the order of the force sums
    aside) with fewer list builds under the pair rule."""
    slabs = _slabs(0)
    runs = {}
    for rule in (1, 0):
        b, Xb, Vb, tb, X0 = _batch(slabs, 150, rule)
        runs[rule] = (Xb, tb, b.work_counters()[4], [b.rows(r) for r in range(b.nrep)])
        b.close()
    (X1, t1, rb1, rows), (X0, t0, rb0, _) = runs[1], runs[0]
    assert np.all(np.abs(t1 - t0) <= 1e-10 * t0)
    for r, sl in enumerate(slabs):
        Lb = np.array(sl.params.Lb[:])
        d = X1[rows[r]] - X0[rows[r]]
        d[:, :2] -= Lb[:2] * np.rint(d[:, :2] / Lb[:2])
        assert np.abs(d).max() < 1e-16, (r, np.abs(d).max())
    assert 1 < rb1 < rb0, (rb1, rb0)
