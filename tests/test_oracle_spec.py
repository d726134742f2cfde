"""The oracle's spec mode on its own (CPU): the set-up, the lists, the step
rule and the integrator, against answers that follow from their
definitions. The GPU's spec mode is checked against this in
test_gpu_spec_oracle.py."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_ffi as of


def _pairs_within(X, Lb, r, sel, keep):
    """Every pair closer than r by the minimum image on all axes, both atoms
    in keep and at least one in sel: sorted 1-based (i, j), i < j."""
    out = []
    idx = np.nonzero(keep)[0]
    for a, i in enumerate(idx):
        js = idx[a + 1:]
        d = X[js] - X[i]
        d -= Lb * np.rint(d / Lb)
        r2 = np.einsum("ij,ij->i", d, d)
        js = js[r2 < r * r]
        js = js[sel[i] | sel[js]]
        out.append(np.stack([np.full(js.size, i), js], axis=1))
    P = np.concatenate(out).astype(np.int32) + 1
    return P[np.lexsort((P[:, 1], P[:, 0]))]


def _small(seed=3, skin_A=0.4, ion_dz_A=1.2, remove_above_A=12.0):
    p = of.params_default()
    p.list_skin = skin_A * 1e-10
    slab = of.spec_slab((5, 5, 3), seed, 800.0, 10.0, remove_above=remove_above_A * 1e-10,
                        params=p)
    nsg = slab["params"].Nsg
    rs = np.random.default_rng(seed)
    slab["X"][:nsg] += rs.normal(scale=0.1e-10, size=(nsg, 3))
    top = int(np.argmax(slab["X"][:nsg, 2]))
    slab["X"][nsg] = slab["X"][top] + np.array([0.5e-10, -0.3e-10, ion_dz_A * 1e-10])
    return slab


def test_spec_slab_matches_host_setup():
    """The oracle's spec set-up draws the same ran1 numbers in the same
    order as the GPU package's (fibmd_host_maxwell and the ion's draws):
    the two states are identical."""
    import fib_md_gb300 as fm

    for cells, seed, eV, th in [((4, 4, 3), 7, 500.0, 5.0), ((6, 5, 4), 3001, 4200.0, 22.0)]:
        a = fm.spec_slab(cells, seed=seed, ion_eV=eV, polar_deg=th)
        b = of.spec_slab(cells, seed, eV, th)
        for k in ("X", "Xi", "V", "mass", "atype", "tags"):
            assert np.array_equal(getattr(a, k), b[k]), k
        assert a.surface_z == b["surface_z"] and a.params.remove_z == b["params"].remove_z


def test_maxwell_boltzmann_velocities():
    """Box-Muller velocities: every component normal with variance kB T / m
    (Kolmogorov-Smirnov), zero net momentum, the temperature of the mobile
    lattice atoms 300 K within its sampling error."""
    from scipy import stats

    slab = of.spec_slab((10, 10, 6), 11, 500.0, 0.0)
    p = slab["params"]
    nsg = p.Nsg
    mobile = (slab["tags"][:nsg] & of.TAG_FROZEN) == 0
    V = slab["V"][:nsg][mobile]
    m = slab["mass"][:nsg][mobile]
    z = (V / np.sqrt(p.kB * 300.0 / m)[:, None]).ravel()
    assert stats.kstest(z, "norm").pvalue > 1e-3
    # the draw itself has zero net momentum (the fixed layers are zeroed after it)
    rng = of.OrcRng(-5)
    mass = slab["mass"][:nsg].copy()
    W = np.zeros((nsg, 3), order="F")
    of.lib().orc_maxwell(rng.ptr, nsg, nsg, of._dp(mass), 300.0, p.kB, of._dp(W))
    P = (mass[:, None] * W).sum(0)
    assert np.abs(P).max() < 1e-12 * (mass[:, None] * np.abs(W)).sum()
    T = (m[:, None] * V * V).sum() / (3 * len(m) * p.kB)
    assert abs(T - 300.0) < 4 * 300.0 * np.sqrt(2.0 / (3 * len(m)))
    assert np.all(slab["V"][:nsg][~mobile] == 0.0)


def test_spec_first_step_and_thermostat_factor():
    """dt = min(dt_max, dx_max / max|v|) over the atoms in the run, and the
    Berendsen factor sqrt(1 + dt/tau (Ttar/T - 1)) of the tagged layer."""
    slab = _small()
    o = of.spec_oracle(slab)
    p = o.p
    V = slab["V"]
    v2 = np.einsum("ij,ij->i", V, V)
    dt = min(p.dt_max, p.dx_max / np.sqrt(v2.max()))
    sc = o.spec_scalars()
    assert sc["dt"] == pytest.approx(dt, rel=1e-15)
    th = (slab["tags"] & of.TAG_THERMO) != 0
    T = (slab["mass"][th] * v2[th]).sum() / 3 / th.sum() / p.kB
    assert sc["thermo_s"] == pytest.approx(np.sqrt(1 + dt / p.tau_spec * (p.Ttar1 / T - 1)),
                                           rel=1e-14)
    o.close()


@pytest.mark.parametrize("ion_dz_A", [1.2, 9.0])
def test_spec_lists_complete(ion_dz_A):
    """Spec-mode lists: every lattice pair within 0.999 a sigma + skin and
    every pair with the ion within 2.5 sigma + skin (also those two cells
    apart, which the reference's 27-cell stencil misses); removed atoms in
    neither."""
    slab = _small(ion_dz_A=ion_dz_A)
    p = slab["params"]
    nsg = p.Nsg
    slab["tags"][5] |= of.TAG_REMOVED
    o = of.spec_oracle(slab)
    Lb = np.array(p.Lb[:])
    sig = max(p.sigmaSi, p.sigmaGe)
    rc = 0.999 * p.al * sig + p.list_skin
    rclj = 2.5 * sig + p.list_skin
    keep = (slab["tags"] & of.TAG_REMOVED) == 0
    lat = np.zeros(p.Natm, bool)
    lat[:nsg] = True
    sw = _pairs_within(slab["X"], Lb, rc, np.ones(p.Natm, bool), keep & lat)
    assert np.array_equal(o.pairs(0), sw)
    ion = slab["atype"] == 3
    mol = _pairs_within(slab["X"], Lb, rclj, ion, keep)
    assert np.array_equal(o.pairs(1), mol)
    assert o.list_info()["nbr_cntlj_full"] == 2 * len(mol)
    if ion_dz_A < 3.0:
        d = slab["X"][mol[:, 1] - 1] - slab["X"][mol[:, 0] - 1]
        d -= Lb * np.rint(d / Lb)
        assert (np.abs(d).max(axis=1) > rc).any()
    o.close()


def test_spec_force_equals_reference_force():
    """With the ion far away, spec lists (cutoff + skin, complete) and the
    reference's lists (listfac 1.1) hold every pair inside the cutoff, so the
    forces agree up to summation order."""
    slab = _small(ion_dz_A=20.0, remove_above_A=40.0)
    o = of.spec_oracle(slab)
    Fs = o.F.copy()
    q = slab["params"].copy()
    q.mode = 0
    r = of.Oracle(q)
    r.load(slab["X"], slab["V"], slab["Xi"], slab["mass"], slab["atype"],
           np.zeros(q.Natm, dtype=np.int32))
    r.set_impact(1)
    r.si_nlist()
    Fr = r.si_force()
    assert np.abs(Fs - Fr).max() <= 1e-13 * np.abs(Fr).max()
    o.close()
    r.close()


def test_spec_step_kinematics():
    """One step of an ion alone far above the slab: x += v dt exactly (no
    force on it); frozen atoms stay at their sites; the time advances by dt;
    an atom tagged removed takes no part (it keeps its position and its
    velocity as given)."""
    slab = _small(ion_dz_A=25.0, remove_above_A=40.0)
    nsg = slab["params"].Nsg
    slab["tags"][7] |= of.TAG_REMOVED
    o = of.spec_oracle(slab)
    x0 = o.X.copy()
    dt = o.spec_scalars()["dt"]
    assert np.all(o.F[nsg] == 0.0)
    o.spec_step()
    v = slab["V"][nsg]
    assert np.allclose(o.X[nsg], x0[nsg] + v * dt, rtol=0, atol=1e-25)
    fr = (slab["tags"] & of.TAG_FROZEN) != 0
    assert np.array_equal(o.X[fr], slab["Xi"][fr])
    assert np.array_equal(o.X[7], x0[7]) and np.array_equal(o.V[7], slab["V"][7])
    assert o.spec_scalars()["time"] == dt
    o.close()


def test_spec_energy_conservation():
    """No thermostat and no fixed layer: the spec-mode velocity Verlet keeps
    the total energy of a 300 K slab over 400 steps (0.4 ps at the 1 fs cap)
    within a small fraction of kT per atom."""
    p = of.params_default()
    p.list_skin = 0.6e-10
    slab = of.spec_slab((5, 5, 4), 5, 0.0, 0.0, ion_height=30e-10, remove_above=60e-10,
                        params=p)
    slab["tags"][:] = 0
    o = of.spec_oracle(slab)

    def energy():
        U, _ = o.si_potential()
        return U + 0.5 * float(np.sum(o.mass[:, None] * o.V * o.V))

    E0 = energy()
    for _ in range(400):
        o.spec_step()
    E1 = energy()
    nsg = o.p.Nsg
    assert o.spec_scalars()["time"] == pytest.approx(400e-15, rel=1e-12)
    assert abs(E1 - E0) / o.p.ec / nsg < 2e-4
    o.close()


def test_pair_rule_keeps_lists_complete():
    """The two rebuild rules on the same 800 eV cascade (100 steps): with
    the pair rule (rebuild once the two largest displacements since the
    build add up to the skin) the lists at every step still hold each
    lattice pair inside the SW cutoff 0.999 a sigma and each ion pair inside
    2.5 sigma at the step's positions; the two runs are the same trajectory
    (only the force sums' order differs with the lists), and the pair rule
    rebuilds less often."""
    slab = _small()
    p = slab["params"]
    nsg = p.Nsg
    Lb = np.array(p.Lb[:])
    sig = max(p.sigmaSi, p.sigmaGe)
    lat = np.zeros(p.Natm, bool)
    lat[:nsg] = True
    ion = slab["atype"] == 3
    runs = {}
    for rule in (0, 1):
        o = of.spec_oracle(slab)
        o.set_rebuild_rule(rule)
        for n in range(100):
            o.spec_step()
            if rule == 1:
                keep = (o.spec_tags() & of.TAG_REMOVED) == 0
                sw = {tuple(q) for q in o.pairs(0)}
                need = _pairs_within(o.X, Lb, 0.999 * p.al * sig, np.ones(p.Natm, bool), keep & lat)
                assert all(tuple(q) in sw for q in need), n
                mol = {tuple(q) for q in o.pairs(1)}
                need = _pairs_within(o.X, Lb, 2.5 * sig, ion, keep)
                assert all(tuple(q) in mol for q in need), n
        runs[rule] = (o.X.copy(), o.spec_scalars()["rebuilds"])
        o.close()
    (X0, rb0), (X1, rb1) = runs[0], runs[1]
    assert np.abs(X1 - X0).max() < 1e-18
    assert 0 < rb1 < rb0
