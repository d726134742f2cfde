"""Spec-mode path on the GPU: variable dt, skin-triggered rebuilds, the
CUDA-graph step loop, and energy conservation of both precisions."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KB = 1.381e-23


def _spec_system(nc=(6, 6, 4), seed=5, T=300.0, ion_eV=2000.0, precision=0):
    import fib_md_gb300 as fm

    p = fm.params_default()
    p.mode = fm.MODE_SPEC
    p.precision = precision
    s = fm.crystal_system(nc, 1, -seed, params=p)
    nsg = s.params.Nsg
    rs = np.random.default_rng(seed)
    V = np.zeros_like(s.V)
    V[:nsg] = rs.normal(size=(nsg, 3)) * np.sqrt(KB * T / s.mass[:nsg])[:, None]
    V[:nsg] -= (s.mass[:nsg, None] * V[:nsg]).sum(0) / s.mass[:nsg].sum()
    X = s.X.copy(order="F")
    top = np.argmax(X[:nsg, 2])
    X[nsg] = X[top] + np.array([0.7e-10, 0.4e-10, 4.0e-10])
    V[nsg] = [0.0, 0.0, -np.sqrt(2 * ion_eV * s.params.ec / s.params.massGa)]
    return s, X, V


def _ctx(s, X, V, precision, graph=True):
    import fib_md_gb300 as fm

    p = s.params.copy()
    p.precision = precision
    g = fm.FibMD(p)
    g.upload(X, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
    g.set_tags(np.zeros(p.Natm, dtype=np.uint32))
    g.set_impact(1)
    g.set_option("graph", 1 if graph else 0)
    g.si_nlist()
    g.si_force()
    return g


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_loop_matches_plain_steps(gpu_lib, precision):
    """The same steps as one CUDA graph and launch by launch. The binary32
    force paths that the autotuner chooses between by timing round
    differently (1e-7 per atom), so both contexts keep the default path."""
    s, X, V = _spec_system(precision=precision)
    a = _ctx(s, X, V, precision, graph=True)
    b = _ctx(s, X, V, precision, graph=False)
    for g in (a, b):
        g.set_option("autotune", 0)
    la, ta, _, _ = a.steps(2, 120, 0, 0.0, 300.0)
    lb, tb, _, _ = b.steps(2, 120, 0, 0.0, 300.0)
    Xa, Va, _ = a.download()
    Xb, Vb, _ = b.download()
    assert la == lb == 120
    assert abs(ta - tb) <= 1e-12 * tb
    # identical algorithm; only the order of atomic force sums differs
    assert np.abs(Xa - Xb).max() < 1e-18
    ca, cb = a.work_counters(), b.work_counters()
    assert ca[4] == cb[4] and ca[4] > 1  # same number of skin-triggered rebuilds


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_many_leg_centres(gpu_lib, precision):
    """A compressed knot (the 12 second neighbours of an interior atom pulled
    25 % inwards: 16 legs on its centre, more than either path's stage) that
    flies apart over the run: the CUDA-graph loop with the option heavy_if
    (its many-leg kernel in an IF node that the force kernel opens) runs the
    same steps as the launch-by-launch loop, which launches that kernel
    every step. In
    binary64 to 1e-8 A after 60 steps; in binary32, whose binary64 atomic
    sums of a knot's wide range of terms round in the order they arrive
    (which the knot's chaos amplifies), to 1e-5 A after 10 steps, where
    steps without the knot's 3-body forces would be off by ~1e-4 A."""
    s, X, V = _spec_system(nc=(6, 6, 4), ion_eV=0.0, precision=precision)
    X[-1] = X[-1] + np.array([0.0, 0.0, 30e-10])  # keep the ion away
    nsg = s.params.Nsg
    mid = 0.5 * (X[:nsg].max(axis=0) + X[:nsg].min(axis=0))
    c = int(np.argmin(np.linalg.norm(X[:nsg] - mid, axis=1)))
    d = np.linalg.norm(X[:nsg] - X[c], axis=1)
    shell = np.argsort(d)[5:17]
    X[shell] = X[c] + 0.75 * (X[shell] - X[c])
    a = _ctx(s, X, V, precision, graph=True)
    b = _ctx(s, X, V, precision, graph=False)
    for g in (a, b):
        g.set_option("autotune", 0)
    a.set_option("heavy_if", 1)
    assert a.get_option("heavy_if") == 1
    assert a.work_counters()[5] >= 1  # many-leg centres at the start
    n, tol_x, tol_t = (60, 1e-18, 1e-12) if precision == 0 else (10, 1e-15, 1e-7)
    la, ta, _, _ = a.steps(2, n, 0, 0.0, 300.0)
    lb, tb, _, _ = b.steps(2, n, 0, 0.0, 300.0)
    Xa, _, _ = a.download()
    Xb, _, _ = b.download()
    assert la == lb == n
    assert abs(ta - tb) <= tol_t * tb
    assert np.abs(Xa - Xb).max() < tol_x
    a.close()
    b.close()


def _energy(g):
    X, V, F = g.download()
    _, u, U = g.si_force_energy()
    mass = g._mass
    return U + 0.5 * np.sum(mass[:, None] * V * V)


@pytest.mark.parametrize("precision,reactions", [(0, 0), (1, 0), (1, 1)])
def test_nve_energy_conservation(gpu_lib, precision, reactions):
    """No thermostat, no fixed layers, no ion impact: the velocity-Verlet
    total energy is conserved to a small fraction of the thermal energy (in
    binary32 also with the stored-reaction form of the force, where a
    reaction gathered twice or not at all would break it)."""
    s, X, V = _spec_system(nc=(6, 6, 4), ion_eV=0.0, precision=precision)
    X[-1] = X[-1] + np.array([0.0, 0.0, 30e-10])  # keep the ion away
    g = _ctx(s, X, V, precision)
    if precision:
        g.set_option("reactions", reactions)
    g._mass = s.mass
    E0 = _energy(g)
    lt, t, _, _ = g.steps(2, 2000, 0, 0.0, 300.0)
    E1 = _energy(g)
    nsg = s.params.Nsg
    drift_eV_per_atom = abs(E1 - E0) / s.params.ec / nsg
    assert t > 0.5e-12  # dt at its 1 fs cap for thermal speeds
    assert drift_eV_per_atom < 2e-4, drift_eV_per_atom


@pytest.mark.parametrize("precision", [0, 1])
def test_nve_drift_gate(gpu_lib, precision):
    """The stated NVE bar: the total energy of the spec-mode slab (12x12x8
    unit cells at 300 K, the ion parked outside, thermostat off, the fixed
    layers kept) drifts by at most 1e-5 eV per mobile atom per ps, the
    slope of a line fitted to 11 samples over 2 ps (2000 steps at the 1 fs
    cap), in both precisions."""
    import bench

    w = bench.make_workload((12, 12, 8), list_skin_A=0.6)
    drift = bench.nve_drift(w, precision, steps=2000)
    assert abs(drift) <= 1e-5, drift


def _pairs_within(X, Lb, r, sel):
    """Every pair closer than r by the minimum image in x and y (z open),
    with at least one atom in sel, as get_pairs reports it: (i, j), i < j,
    1-based, sorted."""
    out = []
    for i in range(X.shape[0]):
        d = X[i + 1:] - X[i]
        d[:, :2] -= Lb[:2] * np.rint(d[:, :2] / Lb[:2])
        r2 = np.einsum("ij,ij->i", d, d)
        js = i + 1 + np.nonzero(r2 < r * r)[0]
        js = js[sel[i] | sel[js]]
        out.append(np.stack([np.full(js.size, i), js], axis=1))
    P = np.concatenate(out).astype(np.int32) + 1
    return P[np.lexsort((P[:, 1], P[:, 0]))]


def _spec_params(s, skin_A, remove_above_A):
    p = s.params.copy()
    p.mode = 1
    p.list_skin = skin_A * 1e-10
    nsg = p.Nsg
    p.remove_z = float(s.X[:nsg, 2].max()) + remove_above_A * 1e-10
    return p


@pytest.mark.parametrize("ion_dz_A", [1.2, 9.0])
def test_spec_lists_complete(gpu_lib, ion_dz_A):
    """Spec mode (list skin 0.3 A, cell grid cut at remove_z): the SW list
    holds every Si/Ge pair within 0.999*a*sigma + skin and the Moliere list
    every ion pair within 2.5*sigma + skin, beyond the 27-cell stencil."""
    import fib_md_gb300 as fm

    s, X, V = _spec_system(nc=(6, 6, 4), seed=11)
    rs = np.random.default_rng(3)
    nsg = s.params.Nsg
    X[:nsg] += rs.normal(scale=0.1e-10, size=(nsg, 3))
    top = np.argmax(X[:nsg, 2])
    X[nsg] = X[top] + np.array([0.5e-10, -0.3e-10, ion_dz_A * 1e-10])
    Lb = np.array(s.params.Lb[:])
    X[:, :2] = np.mod(X[:, :2] + 2 * Lb[:2], Lb[:2])  # some atoms sit below z = 0
    assert (X[:, 2] < 0).any()
    p = _spec_params(s, 0.3, 12.0)
    g = fm.FibMD(p)
    g.upload(X, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
    g.set_impact(1)
    g.si_nlist()
    sig = max(p.sigmaSi, p.sigmaGe)
    rc = 0.999 * p.al * sig + p.list_skin
    rclj = 2.5 * sig + p.list_skin
    ion = s.atype == 3
    nsg = p.Nsg
    sw = _pairs_within(X[:nsg], Lb, rc, np.ones(nsg, dtype=bool))
    assert np.array_equal(g.get_pairs(0), sw)
    mol = _pairs_within(X, Lb, rclj, ion)
    assert np.array_equal(g.get_pairs(1), mol)
    if ion_dz_A < 3.0:
        assert len(mol) > 0
        # pairs farther than one cell apart, which a 27-cell scan can miss
        d = X[mol[:, 1] - 1] - X[mol[:, 0] - 1]
        d -= Lb * np.rint(d / Lb)
        assert (np.abs(d).max(axis=1) > rc).any()


def test_spec_compact_grid_trajectory(gpu_lib):
    """The z-limited cell grid gives the same lists, hence the same motion,
    as the full periodic grid. Only the order of the force sums differs, and
    with it, at a threshold crossing, the step of a skin-triggered rebuild
    (which changes no force: both lists are complete)."""
    import fib_md_gb300 as fm

    s, X, V = _spec_system(nc=(6, 6, 4), seed=13, ion_eV=500.0)
    runs = []
    for compact in (True, False):
        p = _spec_params(s, 0.3, 12.0)
        if not compact:
            p.remove_z = -1.0  # no removal height: periodic z, full grid
        g = fm.FibMD(p)
        g.upload(X, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
        g.set_tags(np.zeros(p.Natm, dtype=np.uint32))
        g.set_impact(1)
        g.si_nlist()
        g.si_force()
        lt, t, _, _ = g.steps(2, 150, 0, 0.0, 300.0)
        Xg, Vg, _ = g.download()
        g.si_nlist()
        runs.append((lt, t, Xg, g.work_counters(), g.get_pairs(0), g.get_pairs(1)))
    (la, ta, Xa, ca, swa, ma), (lb, tb, Xb, cb, swb, mb) = runs
    # the periodic run wraps atoms that cross z = 0, the open-z run does not
    Lb = np.array(s.params.Lb[:])
    d = Xa - Xb
    d -= Lb * np.rint(d / Lb)
    dmax = np.abs(d).max()
    assert la == lb == 150 and abs(ta - tb) <= 1e-12 * tb
    assert dmax < 1e-18, dmax
    assert ca[4] > 10 and abs(ca[4] - cb[4]) <= 3, (ca[4], cb[4])
    assert np.array_equal(swa, swb) and np.array_equal(ma, mb) and len(ma) > 0


@pytest.mark.parametrize("mode", [0, 1])
def test_nonfinite_state_is_reported(gpu_lib, mode):
    """A non-finite velocity (a failure made on the host: a NaN uploaded)
    ends the step call with FIBMD_ENAN; a valid upload clears it."""
    import fib_md_gb300 as fm

    s, X, V = _spec_system(nc=(4, 4, 3))
    p = s.params.copy()
    p.mode = mode
    g = fm.FibMD(p)
    Vbad = V.copy()
    Vbad[7, 1] = np.nan
    g.upload(X, Vbad, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
    g.set_impact(1)
    g.si_nlist()
    g.si_force()
    with pytest.raises(fm.FibmdError) as e:
        g.steps(2, 4, 0, 0.0, 300.0)
    assert e.value.code == fm._abi.ENAN
    assert "non-finite" in str(e.value)
    g.upload(X, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
    g.si_nlist()
    g.si_force()
    g.steps(2, 4, 0, 0.0, 300.0)
    g.close()


def test_transmitted_ion_is_removed(gpu_lib):
    """With an open z axis an ion that leaves through the bottom of the slab
    is removed once it is 10 A below the lowest plane (z = 0), as an atom
    above remove_z is: its depth below the surface turns from a number to
    NaN (fibmd_gpu_impact_stats)."""
    import fib_md_gb300 as fm

    s, X, V = _spec_system(nc=(4, 4, 3), seed=21)
    nsg = s.params.Nsg
    p = _spec_params(s, 0.3, 12.0)
    # the ion 2 A below the lowest plane, moving down at 5 km/s: the step is
    # capped at 1 fs, 0.05 A per step, so it passes -10 A after ~160 steps
    X[nsg] = [0.5 * p.Lb[0], 0.5 * p.Lb[1], -2.0e-10]
    V[nsg] = [0.0, 0.0, -5.0e3]
    g = fm.FibMD(p)
    g.upload(X, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
    g.set_impact(1)
    g.si_nlist()
    g.si_force()
    surf = float(X[:nsg, 2].max())
    _, _, depth = g.impact_stats([surf])
    assert np.isfinite(depth[0]) and depth[0] > surf
    g.steps(2, 300, 0, 0.0, 300.0)
    _, _, depth = g.impact_stats([surf])
    assert np.isnan(depth[0])
    Xf, _, _ = g.download()
    assert (Xf[:nsg, 2] > -10e-10).all()  # the lattice stays


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("which", ["lattice", "ion"])
def test_removed_neighbour_exerts_no_force(gpu_lib, precision, which):
    """An atom removed while it is still in its neighbours' lists (tagged
    after the list build) acts on nothing: the other atoms' forces equal
    those with the atom far away before the lists are built. A lattice atom
    inside the slab (SW pairs and angle terms), or the ion next to the
    surface (Moliere pairs)."""
    import fib_md_gb300 as fm

    s, X, V = _spec_system(nc=(4, 4, 3), seed=23)
    nsg = s.params.Nsg
    rs = np.random.default_rng(5)
    X[:nsg] += rs.normal(scale=0.08e-10, size=(nsg, 3))
    p = _spec_params(s, 0.3, 12.0)
    p.precision = precision
    surf = float(X[:nsg, 2].max())
    if which == "lattice":
        mid = np.array([0.5 * p.Lb[0], 0.5 * p.Lb[1], 0.5 * surf])
        k = int(np.argmin(np.sum((X[:nsg] - mid) ** 2, axis=1)))
    else:
        k = nsg
        top = np.argmax(X[:nsg, 2])
        X[k] = X[top] + np.array([0.4e-10, 0.3e-10, 1.4e-10])
    tags = np.zeros(p.Natm, dtype=np.uint32)
    tags[k] = fm.TAG_REMOVED
    forces = []
    for far in (False, True):
        Xc = X.copy(order="F")
        if far:
            Xc[k] = [0.5 * p.Lb[0], 0.5 * p.Lb[1], surf + 10e-10]
        g = fm.FibMD(p)
        g.upload(Xc, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
        g.set_impact(1)
        if far:
            g.set_tags(tags)
        g.si_nlist()
        if not far:
            assert g.list_counts()[0] > 0
            g.set_tags(tags)  # removed after the lists were built
        forces.append(g.si_force())
    keep = np.arange(p.Natm) != k
    FA, FB = forces[0][keep], forces[1][keep]
    tol = 1e-10 if precision == 0 else 1e-5
    assert np.abs(FA - FB).max() <= tol * np.abs(FB).max()
    # and the removed atom did act before its removal
    g = fm.FibMD(p)
    g.upload(X, V, None, s.Xi, s.mass, s.atype, np.zeros_like(s.xsides))
    g.set_impact(1)
    g.si_nlist()
    F0 = g.si_force()[keep]
    assert np.abs(F0 - FB).max() > 1e3 * tol * np.abs(FB).max()


def test_force_stage_switch_and_autotune(gpu_lib):
    """Mixed precision: the binary32 force path (6 or 10 staged legs per
    thread, or 1: eight lanes per centre) changed between graph runs
    recaptures the step graph; the run matches one at a fixed stage (the
    paths differ only in the order of binary32 sums). With autotune on, the
    stage in use is one of the three."""
    s, X, V = _spec_system(precision=1)
    a = _ctx(s, X, V, 1)
    b = _ctx(s, X, V, 1)
    a.set_option("stage", 6)
    b.set_option("stage", 6)
    a.steps(2, 60, 0, 0.0, 300.0)
    b.steps(2, 60, 0, 0.0, 300.0)
    a.set_option("stage", 10)
    assert a.get_option("stage") == 10 and a.get_option("autotune") == 0
    la, ta, _, _ = a.steps(2, 60, 60, 0.0, 300.0)
    a.set_option("stage", 1)
    assert a.get_option("stage") == 1
    la, ta, _, _ = a.steps(2, 60, la, ta, 300.0)
    lb, tb, _, _ = b.steps(2, 60, 60, 0.0, 300.0)
    lb, tb, _, _ = b.steps(2, 60, lb, tb, 300.0)
    assert la == lb == 180
    Xa, _, _ = a.download()
    Xb, _, _ = b.download()
    assert np.isfinite(Xa).all()
    assert np.abs(Xa - Xb).max() < 1e-15  # 1e-5 A after 180 steps of a 2 keV cascade
    c = _ctx(s, X, V, 1)
    c.set_option("autotune", 1)
    c.steps(2, 1200, 0, 0.0, 300.0)  # tunes before each 1000 steps
    assert c.get_option("stage") in (6, 10, 1)
    assert c.get_option("autotune") == 1


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_kick_drift_matches_unfused(gpu_lib, precision):
    """The graph's fused kick + next drift (one persistent kernel with a grid
    barrier) runs the same steps as the unfused graph: positions within
    1e-8 A (the force sums' order differs), the same time and rebuilds,
    across calls of odd and even step counts."""
    s, X, V = _spec_system(precision=precision)
    a = _ctx(s, X, V, precision, graph=True)
    b = _ctx(s, X, V, precision, graph=True)
    b.set_option("fuse", 0)
    # the binary32 force paths the autotuner picks by timing round
    # differently: both keep the default path
    for g in (a, b):
        g.set_option("autotune", 0)
    assert a.get_option("fuse") == 1 and b.get_option("fuse") == 0
    la, ta, lb, tb = 0, 0.0, 0, 0.0
    for n in (120, 37, 60):
        la, ta, _, _ = a.steps(2, n, la, ta, 300.0)
        lb, tb, _, _ = b.steps(2, n, lb, tb, 300.0)
    Xa, _, _ = a.download()
    Xb, _, _ = b.download()
    assert la == lb == 217 and abs(ta - tb) <= 1e-12 * tb
    assert np.abs(Xa - Xb).max() < 1e-18
    assert a.work_counters()[4] == b.work_counters()[4]
    assert np.array_equal(a.get_tags(), b.get_tags())


def test_fused_barrier_timeout_is_reported(gpu_lib):
    """The fused kernel's grid barrier gives up after a bounded wait: with a
    grid larger than the blocks the device holds at once (the kd_grid test
    hook; a 256k-atom slab has more chunks than resident blocks), the
    resident blocks' waits run out, the call returns FIBMD_ETIMEOUT and the
    context stays usable: after a fresh upload it steps normally."""
    import bench
    import fib_md_gb300 as fm

    w = bench.make_workload((40, 40, 20), list_skin_A=0.6)
    g = bench.make_ctx(w, 1)
    resident = int(g.get_option("kd_grid"))
    nchunk = (w["params"].Natm + 255) // 256
    assert 0 < resident < nchunk
    assert g.get_option("fuse") == 0  # more chunks than resident blocks: unfused
    g.set_option("kd_grid", nchunk)
    assert g.get_option("fuse") == 1
    with pytest.raises(fm.FibmdError) as e:
        g.steps(2, 2, 0, 0.0, 300.0)
    assert e.value.code == fm._abi.ETIMEOUT and "grid barrier" in str(e.value)
    g.set_option("kd_grid", 0)
    g.set_option("fuse", 1)
    bench.fresh_state(g, w)
    lt, t, _, _ = g.steps(2, 20, 0, 0.0, 300.0)
    X, _, _ = g.download()
    assert lt == 20 and t > 0 and np.isfinite(X).all()
    g.close()


@pytest.mark.parametrize("path", ["plain", "graph", "fused"])
def test_pair_rule_lists_complete(gpu_lib, path):
    """The pair rule (rebuild once the two largest displacements since the
    build add up to the skin) on a 2 keV cascade, decided launch by launch,
    in the unfused graph's condition kernel and in the fused kick-drift's
    last block: after each of three calls of 40 steps the SW list holds
    every pair inside the cutoff 0.999 a sigma and the Moliere list every
    ion pair inside 2.5 sigma (minimum image in x and y); the run is the
    half-skin rule's (positions within 1e-8 A) with fewer rebuilds."""
    s, X, V = _spec_system(precision=0)
    p = s.params
    sig = max(p.sigmaSi, p.sigmaGe)
    Lb = np.array(p.Lb[:])
    nsg = p.Nsg
    ctxs = {}
    for rule in (1, 0):
        g = _ctx(s, X, V, 0, graph=path != "plain")
        g.set_option("rebuild_rule", rule)
        if path == "graph":
            g.set_option("fuse", 0)
        assert g.get_option("rebuild_rule") == rule
        ctxs[rule] = g
    g = ctxs[1]
    assert g.get_option("fuse") == (1 if path == "fused" else 0) or path == "plain"
    lt = {0: 0, 1: 0}
    t = {0: 0.0, 1: 0.0}
    for call in range(3):
        for rule, c in ctxs.items():
            lt[rule], t[rule], _, _ = c.steps(2, 40, lt[rule], t[rule], 300.0)
        Xg, _, _ = g.download()
        sw = {tuple(q) for q in g.get_pairs(0)}
        mol = {tuple(q) for q in g.get_pairs(1)}
        for a in range(p.Natm - 1):
            d = Xg[a + 1:] - Xg[a]
            d[:, :2] -= Lb[:2] * np.rint(d[:, :2] / Lb[:2])
            r2 = np.einsum("ij,ij->i", d, d)
            if a < nsg:
                close = np.nonzero(r2[: nsg - a - 1] < (0.999 * p.al * sig) ** 2)[0]
                for c in close:
                    assert (a + 1, a + 2 + c) in sw, (call, a, c)
            near = np.nonzero(r2 < (2.5 * sig) ** 2)[0]
            for c in near:
                if a >= nsg or a + 1 + c >= nsg:
                    assert (a + 1, a + 2 + c) in mol, (call, a, c)
    X1, _, _ = ctxs[1].download()
    X0, _, _ = ctxs[0].download()
    assert lt[0] == lt[1] == 120 and abs(t[1] - t[0]) <= 1e-12 * t[0]
    assert np.abs(X1 - X0).max() < 1e-18
    assert 1 < ctxs[1].work_counters()[4] < ctxs[0].work_counters()[4]
    for c in ctxs.values():
        c.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_pdl_graph_matches_plain_launches(gpu_lib, precision):
    """The unfused step graph with programmatic dependent launches (option
    "pdl") runs the same steps as the same graph with plain launches."""
    s, X, V = _spec_system(precision=precision)
    a = _ctx(s, X, V, precision)
    b = _ctx(s, X, V, precision)
    for g in (a, b):
        g.set_option("fuse", 0)
        g.set_option("autotune", 0)
    a.set_option("pdl", 1)
    assert a.get_option("pdl") == 1 and b.get_option("pdl") == 0
    la, ta, _, _ = a.steps(2, 120, 0, 0.0, 300.0)
    lb, tb, _, _ = b.steps(2, 120, 0, 0.0, 300.0)
    Xa, _, _ = a.download()
    Xb, _, _ = b.download()
    assert la == lb == 120 and abs(ta - tb) <= 1e-12 * tb
    assert np.abs(Xa - Xb).max() < 1e-18
    assert a.work_counters()[4] == b.work_counters()[4]
    a.close()
    b.close()
