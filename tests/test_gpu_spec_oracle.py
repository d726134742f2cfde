"""Spec mode (variable dt, skin-triggered rebuilds, layer tags, removal) of
the GPU's binary64 path against the oracle's spec mode, through the C-ABI.

Both sides start from the same seeded state (the oracle's own set-up,
oracle_ffi.spec_slab, which equals the GPU package's spec_slab bit for bit)
and run the same step: thermostat scaling of the tagged layer, drift,
pinning of the frozen layers, removal above remove_z (and 10 A below z = 0
with z an open axis), the rebuild test (by default the pair rule: the two
largest displacements since the build reach the skin; or any atom's
reaching half of it), force, kick, and the next
dt = min(1 fs, 0.05 A / max|v|). Bars: positions within 1e-8 A after 100
steps, the dt of every step within 1e-12 relative, the same steps
rebuilding the lists, the same atoms removed; forces per atom within 1e-10
of max(|F_ref,i|, RMS(F_ref)).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_ffi as of

pytestmark = pytest.mark.gpu

TRAJ_ATOL_M = 1e-18   # 1e-8 Angstrom
DT_RTOL = 1e-12
FORCE_RTOL = 1e-10    # per atom, of max(|F_ref,i|, RMS(F_ref))


per_atom_err = of.per_atom_err


def slab_8x8x8(ion_height_A=10.0, skin_A=0.6, cells=(8, 8, 8), seed=1001, eV=500.0, polar=0.0,
            remove_above_A=35.0):
    """The 8x8x8-cell slab (4096 Si + 1 Ga), 500 eV Ga at normal incidence
    ion_height_A above the surface, 300 K Maxwell-Boltzmann velocities,
    bottom 2 (001) planes fixed and the next 4 thermostatted, list skin
    skin_A, binary64."""
    p = of.params_default()
    p.list_skin = skin_A * 1e-10
    p.precision = 0
    return of.spec_slab(cells, seed, eV, polar, ion_height=ion_height_A * 1e-10,
                        remove_above=remove_above_A * 1e-10, params=p)


def gpu_ctx(slab, graph=False, precision=0, rule=1):
    import fib_md_gb300 as fm

    p = slab["params"].copy()
    p.mode = 1
    p.precision = precision
    g = fm.FibMD(p)
    g.upload(slab["X"], slab["V"], None, slab["Xi"], slab["mass"], slab["atype"],
             np.zeros(p.Natm, dtype=np.int32))
    g.set_tags(slab["tags"])
    g.set_impact(1)
    g.set_option("graph", 1 if graph else 0)
    g.set_option("rebuild_rule", rule)
    g.si_nlist()
    g.si_force()
    return g


def step_both(o, g, n):
    """n steps on both sides, one step per call on the GPU: per step the
    simulated time, dt and whether the lists were rebuilt."""
    rb0 = g.work_counters()[4]
    rec_o, rec_g = [], []
    lt, t, T = 0, 0.0, 300.0
    for _ in range(n):
        reb = o.spec_step()
        sc = o.spec_scalars()
        rec_o.append((sc["time"], sc["dt"], int(reb)))
        lt, t, T, _ = g.steps(2, 1, lt, t, T)
        tg, dtg, _ = g.spec_scalars()
        rb = g.work_counters()[4]
        rec_g.append((tg, dtg, int(rb - rb0)))
        rb0 = rb
    return np.array(rec_o), np.array(rec_g)


def check_runs(o, g, rec_o, rec_g):
    assert np.abs(rec_g[:, 1] - rec_o[:, 1]).max() <= DT_RTOL * rec_o[:, 1].max()
    assert np.abs(rec_g[:, 0] - rec_o[:, 0]).max() <= DT_RTOL * rec_o[:, 0].max()
    assert np.array_equal(np.nonzero(rec_g[:, 2])[0], np.nonzero(rec_o[:, 2])[0])
    X, V, _ = g.download()
    dx = np.abs(X - o.X).max()
    assert dx < TRAJ_ATOL_M, dx
    vs = np.abs(o.V).max()
    assert np.abs(V - o.V).max() <= 1e-8 * vs
    assert np.array_equal(g.get_tags(), o.spec_tags())
    return dx


@pytest.mark.parametrize("ion_height_A,rule", [(10.0, 1), (1.5, 1), (1.5, 0)])
def test_spec_trajectory_8x8x8(gpu_lib, ion_height_A, rule):
    """The 8x8x8-cell slab for 100 steps: with the ion 10 A up (the
    approach) and 1.5 A up (the first 100 steps of the cascade), under the
    pair rule and (the cascade) the half-skin rule."""
    slab = slab_8x8x8(ion_height_A=ion_height_A)
    o = of.spec_oracle(slab)
    o.set_rebuild_rule(rule)
    g = gpu_ctx(slab, rule=rule)
    F0 = g.si_force()
    assert per_atom_err(F0, o.F) < FORCE_RTOL
    rec_o, rec_g = step_both(o, g, 100)
    check_runs(o, g, rec_o, rec_g)
    assert rec_o[:, 2].sum() >= 5  # the 0.6 A skin is crossed every few steps
    if ion_height_A < 2.0:
        # the cascade has started: the ion has lost speed to the lattice
        assert rec_o[-1, 1] > 1.05 * rec_o[0, 1]
    # the CUDA-graph step loop runs the same 100 steps
    g2 = gpu_ctx(slab, graph=True, rule=rule)
    lt, t, _, _ = g2.steps(2, 100, 0, 0.0, 300.0)
    X2, _, _ = g2.download()
    assert lt == 100 and abs(t - rec_o[-1, 0]) <= DT_RTOL * rec_o[-1, 0]
    assert np.abs(X2 - o.X).max() < TRAJ_ATOL_M
    # the graph's fused kick-drift decides the rebuilds in its last block
    assert g2.work_counters()[4] == g.work_counters()[4]
    g.close()
    g2.close()
    o.close()


def test_spec_removal_sets(gpu_lib):
    """A surface atom kicked upwards leaves above remove_z and an ion moving
    down leaves 10 A below the lowest plane: the same atoms are removed at
    the same steps, they stay where they left, and the run goes on without
    them."""
    p = of.params_default()
    p.list_skin = 0.5e-10
    slab = of.spec_slab((4, 4, 3), 31, 500.0, 0.0, remove_above=3.0e-10, params=p)
    nsg = slab["params"].Nsg
    X, V = slab["X"], slab["V"]
    top = int(np.argmax(X[:nsg, 2]))
    V[top] = [1.0e3, -2.0e3, 2.2e4]        # ~70 eV upwards: sputtered
    X[nsg] = [0.5 * slab["params"].Lb[0], 0.5 * slab["params"].Lb[1], -3.0e-10]
    V[nsg] = [0.0, 0.0, -3.0e4]            # the ion leaves through the bottom
    o = of.spec_oracle(slab)
    g = gpu_ctx(slab)
    rec_o, rec_g = step_both(o, g, 200)
    check_runs(o, g, rec_o, rec_g)
    sc = o.spec_scalars()
    tags = o.spec_tags()
    assert sc["removed"] >= 1 and sc["ions_removed"] == 1
    assert tags[top] & of.TAG_REMOVED and tags[nsg] & of.TAG_REMOVED
    _, _, removed = g.spec_scalars()
    assert removed == sc["removed"]
    g.close()
    o.close()


@pytest.mark.parametrize("ion", ["contact", "far"])
def test_spec_force_256k(gpu_lib, ion):
    """The 40x40x20-cell slab (256,000 Si + 1 Ga) with thermal noise and
    0.6 A-skin spec-mode lists: binary64 forces per atom within 1e-10 of
    the oracle's, the ion in contact with the surface or far above it; the
    mixed path's error against the oracle stated as RMS and max."""
    p = of.params_default()
    p.list_skin = 0.6e-10
    slab = of.spec_slab((40, 40, 20), 2001, 5000.0, 7.0, params=p)
    nsg = slab["params"].Nsg
    rs = np.random.default_rng(17)
    X = slab["X"]
    X[:nsg] += rs.normal(scale=0.08e-10, size=(nsg, 3))
    top = int(np.argmax(X[:nsg, 2]))
    if ion == "contact":
        X[nsg] = X[top] + np.array([0.3e-10, 0.2e-10, 1.6e-10])
    o = of.spec_oracle(slab)
    Fr = o.F.copy()
    g = gpu_ctx(slab)
    F = g.si_force()
    assert per_atom_err(F, Fr) < FORCE_RTOL
    if ion == "contact":
        assert np.linalg.norm(Fr[nsg]) > 10 * np.sqrt(np.mean(np.sum(Fr * Fr, axis=1)))
    g.close()
    gm = gpu_ctx(slab, precision=1)
    Fm = gm.si_force()
    d = np.linalg.norm(Fm - Fr, axis=1)
    rms = np.sqrt(np.mean(np.sum(Fr * Fr, axis=1)))
    assert np.sqrt(np.mean(d * d)) / rms < 2e-5
    gm.close()
    o.close()


@pytest.mark.parametrize("graph", [False, True])
def test_skin_switch_keeps_trajectory(gpu_lib, graph):
    """The list skin changed in the middle of a run (one of the context's
    candidates, 0.75 x the start): the next step rebuilds the lists with the
    new radius and cell grid, and the trajectory stays the oracle's (which
    keeps the start skin) within 1e-8 A over 100 steps of the cascade."""
    slab = slab_8x8x8(ion_height_A=1.5)
    o = of.spec_oracle(slab)
    g = gpu_ctx(slab, graph=graph)
    assert g.get_option("skin_candidates") == 3 and abs(g.get_option("skin") - 0.6) < 1e-9
    lt, t, T = 0, 0.0, 300.0
    lt, t, T, _ = g.steps(2, 50, lt, t, T)
    g.set_option("skin", 0.45)
    assert abs(g.get_option("skin") - 0.45) < 1e-9 and g.get_option("skin_tune") == 0
    lt, t, T, _ = g.steps(2, 50, lt, t, T)
    for _ in range(100):
        o.spec_step()
    X, _, _ = g.download()
    assert lt == 100 and abs(t - o.spec_scalars()["time"]) <= DT_RTOL * t
    assert np.abs(X - o.X).max() < TRAJ_ATOL_M
    g.close()
    o.close()


def test_skin_tuner_chooses_a_candidate(gpu_lib):
    """A long call (at least 2000 steps) with the skin left to the context
    (list_skin < 0: start 0.6 A) re-times the three candidates and keeps one;
    the run goes on through the trial steps (the step count is the one asked
    for)."""
    p = of.params_default()
    p.list_skin = -1.0
    slab = of.spec_slab((8, 8, 8), 1001, 500.0, 0.0, params=p)
    g = gpu_ctx(slab, graph=True, precision=1)
    assert abs(g.get_option("skin") - 0.6) < 1e-9 and g.get_option("skin_tune") == 1
    lt, t, _, _ = g.steps(2, 2400, 0, 0.0, 300.0)
    assert lt == 2400 and t > 0
    assert min(abs(g.get_option("skin") - s) for s in (0.45, 0.6, 0.81)) < 1e-9
    X, _, _ = g.download()
    assert np.isfinite(X).all()
    g.close()


def test_stored_reactions_match_atomics(gpu_lib):
    """The binary32 path's atomic-free form (option "reactions": each centre
    stores the 3-body reactions on its legs and its own force, and a second
    pass gathers them per atom in binary64) against the binary64-atomic form
    and the oracle. The 256k slab with thermal noise, the ion in contact and
    a compressed knot (the 12 second neighbours of an interior atom pulled
    20 % inwards) whose centres go to the many-leg kernel: per atom within
    1e-6 of the atomic form (the same binary32 terms from another
    instantiation, binary64 sums in another order), the oracle's RMS bar."""
    p = of.params_default()
    p.list_skin = 0.6e-10
    slab = of.spec_slab((40, 40, 20), 2001, 5000.0, 7.0, params=p)
    nsg = slab["params"].Nsg
    rs = np.random.default_rng(23)
    X = slab["X"]
    X[:nsg] += rs.normal(scale=0.08e-10, size=(nsg, 3))
    mid = 0.5 * (X[:nsg].max(axis=0) + X[:nsg].min(axis=0))
    c = int(np.argmin(np.linalg.norm(X[:nsg] - mid, axis=1)))
    d = np.linalg.norm(X[:nsg] - X[c], axis=1)
    shell = np.argsort(d)[5:17]
    X[shell] = X[c] + 0.8 * (X[shell] - X[c])
    top = int(np.argmax(X[:nsg, 2]))
    X[nsg] = X[top] + np.array([0.3e-10, 0.2e-10, 1.6e-10])
    o = of.spec_oracle(slab)
    Fr = o.F.copy()
    F = {}
    for react in (0, 1):
        g = gpu_ctx(slab, precision=1)
        g.set_option("stage", 6)
        g.set_option("force_block", 128)
        g.set_option("reactions", react)
        assert g.get_option("reactions") == react
        F[react] = g.si_force()
        if react:
            assert g.work_counters()[5] >= 1  # many-leg centres took part
        g.close()
    o.close()
    assert per_atom_err(F[1], F[0]) < 1e-6
    rms = np.sqrt(np.mean(np.sum(Fr * Fr, axis=1)))
    d = np.linalg.norm(F[1] - Fr, axis=1)
    assert np.sqrt(np.mean(d * d)) / rms < 2e-5
