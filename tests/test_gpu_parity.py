"""GPU (sm_103a) path against the CPU oracle, through the C-ABI.

Bars: neighbour lists bit-exact as sorted (i,j) sets (and the connected
triplet set); every atom's force and energy within 1e-10 of the oracle's,
relative to max(|value_i|, RMS over atoms) (oracle_ffi.per_atom_err);
positions within 1e-8 Angstrom after 100 steps of the reference's onestep.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_ffi as of

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-10     # per atom: |F_gpu,i - F_ref,i| / max(|F_ref,i|, RMS(F_ref))
ENERGY_RTOL = 1e-10    # per atom: |u_gpu,i - u_ref,i| / max(|u_ref,i|, RMS(u_ref))
per_atom_err = of.per_atom_err
TRAJ_ATOL_M = 1e-18    # 1e-8 Angstrom


def _slab(nc=(8, 8, 8), sigma_A=0.08, seed=7, fire=True, ion_height_A=1.6, params=None):
    o, rng, Xr = of.crystal(nc, 1, -1001, params=params)
    rs = np.random.default_rng(seed)
    nsg = o.p.Nsg
    o.X[:nsg] += rs.normal(scale=sigma_A * 1e-10, size=(nsg, 3))
    o.X[:nsg] = np.mod(o.X[:nsg] + 2 * np.array(o.p.Lb[:]), np.array(o.p.Lb[:]))
    if fire:
        top = np.argmax(o.X[:nsg, 2])
        o.X[nsg] = o.X[top] + np.array([0.3e-10, 0.2e-10, ion_height_A * 1e-10])
        o.set_impact(1)
    return o


def _gpu(o, impact=None):
    import fib_md_gb300 as fm

    g = fm.FibMD(o.p)
    g.upload(o.X, o.V, o.F, o.Xi, o.mass, o.atype, o.xsides)
    if impact is not None:
        g.set_impact(impact)
    return g


def _maxrel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_lists_bitexact(gpu_lib):
    o = _slab()
    g = _gpu(o, impact=1)
    o.si_nlist()
    g.si_nlist()
    assert np.array_equal(g.get_pairs(0), o.pairs(0))
    mol = o.pairs(1)
    assert len(mol) > 0
    assert np.array_equal(g.get_pairs(1), mol)
    assert np.array_equal(g.get_triplets(), o.triplets())
    info = o.list_info()
    nsw, nmol, ntr = g.list_counts()
    assert (nsw, nmol, ntr) == (info["nbr_cnt_full"], info["nbr_cntlj_full"], info["Nbrs"])


def test_lists_small_boxes(gpu_lib):
    """Axes with 1 or 2 cells have no periodic ghost layers in the reference
    (nlist.f90:53-64); the stencil and the minimum image still agree."""
    for nc in [(1, 1, 2), (2, 2, 2), (3, 1, 2)]:
        o = _slab(nc, sigma_A=0.15, fire=False)
        g = _gpu(o)
        o.si_nlist()
        g.si_nlist()
        assert np.array_equal(g.get_pairs(0), o.pairs(0)), nc
        assert np.array_equal(g.get_triplets(), o.triplets()), nc


@pytest.mark.parametrize("ion_height_A", [1.6, 12.0])
def test_force_and_energy_parity_fp64(gpu_lib, ion_height_A):
    """The ion in contact (its Moliere force ~50 times the thermal SW forces)
    and far above the surface: every atom at its own scale."""
    o = _slab(ion_height_A=ion_height_A)
    g = _gpu(o, impact=1)
    o.si_nlist()
    g.si_nlist()
    Fr = o.si_force()
    Ur, ur = o.si_potential()
    F, u, U = g.si_force_energy()
    assert per_atom_err(F, Fr) < FORCE_RTOL
    assert per_atom_err(u, ur) < ENERGY_RTOL
    assert abs(U - Ur) < 1e-12 * abs(Ur)
    if ion_height_A < 2.0:
        # the fired ion feels the Moliere force
        assert np.abs(Fr[-1]).max() > 0 and _maxrel(F[-1], Fr[-1]) < FORCE_RTOL


def test_unfired_ions_skipped(gpu_lib):
    o = _slab(fire=True)
    o.set_impact(0)  # ion present but not fired
    g = _gpu(o, impact=0)
    o.si_nlist()
    g.si_nlist()
    Fr = o.si_force()
    F = g.si_force()
    assert np.all(Fr[-1] == 0.0) and np.all(F[-1] == 0.0)
    assert per_atom_err(F, Fr) < FORCE_RTOL
    # si_potential still counts the unfired ion's Moliere energy
    Ur, ur = o.si_potential()
    _, u, U = g.si_force_energy()
    assert per_atom_err(u, ur) < ENERGY_RTOL


def _run_both(o, g, whichctrl, nsteps, lt0=0, time0=0.0, temp0=300.0):
    """nsteps of onestep on both sides (GPU through fibmd_gpu_steps, which
    returns early at dump steps)."""
    t_o, T_o = time0, temp0
    for k in range(nsteps):
        t_o, T_o = o.onestep(whichctrl, lt0 + k + 1, t_o, T_o)
    lt, t, T = lt0, time0, temp0
    while lt < lt0 + nsteps:
        lt, t, T, why = g.steps(whichctrl, lt0 + nsteps - lt, lt, t, T)
    return (t_o, T_o), (lt, t, T)


def test_trajectory_100_steps(gpu_lib):
    """An incoming 500 eV Ga 1.6 A above the surface: 100 reference steps
    (Ts = 0.02 fs, lists every 50 steps, edge thermostat, parking)."""
    o = _slab(ion_height_A=2.0)
    nsg = o.p.Nsg
    v = 1663.6334 * np.sqrt(500.0)
    o.V[nsg] = [0.0, 0.0, -v]
    g = _gpu(o, impact=1)
    o.si_nlist()
    g.si_nlist()
    o.F[:] = o.si_force()
    g.si_force()
    (t_o, _), (lt, t, _) = _run_both(o, g, 1, 100)
    X, V, F = g.download()
    assert lt == 100 and t == t_o
    assert np.abs(X - o.X).max() < TRAJ_ATOL_M
    assert _maxrel(V, o.V) < 1e-8
    assert _maxrel(F, o.F) < 1e-8


def test_stale_list_terms(gpu_lib):
    """With lists never rebuilt, a 250 eV recoil runs past the list skin; the
    reference keeps evaluating the angle terms of its build-time connected
    triplets, which the correction pass must reproduce."""
    p = of.params_default()
    p.ntlist_i = 10 ** 9
    p.atlist_i = 10 ** 9
    o = _slab((4, 4, 4), sigma_A=0.02, fire=False, params=p)
    nsg = o.p.Nsg
    c = int(np.argmin(np.linalg.norm(o.X[:nsg] - np.array(o.p.Lb[:]) * [0.5, 0.5, 0.05], axis=1)))
    vdir = np.array([0.3, 0.2, 0.93])
    vdir /= np.linalg.norm(vdir)
    o.V[c] = vdir * np.sqrt(2 * 250.0 * o.p.ec / o.mass[c])
    g = _gpu(o)
    o.si_nlist()
    g.si_nlist()
    o.F[:] = o.si_force()
    g.si_force()
    _run_both(o, g, 2, 400)
    X, V, F = g.download()
    assert np.abs(X - o.X).max() < TRAJ_ATOL_M
    # forces at the final state, both from the stale build-time lists
    Fg = g.si_force()
    Fr = o.si_force()
    assert _maxrel(Fg, Fr) < 1e-9
    stale_terms = g.work_counters()[3]
    assert stale_terms > 0


def test_warmup_loop(gpu_lib):
    """TI(0): global Berendsen (Tau = 1e-14 s) until |T - Ttar| <= Teps."""
    o = _slab((4, 4, 4), fire=False)
    o.set_tau(1e-14)
    g = _gpu(o)
    g.set_tau(1e-14)
    o.si_nlist()
    g.si_nlist()
    o.F[:] = o.si_force()
    g.si_force()
    T0 = g.temperature()
    assert abs(T0 - o.temperature()) < 1e-12 * T0
    n_o, lt_o, t_o, T_o = o.TI(0, 0, 0.0, 0, 0.0, max_steps=60)
    lt, t, T = 0, 0.0, T0
    lt, t, T, why = g.steps(0, 60, lt, t, T)
    assert lt == lt_o and abs(T - T_o) < 1e-10 * T_o
    X, V, _ = g.download()
    assert _maxrel(V, o.V) < 1e-9
    assert np.abs(X - o.X).max() < TRAJ_ATOL_M


def test_regime_switch_and_parking(gpu_lib):
    """calc_atm switches to the slow regime at the first check below
    ke_limit_1; atoms inside the vacuum bands are parked every atlist."""
    p = of.params_default()
    p.dslist_i = 10
    p.atlist_i = 5
    p.ke_limit_1 = 1.0e9
    o = _slab((4, 4, 4), fire=False, params=p)
    nsg = o.p.Nsg
    L3 = o.p.Lb[2]
    free = np.nonzero(o.xsides[:nsg] == 0)[0]  # edge atoms are pinned to Xi
    a, b = int(free[-1]), int(free[-2])
    o.X[a, 2] = 2.0 * L3 / 10  # inside outz(1)..outz(2)
    o.X[b, 2] = 8.0 * L3 / 10  # inside outz(3)..outz(4)
    o.set_impact(1)
    o.set_fast(True)
    g = _gpu(o, impact=1)
    g.ionrun(1)
    o.si_nlist()
    g.si_nlist()
    o.F[:] = o.si_force()
    g.si_force()
    _run_both(o, g, 1, 30)
    Ts, tic = g.regime()
    Ts_o, _, ints = o.regime()
    assert tic == 2 and Ts == Ts_o == o.p.Ts_r and ints[4] == 0
    X, V, F = g.download()
    # parked, then reboxed each step: MOD(X + 2Lb, Lb) moves the last bits
    assert X[a, 2] == o.X[a, 2] and abs(X[a, 2] - o.p.atomz[0] * L3 / 10.0) < 1e-22
    assert X[b, 2] == o.X[b, 2] and abs(X[b, 2] - o.p.atomz[1] * L3 / 10.0) < 1e-22
    assert np.abs(X - o.X).max() < TRAJ_ATOL_M


@pytest.mark.parametrize("stage", [6, 10, 1])
def test_mixed_precision_force_error(gpu_lib, stage):
    """binary32 force arithmetic (reduced units) against the binary64 oracle;
    the 2-body term is analytic in binary32, tabulated in the reference.
    Stages 6 and 10: one thread per centre; 1: eight lanes per centre."""
    o = _slab()
    o.si_nlist()
    Fr = o.si_force()
    p = o.p.copy()
    p.precision = 1
    import fib_md_gb300 as fm

    g = fm.FibMD(p)
    g.set_option("stage", stage)
    g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
    g.set_impact(1)
    g.si_nlist()
    F = g.si_force()
    rms_rel = np.sqrt(np.mean(np.sum((F - Fr) ** 2, axis=1))) / np.sqrt(np.mean(np.sum(Fr ** 2, axis=1)))
    assert rms_rel < 2e-5, rms_rel
    assert _maxrel(F, Fr) < 1e-4


def _compressed_core(scale=0.8, radius_A=6.0):
    """The slab with a compressed core, as in a cascade: displacements from
    the middle of the lattice within radius_A scaled by `scale`. Second
    neighbours move inside the SW cutoff, so the core's centres have ~16
    legs, more than either force kernel stages per thread."""
    o = _slab()
    nsg = o.p.Nsg
    X = o.X[:nsg]
    c = np.median(X, axis=0)
    d = X - c
    sel = np.sqrt(np.sum(d * d, axis=1)) < radius_A * 1e-10
    X[sel] = c + scale * d[sel]
    assert sel.sum() > 20
    return o


def test_group_path_energies(gpu_lib):
    """Mixed precision: forces and per-atom energies of the eight-lanes-per-
    centre path (stage 1) against the one-thread-per-centre path with its
    many-leg kernel (stage 6) on the compressed-core slab: the same terms
    summed in another order, so equal to binary32 rounding."""
    import fib_md_gb300 as fm

    o = _compressed_core()
    p = o.p.copy()
    p.precision = 1
    out = {}
    for stage in (6, 1):
        g = fm.FibMD(p)
        g.set_option("stage", stage)
        g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
        g.set_impact(1)
        g.si_nlist()
        out[stage] = g.si_force_energy()
        g.close()
    (F6, u6, U6), (F1, u1, U1) = out[6], out[1]
    assert np.isfinite(u1).all() and np.abs(u6).max() > 0
    assert _maxrel(F1, F6) < 1e-5
    assert _maxrel(u1, u6) < 1e-5
    assert abs(U1 - U6) < 1e-6 * abs(U6)


@pytest.mark.parametrize("precision,stage", [(0, 6), (1, 6), (1, 10), (1, 1)])
def test_many_leg_centres(gpu_lib, precision, stage):
    """Centres with more legs than the per-thread stage (the many-leg paths:
    the warp-per-centre kernel in binary64, the eight-lane groups of the
    binary32 many-leg kernel; stage 1 takes every centre in eight-lane
    groups) against the binary64 oracle: within 1e-10 in binary64, at the
    crystal test's binary32 tolerances in mixed precision."""
    import fib_md_gb300 as fm

    o = _compressed_core()
    o.si_nlist()
    Fr = o.si_force()
    p = o.p.copy()
    p.precision = precision
    g = fm.FibMD(p)
    g.set_option("stage", stage)
    g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
    g.set_impact(1)
    g.si_nlist()
    F = g.si_force()
    # the many-leg kernel ran (stage 1 has no separate many-leg pass)
    assert (g.work_counters()[5] > 0) == (stage != 1)
    if precision == 0:
        assert per_atom_err(F, Fr) < FORCE_RTOL
    else:
        rms_rel = np.sqrt(np.mean(np.sum((F - Fr) ** 2, axis=1))) / np.sqrt(
            np.mean(np.sum(Fr ** 2, axis=1)))
        assert rms_rel < 2e-5, rms_rel
        assert _maxrel(F, Fr) < 1e-4


def test_block_size_variants(gpu_lib):
    """The tuned atoms-per-block variants compute the same thing: the
    pair-list build in blocks of 64, 128 or 256 gives the oracle's pair
    sets, and the binary32 force kernel in blocks of 64 or 128 gives forces
    equal to binary32 rounding."""
    import fib_md_gb300 as fm

    o = _slab()
    o.si_nlist()
    sw, mol = o.pairs(0), o.pairs(1)
    for bb in (64, 128, 256):
        g = _gpu(o, impact=1)
        g.set_option("build_block", bb)
        g.si_nlist()
        assert np.array_equal(g.get_pairs(0), sw) and np.array_equal(g.get_pairs(1), mol), bb
        g.close()
    p = o.p.copy()
    p.precision = 1
    out = {}
    for fb in (128, 64):
        g = fm.FibMD(p)
        g.set_option("stage", 6)
        g.set_option("force_block", fb)
        g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
        g.set_impact(1)
        g.si_nlist()
        out[fb] = g.si_force()
        assert g.get_option("force_block") == fb
        g.close()
    # each centre's binary32 arithmetic is the same source in either block
    # size; the two instantiations are compiled apart, so the bar is a few
    # binary32 roundings (the mixed path's own error against binary64 is
    # ~1e-6 per atom, test_mixed_precision_force_error)
    assert per_atom_err(out[64], out[128]) < 1e-6


def test_impact_loop_exit(gpu_lib):
    """TI's impact loop (src/timeint.f90:138-147) ends at the first step
    whose start finds time > impact*dti: the GPU's fibmd_gpu_steps (called
    until FIBMD_STOP_DONE, resuming after the dump stops at atm_out steps)
    and the oracle's TI take the same number of steps, end at the same time
    and at the same positions."""
    import fib_md_gb300 as fm

    p = of.params_default()
    p.dti = 1.0e-15  # 50 fast-regime steps of Ts_i = 2e-17 s
    o = _slab((4, 4, 4), ion_height_A=3.0, params=p)
    o.set_fast(True)
    g = _gpu(o, impact=1)
    g.ionrun(1)
    o.si_nlist()
    g.si_nlist()
    o.F[:] = o.si_force()
    g.si_force()
    n_o, lt_o, t_o, _ = o.TI(1, 0, 0.0, 0, 300.0, max_steps=1000)
    lt, t, T, why, calls = 0, 0.0, 300.0, 0, 0
    while not why & fm.STOP_DONE:
        lt, t, T, why = g.steps(1, 1000, lt, t, T)
        calls += 1
        assert calls < 20
    assert 50 <= n_o <= 51 and lt == lt_o == n_o + 1 and t == t_o
    X, _, _ = g.download()
    assert np.abs(X - o.X).max() < TRAJ_ATOL_M
