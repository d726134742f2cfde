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
    s, X, V = _spec_system(precision=precision)
    a = _ctx(s, X, V, precision, graph=True)
    b = _ctx(s, X, V, precision, graph=False)
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


def _energy(g):
    X, V, F = g.download()
    _, u, U = g.si_force_energy()
    mass = g._mass
    return U + 0.5 * np.sum(mass[:, None] * V * V)


@pytest.mark.parametrize("precision", [0, 1])
def test_nve_energy_conservation(gpu_lib, precision):
    """No thermostat, no fixed layers, no ion impact: the velocity-Verlet
    total energy is conserved to a small fraction of the thermal energy."""
    s, X, V = _spec_system(nc=(6, 6, 4), ion_eV=0.0, precision=precision)
    X[-1] = X[-1] + np.array([0.0, 0.0, 30e-10])  # keep the ion away
    g = _ctx(s, X, V, precision)
    g._mass = s.mass
    E0 = _energy(g)
    lt, t, _, _ = g.steps(2, 2000, 0, 0.0, 300.0)
    E1 = _energy(g)
    nsg = s.params.Nsg
    drift_eV_per_atom = abs(E1 - E0) / s.params.ec / nsg
    assert t > 0.5e-12  # dt at its 1 fs cap for thermal speeds
    assert drift_eV_per_atom < 2e-4, drift_eV_per_atom
