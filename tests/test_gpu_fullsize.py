"""The full-size slabs (256,001 atoms: 40x40x20 unit cells and one Ga; and
1,048,577 atoms: 64x64x32 unit cells and one Ga) through properties that do
not depend on size:

* reference mode at 256k against the oracle: neighbour pair sets bit-exact,
  every atom's force within 1e-10 of max(|F_ref,i|, RMS(F_ref)) (the
  small-slab bar), the ion in contact and far above the surface;
* Newton's third law: every pair and angle term adds opposite forces, so the
  force sum over all atoms vanishes up to rounding, at 256k and at 1M: within
  1e-13 of the summed magnitudes in binary64; in mixed precision within 1e-6
  of the largest per-atom force (a centre sums its own terms in binary32
  before its one binary64 atomic, the partners receive each term apart);
* mixed against binary64 forces at 256k, at the small-slab tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_ffi as of

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-10


def _ref_slab_256k(ion_height_A=1.6):
    """The bench slab's lattice in reference mode, 0.08 A of noise, the ion
    ion_height_A above the highest atom (fired)."""
    o, _, _ = of.crystal((40, 40, 20), 1, -2001)
    rs = np.random.default_rng(11)
    nsg = o.p.Nsg
    o.X[:nsg] += rs.normal(scale=0.08e-10, size=(nsg, 3))
    o.X[:nsg] = np.mod(o.X[:nsg] + 2 * np.array(o.p.Lb[:]), np.array(o.p.Lb[:]))
    top = np.argmax(o.X[:nsg, 2])
    o.X[nsg] = o.X[top] + np.array([0.3e-10, 0.2e-10, ion_height_A * 1e-10])
    o.set_impact(1)
    return o


def _maxrel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("ion_height_A", [1.6, 12.0])
def test_ref_parity_256k(gpu_lib, ion_height_A):
    import fib_md_gb300 as fm

    o = _ref_slab_256k(ion_height_A)
    assert o.p.Natm == 256001
    g = fm.FibMD(o.p)
    g.upload(o.X, o.V, o.F, o.Xi, o.mass, o.atype, o.xsides)
    g.set_impact(1)
    o.si_nlist()
    g.si_nlist()
    assert np.array_equal(g.get_pairs(0), o.pairs(0))
    assert np.array_equal(g.get_pairs(1), o.pairs(1))
    Fr = o.si_force()
    F = g.si_force()
    assert of.per_atom_err(F, Fr) < FORCE_RTOL


def _spec_workload(cells, seed, energy_eV, polar_deg, centre):
    import bench

    return bench.make_workload(cells, seed=seed, energy_eV=energy_eV, polar_deg=polar_deg,
                               list_skin_A=0.6, centre=centre)


def _forces(w, precision):
    import bench

    g = bench.make_ctx(w, precision)
    F = g.si_force()
    g.close()
    return F


@pytest.mark.parametrize("size", ["256k", "1M"])
def test_newton_third_law(gpu_lib, size):
    import fib_md_gb300 as fm

    if size == "256k":
        w = _spec_workload((40, 40, 20), 2001, 5000.0, 7.0, False)
    else:
        w = _spec_workload((64, 64, 32), 5001, 30000.0, 0.0, True)
    # the ion is 10 A above the surface: move it into the slab so that it
    # interacts (a close Ga-Si pair through the Moliere term)
    nsg = w["params"].Nsg
    top = np.argmax(w["X"][:nsg, 2])
    w["X"][nsg] = w["X"][top] + np.array([0.4e-10, 0.3e-10, 1.2e-10])
    F = _forces(w, fm.PREC_FP64)
    assert np.isfinite(F).all()
    assert (np.abs(F.sum(axis=0)) <= 1e-13 * np.abs(F).sum(axis=0)).all(), size
    F = _forces(w, fm.PREC_MIXED)
    assert np.isfinite(F).all()
    assert (np.abs(F.sum(axis=0)) <= 1e-6 * np.abs(F).max(axis=0)).all(), size


def test_mixed_vs_fp64_256k(gpu_lib):
    import fib_md_gb300 as fm

    w = _spec_workload((40, 40, 20), 2001, 5000.0, 7.0, False)
    # thermal disorder (0.08 A), as in the small-slab comparison: on the
    # perfect lattice every force is rounding noise
    nsg = w["params"].Nsg
    w["X"][:nsg] += np.random.default_rng(12).normal(scale=0.08e-10, size=(nsg, 3))
    F64 = _forces(w, fm.PREC_FP64)
    F32 = _forces(w, fm.PREC_MIXED)
    rms_rel = np.sqrt(np.mean(np.sum((F32 - F64) ** 2, axis=1))) / np.sqrt(
        np.mean(np.sum(F64 ** 2, axis=1)))
    assert rms_rel < 2e-5, rms_rel
    assert _maxrel(F32, F64) < 1e-4
