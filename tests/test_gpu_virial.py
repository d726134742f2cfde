"""The virial (fibmd_gpu_virial) against the strain derivative of the
binary64 energy, which the parity tests pin to the oracle: for a uniform
strain h along x, y and z (positions and the periodic box lengths scaled)
and the shears x += h z and y += h z (z is the open axis, so no box change),
W_ab = -dU/dh by central differences with h = 1e-6, within 1e-5 of the
largest diagonal component; the per-atom shares sum to W. Both precisions'
contexts evaluate it the same way (binary64)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _slab():
    import fib_md_gb300 as fm

    p = fm.params_default()
    p.list_skin = 0.6e-10
    sl = fm.spec_slab((4, 4, 3), seed=5, ion_eV=500.0, polar_deg=0.0, ion_height=3e-10,
                      params=p)
    nsg = sl.params.Nsg
    rs = np.random.default_rng(41)
    X = sl.X.copy(order="F")
    X[:nsg] += rs.normal(scale=0.1e-10, size=(nsg, 3))
    top = int(np.argmax(X[:nsg, 2]))
    X[nsg] = X[top] + np.array([0.4e-10, 0.3e-10, 1.7e-10])  # Moliere contact
    return sl, X


def _ctx(sl, X, Lb, precision=0):
    import fib_md_gb300 as fm

    p = sl.params.copy()
    p.precision = precision
    for d in range(3):
        p.Lb[d] = Lb[d]
    g = fm.FibMD(p)
    g.upload(X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(p.Natm, np.int32))
    g.set_tags(sl.tags)
    g.set_impact(1)
    g.si_nlist()
    return g


def _energy(sl, X, Lb):
    g = _ctx(sl, X, Lb)
    U, _ = g.si_potential()
    g.close()
    return U


def _strained(X, Lb, kind, h):
    X2 = X.copy(order="F")
    L2 = list(Lb)
    if kind in (0, 1, 2):
        X2[:, kind] *= 1.0 + h
        if kind < 2:
            L2[kind] *= 1.0 + h
    elif kind == 4:  # x += h z
        X2[:, 0] += h * X[:, 2]
    elif kind == 5:  # y += h z
        X2[:, 1] += h * X[:, 2]
    return X2, L2


@pytest.mark.parametrize("precision", [0, 1])
def test_virial_is_the_strain_derivative(gpu_lib, precision):
    sl, X = _slab()
    Lb = [sl.params.Lb[d] for d in range(3)]
    g = _ctx(sl, X, Lb, precision)
    W, wa = g.virial(per_atom=True)
    g.close()
    h = 1e-6
    scale = np.abs(W[:3]).max()
    assert scale > 0
    for comp in (0, 1, 2, 4, 5):
        Up = _energy(sl, *_strained(X, Lb, comp, h))
        Um = _energy(sl, *_strained(X, Lb, comp, -h))
        dUdh = (Up - Um) / (2 * h)
        assert abs(W[comp] + dUdh) <= 1e-5 * scale, (comp, W[comp], -dUdh)
    assert np.allclose(wa.sum(axis=0), W, rtol=1e-12, atol=1e-12 * scale)
