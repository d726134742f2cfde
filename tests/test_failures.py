"""Failure detection, made on the host (no GPU fault): capacities forced too
small and parameters the reference would trip over at run time.

The reference prints and carries on at a full list (src/si.f90:264-272) and
at a 2-body table index beyond Ntable (src/si.f90:562-564); here the first
returns FIBMD_EOVERFLOW with the capacity that was needed, and the second is
refused when the context is created (FIBMD_ETABLE), since a list radius
beyond the table is a parameter error."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_ffi as of


def test_list_radius_beyond_table_refused(gpu_lib):
    """A spec-mode list skin so wide that listed pairs lie beyond the table's
    last abscissa: create returns FIBMD_ETABLE before touching a device (so
    this runs without one)."""
    import fib_md_gb300 as fm

    o, _, _ = of.crystal((3, 3, 3), 1, -1001)
    p = fm.md.as_params(o.p)
    p.mode = fm.MODE_SPEC
    p.list_skin = 8.0e-10
    with pytest.raises(fm.FibmdError) as e:
        fm.FibMD(p)
    assert e.value.code == fm._abi.ETABLE
    assert "2-body table" in str(e.value)
    p.list_skin = 0.6e-10  # an ordinary skin passes the check
    try:
        fm.FibMD(p).close()
    except fm.FibmdError as e2:
        assert e2.code == fm._abi.ECUDA  # no device here: the next check


@pytest.mark.gpu
def test_sw_overflow_reports_needed_capacity(gpu_lib):
    """max_sw_nbrs forced below the 16 listed neighbours of a crystal atom:
    the list build returns FIBMD_EOVERFLOW naming the capacity and the 16
    needed; a context re-created with room builds the oracle's lists."""
    import fib_md_gb300 as fm

    o, _, _ = of.crystal((4, 4, 4), 1, -1001)
    p = fm.md.as_params(o.p)
    p.max_sw_nbrs = 10
    g = fm.FibMD(p)
    g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
    with pytest.raises(fm.FibmdError) as e:
        g.si_nlist()
    assert e.value.code == fm._abi.EOVERFLOW
    assert "capacity 10, needed 16" in str(e.value)
    g.close()
    p.max_sw_nbrs = 16
    g = fm.FibMD(p)
    g.upload(o.X, o.V, None, o.Xi, o.mass, o.atype, o.xsides)
    g.si_nlist()
    o.si_nlist()
    assert np.array_equal(g.get_pairs(0), o.pairs(0))
    g.close()
