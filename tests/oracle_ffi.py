"""ctypes harness of the CPU oracle (oracle/liboracle_fibmd.so).

Test infrastructure: the oracle is the binary64 restatement of the
reference's Fortran routines that the GPU library is checked against.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from fib_md_gb300._abi import Params  # noqa: E402  (struct layout shared with the header)

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_VP = C.c_void_p

_SIG = {
    "orc_params_default": (None, [C.POINTER(Params)]),
    "orc_create": (_VP, [C.POINTER(Params)]),
    "orc_destroy": (None, [_VP]),
    "orc_arrays": (None, [_VP] + [C.POINTER(_DP)] * 5 + [C.POINTER(_IP)] * 2),
    "orc_set_impact": (None, [_VP, C.c_int]),
    "orc_set_tau": (None, [_VP, C.c_double]),
    "orc_set_fast": (None, [_VP, C.c_int, C.c_int]),
    "orc_regime": (None, [_VP, _DP, _DP, _IP]),
    "orc_list_info": (None, [_VP, C.POINTER(C.c_longlong)]),
    "orc_geometry": (None, [_VP, _DP, _IP]),
    "orc_table": (_DP, [_VP, C.c_int]),
    "orc_si_nlist": (None, [_VP, _DP]),
    "orc_itable2bd": (C.c_double, [_VP, C.c_double]),
    "orc_si_force": (None, [_VP, _DP, _DP]),
    "orc_si_force_omp": (None, [_VP, _DP, _DP, C.c_int]),
    "orc_si_potential": (None, [_VP, _DP, _DP, _DP]),
    "orc_temperature": (C.c_double, [_VP, _DP]),
    "orc_ionrun": (None, [_VP, C.c_int]),
    "orc_onestep": (None, [_VP, C.c_int, C.c_double, C.c_longlong, _DP, _DP, C.c_int]),
    "orc_TI": (C.c_longlong, [_VP, C.c_int, C.c_double, C.c_longlong, _DP,
                              C.POINTER(C.c_longlong), _DP, C.c_longlong, C.c_int]),
    "orc_rng_seed": (None, [_VP, C.c_int]),
    "orc_ran1": (C.c_double, [_VP]),
    "orc_pureepi": (C.c_int, [C.c_int, C.c_int, C.c_int, _DP, _IP, _DP]),
    "orc_initranions": (None, [_VP, C.c_int, C.c_double, C.c_double, _DP]),
    "orc_initIons": (None, [_VP, _VP]),
    "orc_assignmass": (None, [_VP]),
    "orc_randvel": (None, [_VP, _VP, C.c_double]),
    "orc_knock": (None, [_VP, _VP, C.c_int, C.c_double, C.c_double, C.c_double, _DP, C.c_int]),
    "orc_get_pairs": (C.c_longlong, [_VP, C.c_int, _IP, C.c_longlong]),
    "orc_get_triplets": (C.c_longlong, [_VP, _IP, C.c_longlong]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        sys.path.insert(0, str(ROOT / "oracle"))
        from oracle import build as obuild  # type: ignore

        path = obuild.build()
        L = C.CDLL(str(path))
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_DP)


def _ip(a):
    return a.ctypes.data_as(_IP)


def params_default() -> Params:
    p = Params()
    lib().orc_params_default(C.byref(p))
    return p


class OrcRng:
    """ran1 state of the oracle (Park-Miller + Bays-Durham)."""

    def __init__(self, seed: int):
        self.buf = (C.c_int * 34)()
        lib().orc_rng_seed(C.cast(self.buf, _VP), int(seed))

    @property
    def ptr(self):
        return C.cast(self.buf, _VP)

    def __call__(self) -> float:
        return lib().orc_ran1(self.ptr)

    @property
    def idum(self) -> int:
        return self.buf[33]


class Oracle:
    """One oracle system (orc_sys) with numpy views of its state arrays."""

    def __init__(self, params: Params):
        self.p = params.copy()
        self.h = lib().orc_create(C.byref(self.p))
        if not self.h:
            raise RuntimeError("orc_create failed")
        self.N = params.Natm
        ptrs = [_DP() for _ in range(5)] + [_IP() for _ in range(2)]
        lib().orc_arrays(self.h, *[C.byref(x) for x in ptrs])
        N = self.N

        def view(ptr, shape, dtype):
            n = int(np.prod(shape))
            ctype = C.c_double if dtype == np.float64 else C.c_int
            arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,))
            return arr.reshape(shape, order="F") if len(shape) > 1 else arr

        self.X = view(ptrs[0], (N, 3), np.float64)
        self.Xi = view(ptrs[1], (N, 3), np.float64)
        self.V = view(ptrs[2], (N, 3), np.float64)
        self.F = view(ptrs[3], (N, 3), np.float64)
        self.mass = view(ptrs[4], (N,), np.float64)
        self.atype = view(ptrs[5], (N,), np.int32)
        self.xsides = view(ptrs[6], (N,), np.int32)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, X, V, Xi, mass, atype, xsides, F=None):
        self.X[:] = X
        self.V[:] = V
        self.Xi[:] = Xi
        self.mass[:] = mass
        self.atype[:] = atype
        self.xsides[:] = xsides
        self.F[:] = 0.0 if F is None else F

    def set_impact(self, k: int):
        lib().orc_set_impact(self.h, k)

    def set_tau(self, tau: float):
        lib().orc_set_tau(self.h, tau)

    def set_fast(self, fast: bool, slow: bool = False):
        lib().orc_set_fast(self.h, int(fast), int(slow))

    def ionrun(self, tic: int):
        lib().orc_ionrun(self.h, tic)

    def regime(self):
        Ts, Tau = C.c_double(), C.c_double()
        ints = (C.c_int * 5)()
        lib().orc_regime(self.h, C.byref(Ts), C.byref(Tau), ints)
        return Ts.value, Tau.value, list(ints)

    def si_nlist(self, X=None):
        X = self.X if X is None else np.asfortranarray(X)
        lib().orc_si_nlist(self.h, _dp(X))

    def list_info(self):
        out = (C.c_longlong * 6)()
        lib().orc_list_info(self.h, out)
        keys = ["nbr_cnt_full", "nbr_cntlj_full", "Nbrs", "overflow", "cell_oob", "table_err"]
        return dict(zip(keys, list(out)))

    def geometry(self):
        d = (C.c_double * 4)()
        n = (C.c_int * 3)()
        lib().orc_geometry(self.h, d, n)
        return dict(rc=d[0], rclj=d[1], rlj2=d[2], umax=d[3], Nc=list(n))

    def table(self):
        t = lib().orc_table(self.h, 0)
        u = lib().orc_table(self.h, 1)
        n = self.p.Ntable
        return (np.ctypeslib.as_array(t, shape=(n,)).copy(),
                np.ctypeslib.as_array(u, shape=(n,)).copy())

    def itable2bd(self, ue: float) -> float:
        return lib().orc_itable2bd(self.h, ue)

    def si_force(self, X=None, nthreads: int = 0) -> np.ndarray:
        X = self.X if X is None else np.asfortranarray(X)
        F = np.zeros((self.N, 3), order="F")
        if nthreads > 1:
            lib().orc_si_force_omp(self.h, _dp(X), _dp(F), nthreads)
        else:
            lib().orc_si_force(self.h, _dp(X), _dp(F))
        return F

    def si_potential(self, X=None):
        X = self.X if X is None else np.asfortranarray(X)
        U = C.c_double()
        u = np.zeros(self.N)
        lib().orc_si_potential(self.h, _dp(X), C.byref(U), _dp(u))
        return U.value, u

    def temperature(self) -> float:
        return lib().orc_temperature(self.h, _dp(self.V))

    def onestep(self, whichctrl, lt, time, temp, nthreads=0):
        t = C.c_double(time)
        T = C.c_double(temp)
        lib().orc_onestep(self.h, whichctrl, self.p.Ttar1, lt, C.byref(t), C.byref(T), nthreads)
        return t.value, T.value

    def TI(self, whichctrl, Nt, time, lt, temp, max_steps=0, nthreads=0):
        t = C.c_double(time)
        l = C.c_longlong(lt)
        T = C.c_double(temp)
        n = lib().orc_TI(self.h, whichctrl, self.p.Ttar1, Nt, C.byref(t), C.byref(l), C.byref(T),
                         max_steps, nthreads)
        return n, l.value, t.value, T.value

    def pairs(self, kind: int = 0) -> np.ndarray:
        n = lib().orc_get_pairs(self.h, kind, None, 0)
        out = np.zeros((max(n, 1), 2), dtype=np.int32)
        lib().orc_get_pairs(self.h, kind, _ip(out), n)
        return out[:n]

    def triplets(self) -> np.ndarray:
        n = lib().orc_get_triplets(self.h, None, 0)
        out = np.zeros((max(n, 1), 3), dtype=np.int32)
        lib().orc_get_triplets(self.h, _ip(out), n)
        return out[:n]

    def knock(self, rng: OrcRng, knc, eV, phiz, phixy, Xrand):
        Xr = np.asfortranarray(Xrand, dtype=np.float64)
        lib().orc_knock(self.h, rng.ptr, knc, eV, phiz, phixy, _dp(Xr), Xr.shape[0])


def pureepi(nc1, nc2, nc3):
    n = 8 * nc1 * nc2 * nc3
    XX = np.zeros((n, 3), order="F")
    xs = np.zeros(n, dtype=np.int32)
    Lb = np.zeros(3)
    lib().orc_pureepi(nc1, nc2, nc3, _dp(XX), _ip(xs), _dp(Lb))
    return XX, xs, Lb


def crystal(nc=(4, 4, 4), nlj=1, seed=-1001, nrand=10000, fwhm=2.0, Uo=150.0, params=None,
            periodic_z=False):
    """The reference's initial state (pureepi, initranions, initIons,
    assignmass, randvel) from the oracle's restatements."""
    p = params_default() if params is None else params.copy()
    XX, xs, Lb = pureepi(*nc)
    nsg = XX.shape[0]
    p.Nsg, p.Nlj, p.Natm = nsg, nlj, nsg + nlj
    for d in range(3):
        p.Lb[d] = Lb[d]
    if periodic_z:
        p.Lb[2] = Lb[2] / 10.0
    rng = OrcRng(seed)
    Xrand = np.zeros((nrand, 2), order="F")
    lib().orc_initranions(rng.ptr, nrand, fwhm, 4.0 * np.arctan(1.0), _dp(Xrand))
    o = Oracle(p)
    o.X[:nsg] = XX
    o.atype[:nsg] = 1
    lib().orc_initIons(o.h, rng.ptr)
    o.Xi[:] = o.X
    lib().orc_assignmass(o.h)
    lib().orc_randvel(o.h, rng.ptr, Uo)
    o.xsides[:nsg] = xs
    return o, rng, Xrand
