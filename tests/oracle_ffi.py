"""ctypes harness of the CPU oracle (oracle/liboracle_fibmd.so).

Test infrastructure: the oracle is the binary64 restatement of the
reference's Fortran routines that the GPU library is checked against.
"""
from __future__ import annotations

import ctypes as C
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

_D = C.c_double
_I = C.c_int


class Params(C.Structure):
    """ctypes mirror of `fibmd_params` (include/fibmd_gpu.h), which the
    oracle takes too. Declared here so that the oracle harness loads nothing
    of the GPU package; tests/test_oracle_kat.py checks it field by field
    against the package's mirror and the library's struct size."""

    _fields_ = [
        ("abi_version", _I), ("mode", _I), ("precision", _I),
        ("Natm", _I), ("Nsg", _I), ("Nlj", _I),
        ("Lb", _D * 3),
        ("A", _D), ("B", _D), ("psi", _D), ("qsi", _D), ("al", _D), ("gamma", _D),
        ("lambdaSi", _D), ("lambdaGe", _D), ("epsSi", _D), ("epsGe", _D),
        ("sigmaSi", _D), ("sigmaGe", _D),
        ("massSi", _D), ("massGe", _D), ("massGa", _D),
        ("ZSi", _D), ("ZGe", _D), ("ZGa", _D),
        ("Amol", _D), ("Bmol", _D), ("Cmol", _D),
        ("alpha_mol", _D), ("beta_mol", _D), ("gamma_mol", _D),
        ("kB", _D), ("eps0", _D), ("ec", _D), ("ao", _D),
        ("listfac", _D), ("Ntable", _I),
        ("Ts_i", _D), ("Ts_r", _D), ("Ttar1", _D), ("ke_limit_1", _D),
        ("Tau_i", _D), ("Tau_r", _D), ("Teps", _D),
        ("ntlist_i", _I), ("ntlist_r", _I), ("atlist_i", _I), ("atlist_r", _I),
        ("dslist_i", _I), ("dslist_r", _I),
        ("atm_out_i", _I), ("atm_out_r", _I), ("res_out", _I),
        ("outz", _D * 4), ("atomz", _D * 2), ("ionz", _D), ("knockz", _D),
        ("sidewidth", _D), ("dti", _D),
        ("dt_max", _D), ("dx_max", _D), ("tau_spec", _D), ("remove_z", _D),
        ("mixed_mol_fp64_r", _D), ("list_skin", _D),
        ("max_sw_nbrs", _I), ("max_mol_pairs", _I), ("reserved", _I * 8),
    ]

    def copy(self) -> "Params":
        q = Params()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(Params))
        return q

    def as_ctype(self, cls):
        """The same bytes as another mirror class of the struct."""
        q = cls()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(cls))
        return q


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
    "orc_spec_init": (None, [_VP, C.POINTER(C.c_uint), C.c_double]),
    "orc_spec_step": (C.c_int, [_VP, C.c_int]),
    "orc_spec_set_rule": (None, [_VP, C.c_int]),
    "orc_spec_scalars": (None, [_VP, _DP]),
    "orc_spec_tags": (C.POINTER(C.c_uint), [_VP]),
    "orc_spec_inject": (None, [_VP, C.c_int, _DP, _DP]),
    "orc_maxwell": (None, [_VP, C.c_int, C.c_int, _DP, C.c_double, C.c_double, _DP]),
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


def per_atom_err(A, B):
    """The parity measure of per-atom forces or energies: the largest
    |A_i - B_i| / max(|B_i|, RMS(B)) over atoms i (vector norms for (N,3)
    forces). Every atom is held to its own scale, and atoms whose reference
    value is near zero (a perfect crystal) to the system's RMS."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    if A.ndim == 1:
        A, B = A[:, None], B[:, None]
    d = np.linalg.norm(A - B, axis=1)
    n = np.linalg.norm(B, axis=1)
    rms = float(np.sqrt(np.mean(n * n)))
    return float(np.max(d / np.maximum(n, max(rms, 1e-300))))


def _ip(a):
    return a.ctypes.data_as(_IP)


def as_params(p) -> Params:
    """A copy of p as this harness's Params (p: any same-layout mirror)."""
    if C.sizeof(type(p)) != C.sizeof(Params):
        raise TypeError(f"{type(p).__name__} is not a fibmd_params mirror")
    q = Params()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(Params))
    return q


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
        self.p = as_params(params)
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

    # ---- spec mode (params.mode == 1)
    def spec_init(self, tags=None, time0: float = 0.0):
        t = None if tags is None else np.ascontiguousarray(tags, dtype=np.uint32)
        lib().orc_spec_init(self.h, None if t is None else t.ctypes.data_as(C.POINTER(C.c_uint)),
                            float(time0))

    def spec_step(self, nthreads: int = 0) -> bool:
        """One spec-mode step; True when it rebuilt the lists."""
        return bool(lib().orc_spec_step(self.h, nthreads))

    def set_rebuild_rule(self, rule: int) -> None:
        """1 (the default): rebuild when the two largest displacements since
        the build reach the skin; 0: when any reaches half the skin."""
        lib().orc_spec_set_rule(self.h, int(rule))

    def spec_scalars(self) -> dict:
        out = (C.c_double * 7)()
        lib().orc_spec_scalars(self.h, out)
        keys = ["time", "dt", "thermo_s", "vmax2", "removed", "ions_removed", "rebuilds"]
        return dict(zip(keys, list(out)))

    def spec_inject(self, i: int, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().orc_spec_inject(self.h, int(i), _dp(x), _dp(v))

    def spec_dose(self, ion_atoms, X0, V0, steps: int, relax_s: float = 0.0, nthreads: int = 0):
        """Successive impacts as the device dose runs them: inject, the
        cascade's steps (rounded up to even), then step pairs until relax_s
        of simulated time has passed (at least one pair). Returns the
        simulated time after each impact."""
        times = []
        for k, a in enumerate(ion_atoms):
            self.spec_inject(int(a), X0[k], V0[k])
            for _ in range(2 * ((steps + 1) // 2)):
                self.spec_step(nthreads)
            if relax_s > 0.0:
                t_stop = self.spec_scalars()["time"] + relax_s
                while True:
                    self.spec_step(nthreads)
                    self.spec_step(nthreads)
                    if not self.spec_scalars()["time"] < t_stop:
                        break
            times.append(self.spec_scalars()["time"])
        return times

    def spec_tags(self) -> np.ndarray:
        t = lib().orc_spec_tags(self.h)
        return np.ctypeslib.as_array(t, shape=(self.N,)).copy()

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
    p = params_default() if params is None else as_params(params)
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


A_LATTICE = 5.431073e-10
TAG_FROZEN, TAG_THERMO, TAG_REMOVED = 1, 2, 4


def spec_slab(cells, seed: int, ion_eV: float, polar_deg: float, T: float = 300.0,
              ion_height: float = 10e-10, remove_above: float = 35e-10, fixed_layers: int = 2,
              thermo_layers: int = 4, params=None, azimuth=None, impact_xy=None) -> dict:
    """The spec-mode impact set-up from the oracle's restatements alone: the
    reference's crystal (pureepi, initranions, initIons, assignmass, randvel
    with ran1 seed -|seed|-1), Maxwell-Boltzmann velocities continuing that
    ran1 stream (orc_maxwell), the bottom fixed_layers (001) planes frozen
    and the next thermo_layers thermostatted, and the ion ion_height above
    the top plane at a ran1 azimuth and point (or the given ones), moving
    polar_deg off the inward normal with ion_eV. The same draws in the same
    order as the GPU package's spec_slab."""
    p = params_default() if params is None else as_params(params)
    p.mode = 1
    o, rng, _ = crystal(tuple(cells), 1, -abs(int(seed)) - 1, params=p)
    q = o.p.copy()
    N, nsg = q.Natm, q.Nsg
    mass = o.mass.copy()
    V = np.zeros((N, 3), order="F")
    lib().orc_maxwell(rng.ptr, nsg, N, _dp(mass), float(T), q.kB, _dp(V))
    X = o.X.copy(order="F")
    Xi = o.Xi.copy(order="F")
    atype = o.atype.copy()
    o.close()
    z = X[:nsg, 2]
    layer = np.rint(z / (A_LATTICE / 4)).astype(int)
    tags = np.zeros(N, dtype=np.uint32)
    tags[:nsg][layer < fixed_layers] = TAG_FROZEN
    tags[:nsg][(layer >= fixed_layers) & (layer < fixed_layers + thermo_layers)] = TAG_THERMO
    V[:nsg][layer < fixed_layers] = 0.0
    surf = float(z.max())
    az = 2 * np.pi * rng() if azimuth is None else float(azimuth)
    th = np.deg2rad(polar_deg)
    speed = np.sqrt(2 * ion_eV * q.ec / q.massGa)
    if impact_xy is None:
        xr = rng()
        yr = rng()
        xy = (xr * q.Lb[0], yr * q.Lb[1])
    else:
        xy = impact_xy
    X[nsg] = [xy[0], xy[1], surf + ion_height]
    V[nsg] = speed * np.array([np.sin(th) * np.cos(az), np.sin(th) * np.sin(az), -np.cos(th)])
    q.remove_z = surf + remove_above
    return dict(params=q, X=X, Xi=Xi, V=V, mass=mass, atype=atype, tags=tags, surface_z=surf)


def spec_oracle(slab: dict, params=None, impact: int = 1) -> Oracle:
    """An oracle in spec mode holding the slab's state, its lists built and
    its first force evaluated (what a context's upload, set_tags, si_nlist
    and si_force leave)."""
    p = (slab["params"] if params is None else params).copy()
    p.mode = 1
    o = Oracle(p)
    o.load(slab["X"], slab["V"], slab["Xi"], slab["mass"], slab["atype"],
           np.zeros(p.Natm, dtype=np.int32))
    o.set_impact(impact)
    o.spec_init(slab["tags"], 0.0)
    o.si_nlist()
    o.F[:] = o.si_force()
    return o


def impact_stats(X, Xi, atype, Lb, surface_z: float, remove_z: float,
                 displaced_threshold: float = 1.0e-10):
    """The outcome of one impact, restated atom by atom in plain loops as a
    check of the device statistics: (sputtered, ion depth below the surface
    or nan, displaced). Sputtered: lattice atoms (atype < 3) above remove_z,
    the spec-mode counterpart of cntsputter's count of lattice atoms in the
    containment layer (src/temp.f90:69-93). Displaced: lattice atoms below
    remove_z farther than the threshold from their initial site, by the
    minimum image in x and y. Ion depth: the first ion's distance below
    surface_z."""
    n = len(atype)
    sputtered = displaced = 0
    depth = float("nan")
    ion_seen = False
    thr2 = displaced_threshold * displaced_threshold
    for i in range(n):
        t = int(atype[i])
        z = float(X[i][2])
        if t == 3:
            if not ion_seen and z <= surface_z:
                depth = surface_z - z
            ion_seen = True
            continue
        if z > remove_z:
            sputtered += 1
            continue
        r2 = 0.0
        for d in range(3):
            dd = float(X[i][d]) - float(Xi[i][d])
            if d < 2:
                dd -= Lb[d] * round(dd / Lb[d])
            r2 += dd * dd
        if r2 > thr2:
            displaced += 1
    return sputtered, depth, displaced
