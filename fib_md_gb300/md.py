"""Python host interface of the GB300 backend for FIB_MD's per-step hot path.

Method names follow the reference routines the calls replace (si_nlist,
si_force, si_potential, temperature, ionrun, knock, onestep/TI); arrays are
numpy arrays shaped (Natm, 3) like the Fortran X(Natm,3) and are passed to
the library in Fortran (column-major) order. Every call goes to
libfibmd_gpu.so; errors raise FibmdError with the library's message.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import Params, Replica, Rng, Siga


class FibmdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _fortran(a, dtype=np.float64) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def as_params(p) -> Params:
    """A copy of p as this package's Params: p may be any ctypes mirror of
    fibmd_params with the same layout (the oracle harness keeps its own)."""
    if C.sizeof(type(p)) != C.sizeof(Params):
        raise TypeError(f"{type(p).__name__} is not a fibmd_params mirror")
    q = Params()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(Params))
    return q


def params_default() -> Params:
    """prms.f90's constants and the reference's shipped siga.in."""
    p = Params()
    _abi.load().fibmd_gpu_params_default(C.byref(p))
    return p


def read_siga(path: str, p: Params | None = None) -> tuple[Params, Siga]:
    """Read siga.in's 45 values (prms.f90:221-275) into a Params/Siga pair."""
    lib = _abi.load()
    p = params_default() if p is None else as_params(p)
    s = Siga()
    msg = C.create_string_buffer(512)
    rc = lib.fibmd_host_read_siga(str(path).encode(), C.byref(p), C.byref(s), msg, 512)
    if rc:
        raise FibmdError(rc, msg.value.decode())
    return p, s


class Ran1:
    """ran1 (src/ran1.f). A seed <= 0 initialises the shuffle table."""

    def __init__(self, seed: int):
        self.state = Rng()
        _abi.load().fibmd_host_rng_seed(C.byref(self.state), int(seed))

    def __call__(self) -> float:
        return _abi.load().fibmd_host_ran1(C.byref(self.state))


def pureepi(nc1: int, nc2: int, nc3: int):
    """Diamond-cubic slab (prms.f90:484-557): (XX, xsides, Lb)."""
    n = 8 * nc1 * nc2 * nc3
    XX = np.zeros((n, 3), dtype=np.float64, order="F")
    xs = np.zeros(n, dtype=np.int32)
    Lb = np.zeros(3)
    _abi.load().fibmd_host_pureepi(nc1, nc2, nc3, _dp(XX), _ip(xs), _dp(Lb))
    return XX, xs, Lb


@dataclass
class System:
    """Initial state of a reference run, as ic case 4 prepares it."""

    params: Params
    X: np.ndarray
    Xi: np.ndarray
    V: np.ndarray
    mass: np.ndarray
    atype: np.ndarray
    xsides: np.ndarray
    Xrand: np.ndarray
    rng: Ran1


def crystal_system(nc=(8, 8, 8), nlj: int = 1, seed: int = -1001, params: Params | None = None,
                   nrand: int = 10000, fwhm: float = 2.0, Uo: float = 150.0) -> System:
    """readprms/pureepi, initran, initdata (src/main.f90:31-43) for a
    crystalline target with an explicit ran1 seed (the reference seeds from
    the wall clock, prms.f90:220,296)."""
    lib = _abi.load()
    p = params_default() if params is None else as_params(params)
    XX, xs, Lb = pureepi(*nc)
    nsg = XX.shape[0]
    p.Nsg, p.Nlj, p.Natm = nsg, nlj, nsg + nlj
    for d in range(3):
        p.Lb[d] = Lb[d]
    rng = Ran1(seed)
    Xrand = np.zeros((nrand, 2), dtype=np.float64, order="F")
    lib.fibmd_host_initranions(C.byref(rng.state), nrand, fwhm, _dp(Xrand))
    N = p.Natm
    X = np.zeros((N, 3), order="F")
    X[:nsg] = XX
    Xi = np.zeros((N, 3), order="F")
    V = np.zeros((N, 3), order="F")
    mass = np.zeros(N)
    atype = np.zeros(N, dtype=np.int32)
    rc = lib.fibmd_host_init_state(C.byref(p), C.byref(rng.state), Uo, _dp(X), _dp(Xi), _dp(V),
                                   _dp(mass), _ip(atype))
    if rc:
        raise FibmdError(rc, "init_state")
    xsides = np.zeros(N, dtype=np.int32)
    xsides[:nsg] = xs
    return System(p, X, Xi, V, mass, atype, xsides, Xrand, rng)


KB_SI = 1.381e-23
A_LATTICE = 5.431073e-10


@dataclass
class SpecSlab:
    """A spec-mode impact: a (001) Si slab with a free top surface, fixed
    bottom layers, a thermostat layer above them, Maxwell-Boltzmann
    velocities and one Ga ion above the surface moving towards it."""

    params: Params
    X: np.ndarray
    Xi: np.ndarray
    V: np.ndarray
    mass: np.ndarray
    atype: np.ndarray
    tags: np.ndarray
    surface_z: float


def spec_slab(cells, seed: int, ion_eV: float, polar_deg: float, T: float = 300.0,
              ion_height: float = 10e-10, remove_above: float = 35e-10,
              fixed_layers: int = 2, thermo_layers: int = 4, params: Params | None = None,
              azimuth: float | None = None, impact_xy=None) -> SpecSlab:
    """Slab of cells = (nx, ny, nz) unit cells (pureepi lattice, 8 atoms per
    cell) plus one ion. (001) planes are a/4 apart: the lowest fixed_layers
    are frozen (TAG_FROZEN), the next thermo_layers carry the Berendsen
    thermostat (TAG_THERMO). The ion starts ion_height above the top plane
    at a seeded (or given) point, with ion_eV along a direction polar_deg off
    the inward normal at a seeded (or given) azimuth. Atoms higher than
    remove_above over the surface are removed during the run.

    Every random draw continues the ran1 stream of the reference's set-up
    (crystal_system, seed -|seed|-1): Maxwell-Boltzmann velocities by the
    Box-Muller method (fibmd_host_maxwell), then the azimuth and the impact
    point."""
    p = params_default() if params is None else as_params(params)
    p.mode = _abi.MODE_SPEC
    s = crystal_system(tuple(cells), 1, -abs(int(seed)) - 1, params=p)
    p = s.params
    N, nsg = p.Natm, p.Nsg
    V = np.zeros((N, 3), order="F")
    _abi.load().fibmd_host_maxwell(C.byref(s.rng.state), nsg, N, _dp(s.mass), float(T), p.kB,
                                   _dp(V))
    z = s.X[:nsg, 2]
    layer = np.rint(z / (A_LATTICE / 4)).astype(int)
    tags = np.zeros(N, dtype=np.uint32)
    tags[:nsg][layer < fixed_layers] = _abi.TAG_FROZEN
    tags[:nsg][(layer >= fixed_layers) & (layer < fixed_layers + thermo_layers)] = _abi.TAG_THERMO
    V[:nsg][layer < fixed_layers] = 0.0
    surf = float(z.max())
    az = 2 * np.pi * s.rng() if azimuth is None else float(azimuth)
    th = np.deg2rad(polar_deg)
    speed = np.sqrt(2 * ion_eV * p.ec / p.massGa)
    X = s.X.copy(order="F")
    if impact_xy is None:
        xr = s.rng()
        yr = s.rng()
        xy = (xr * p.Lb[0], yr * p.Lb[1])
    else:
        xy = impact_xy
    X[nsg] = [xy[0], xy[1], surf + ion_height]
    V[nsg] = speed * np.array([np.sin(th) * np.cos(az), np.sin(th) * np.sin(az), -np.cos(th)])
    p.remove_z = surf + remove_above
    return SpecSlab(p, X, s.Xi.copy(order="F"), V, s.mass.copy(), s.atype.copy(), tags, surf)


@dataclass
class DoseSlab:
    """A spec-mode slab with pre-allocated ions for a dose of impacts: the
    ions are atoms Nsg+1 .. Nsg+n (1-based), tagged removed until injected;
    X0/V0 are their start states, one row per impact."""

    slab: SpecSlab
    ion_atoms: np.ndarray
    X0: np.ndarray
    V0: np.ndarray


def dose_slab(cells, nimp: int, seed: int, ion_eV: float = 2000.0, window: float = 30e-10,
              ion_height: float = 10e-10, remove_above: float = 15e-10,
              params: Params | None = None) -> DoseSlab:
    """A slab (spec_slab's layers, tags and 300 K velocities) with nimp ions
    for successive impacts at normal incidence, each at a seeded uniform
    point of a window x window square centred on the slab."""
    p = params_default() if params is None else as_params(params)
    p.mode = _abi.MODE_SPEC
    base = spec_slab(cells, seed, ion_eV, 0.0, ion_height=ion_height, remove_above=remove_above,
                     params=p)
    q = base.params
    nsg = q.Nsg
    s = crystal_system(tuple(cells), nimp, -abs(int(seed)) - 1, params=q)
    q = s.params
    N = q.Natm
    rs = np.random.default_rng(int(seed) + 7919)
    cx, cy = 0.5 * q.Lb[0], 0.5 * q.Lb[1]
    X0 = np.zeros((nimp, 3))
    X0[:, 0] = cx + rs.uniform(-0.5, 0.5, nimp) * window
    X0[:, 1] = cy + rs.uniform(-0.5, 0.5, nimp) * window
    X0[:, 2] = base.surface_z + ion_height
    V0 = np.zeros((nimp, 3))
    V0[:, 2] = -np.sqrt(2 * ion_eV * q.ec / q.massGa)
    X = np.zeros((N, 3), order="F")
    V = np.zeros((N, 3), order="F")
    X[:nsg] = base.X[:nsg]
    V[:nsg] = base.V[:nsg]
    X[nsg:] = X0
    tags = np.zeros(N, dtype=np.uint32)
    tags[:nsg] = base.tags[:nsg]
    tags[nsg:] = _abi.TAG_REMOVED
    q.remove_z = base.params.remove_z
    slab = SpecSlab(q, X, s.Xi.copy(order="F"), V, s.mass.copy(), s.atype.copy(), tags,
                    base.surface_z)
    return DoseSlab(slab, np.arange(nsg + 1, nsg + nimp + 1, dtype=np.int32), X0, V0)


def crater_depth(X, atype, Lb, surface_z: float, remove_z: float, centre, window: float,
                 column: float = 3.0e-10) -> float:
    """Deepest point of the surface inside a window x window square around
    centre (x, y): the top lattice atom of each column x column bin, and the
    largest drop of those below the initial surface (m; 0 if none)."""
    X = np.asarray(X)
    keep = (np.asarray(atype) < 3) & (X[:, 2] <= remove_z)
    L = np.asarray(Lb, dtype=np.float64)[:2]
    d = X[keep, :2] - np.asarray(centre, dtype=np.float64)[None, :]
    d -= L * np.rint(d / L)
    inside = np.all(np.abs(d) < 0.5 * window, axis=1)
    z = X[keep, 2][inside]
    ij = np.floor((d[inside] + 0.5 * window) / column).astype(int)
    nb = int(np.ceil(window / column))
    top = np.full((nb, nb), -np.inf)
    np.maximum.at(top, (ij[:, 0].clip(0, nb - 1), ij[:, 1].clip(0, nb - 1)), z)
    top = top[np.isfinite(top)]
    return float(max(0.0, surface_z - top.min())) if top.size else 0.0


def impact_statistics(X, Xi, atype, Lb, surface_z: float, remove_z: float,
                      displaced_threshold: float = 1.0e-10):
    """Outcome of one impact from its final positions: (sputtered atoms,
    ion depth below the surface in m (nan if the ion is above it), displaced
    lattice atoms). Sputtered atoms are the lattice atoms above remove_z
    (removed atoms stay where they were taken out); an atom is displaced
    when it is farther than displaced_threshold from its initial site
    (minimum image in x and y)."""
    X = np.asarray(X)
    Xi = np.asarray(Xi)
    atype = np.asarray(atype)
    lattice = atype < 3
    up = X[:, 2] > remove_z
    sputtered = int(np.count_nonzero(lattice & up))
    ion = np.nonzero(atype == 3)[0]
    depth = float("nan")
    if ion.size:
        z = float(X[ion[0], 2])
        depth = surface_z - z if z <= surface_z else float("nan")
    d = X - Xi
    L = np.asarray(Lb, dtype=np.float64)[:2]
    d[:, :2] -= L * np.rint(d[:, :2] / L)
    r2 = np.einsum("ij,ij->i", d, d)
    displaced = int(np.count_nonzero(lattice & ~up & (r2 > displaced_threshold ** 2)))
    return sputtered, depth, displaced


def knock(p: Params, rng: Ran1, knc: int, eV: float, phiz: float, phixy: float,
          Xrand: np.ndarray):
    """knock (src/knock.f90:21-55): (1-based ion index, x[3], v[3])."""
    x = np.zeros(3)
    v = np.zeros(3)
    Xr = _fortran(Xrand)
    i = _abi.load().fibmd_host_knock(C.byref(p), C.byref(rng.state), knc, eV, phiz, phixy,
                                     _dp(Xr), Xr.shape[0], _dp(x), _dp(v))
    return i, x, v


def pipe_peaks():
    """Measured (fp64, fp32) FMA TFLOP/s of the current device."""
    a, b = C.c_double(), C.c_double()
    rc = _abi.load().fibmd_gpu_pipe_peaks(C.byref(a), C.byref(b))
    if rc:
        raise FibmdError(rc, "pipe_peaks")
    return a.value, b.value


class FibMD:
    """One device context (libfibmd_gpu's fibmd_ctx)."""

    def __init__(self, params: Params):
        self.lib = _abi.load()
        self.params = as_params(params)
        self.N = params.Natm
        h = C.c_void_p()
        rc = self.lib.fibmd_gpu_create(C.byref(self.params), C.byref(h))
        if rc:
            buf = C.create_string_buffer(512)
            self.lib.fibmd_gpu_last_error(None, buf, 512)
            raise FibmdError(rc, buf.value.decode())
        self.h = h

    # ---- helpers
    def _check(self, rc: int, what: str):
        if rc:
            buf = C.create_string_buffer(1024)
            self.lib.fibmd_gpu_last_error(self.h, buf, 1024)
            raise FibmdError(rc, f"{what}: {buf.value.decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.fibmd_gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state
    def upload(self, X, V, F, Xi, mass, atype, xsides):
        X, V, Xi = _fortran(X), _fortran(V), _fortran(Xi)
        Fa = None if F is None else _fortran(F)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        atype = np.ascontiguousarray(atype, dtype=np.int32)
        xsides = np.ascontiguousarray(xsides, dtype=np.int32)
        self._check(self.lib.fibmd_gpu_upload(self.h, _dp(X), _dp(V),
                                              None if Fa is None else _dp(Fa), _dp(Xi),
                                              _dp(mass), _ip(atype), _ip(xsides)), "upload")

    def upload_system(self, s: System, F=None):
        self.upload(s.X, s.V, F, s.Xi, s.mass, s.atype, s.xsides)

    def download(self):
        X = np.zeros((self.N, 3), order="F")
        V = np.zeros((self.N, 3), order="F")
        F = np.zeros((self.N, 3), order="F")
        self._check(self.lib.fibmd_gpu_download(self.h, _dp(X), _dp(V), _dp(F)), "download")
        return X, V, F

    def set_tags(self, tags):
        t = np.ascontiguousarray(tags, dtype=np.uint32)
        self._check(self.lib.fibmd_gpu_set_tags(self.h, t.ctypes.data_as(C.POINTER(C.c_uint32))),
                    "set_tags")

    def get_tags(self) -> np.ndarray:
        """The per-atom tags as the device holds them (TAG_REMOVED set by
        spec-mode removal)."""
        t = np.zeros(self.N, dtype=np.uint32)
        self._check(self.lib.fibmd_gpu_get_tags(self.h, t.ctypes.data_as(C.POINTER(C.c_uint32))),
                    "get_tags")
        return t

    def spec_scalars(self):
        """(time, dt, removed lattice atoms) of the system (replica 0)."""
        t = np.zeros(1)
        dt = np.zeros(1)
        rm = np.zeros(1, dtype=np.int32)
        self._check(self.lib.fibmd_gpu_batch_scalars(self.h, _dp(t), _dp(dt), _ip(rm)),
                    "batch_scalars")
        return float(t[0]), float(dt[0]), int(rm[0])

    def set_atom(self, i: int, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        self._check(self.lib.fibmd_gpu_set_atom(self.h, int(i), _dp(x), _dp(v)), "set_atom")

    def set_impact(self, impact: int):
        self._check(self.lib.fibmd_gpu_set_impact(self.h, int(impact)), "set_impact")

    def ionrun(self, tic: int):
        self._check(self.lib.fibmd_gpu_ionrun(self.h, int(tic)), "ionrun")

    def set_tau(self, tau: float):
        self._check(self.lib.fibmd_gpu_set_tau(self.h, float(tau)), "set_tau")

    # ---- si.f90
    def si_nlist(self):
        self._check(self.lib.fibmd_gpu_nlist(self.h), "si_nlist")

    def list_counts(self):
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self._check(self.lib.fibmd_gpu_list_counts(self.h, C.byref(a), C.byref(b), C.byref(c)),
                    "list_counts")
        return a.value, b.value, c.value

    def get_pairs(self, kind: int = 0) -> np.ndarray:
        n = C.c_int()
        self._check(self.lib.fibmd_gpu_get_pairs(self.h, kind, C.byref(n), None, 0), "get_pairs")
        out = np.zeros((max(n.value, 1), 2), dtype=np.int32)
        self._check(self.lib.fibmd_gpu_get_pairs(self.h, kind, C.byref(n), _ip(out), n.value),
                    "get_pairs")
        return out[: n.value]

    def get_triplets(self) -> np.ndarray:
        n = C.c_longlong()
        self._check(self.lib.fibmd_gpu_get_triplets(self.h, C.byref(n), None, 0), "get_triplets")
        out = np.zeros((max(n.value, 1), 3), dtype=np.int32)
        self._check(self.lib.fibmd_gpu_get_triplets(self.h, C.byref(n), _ip(out), n.value),
                    "get_triplets")
        return out[: n.value]

    def si_force(self) -> np.ndarray:
        F = np.zeros((self.N, 3), order="F")
        self._check(self.lib.fibmd_gpu_force(self.h, _dp(F), None, None), "si_force")
        return F

    def si_force_energy(self):
        """Forces together with si_potential's per-atom and total energy."""
        F = np.zeros((self.N, 3), order="F")
        u = np.zeros(self.N)
        U = C.c_double()
        self._check(self.lib.fibmd_gpu_force(self.h, _dp(F), _dp(u), C.byref(U)), "si_force")
        return F, u, U.value

    def si_potential(self):
        _, u, U = self.si_force_energy()
        return U, u

    def virial(self, per_atom: bool = False):
        """The virial of the current positions (fibmd_gpu_virial): W as xx,
        yy, zz, xy, xz, yz in J, and with per_atom the (N, 6) per-atom
        shares (else None)."""
        W = np.zeros(6)
        wa = np.zeros((self.N, 6), order="F") if per_atom else None
        self._check(self.lib.fibmd_gpu_virial(self.h, _dp(W), _dp(wa) if per_atom else None),
                    "virial")
        return W, wa

    def work_counters(self):
        c = (C.c_longlong * 6)()
        self._check(self.lib.fibmd_gpu_work_counters(self.h, c), "work_counters")
        return list(c)

    # ---- timeint.f90 / temp.f90
    def steps(self, whichctrl: int, max_steps: int, lt: int, time: float, temp: float):
        l = C.c_longlong(lt)
        t = C.c_double(time)
        T = C.c_double(temp)
        why = C.c_int()
        self._check(self.lib.fibmd_gpu_steps(self.h, whichctrl, max_steps, C.byref(l), C.byref(t),
                                             C.byref(T), C.byref(why)), "steps")
        return l.value, t.value, T.value, why.value

    def dose(self, ion_atoms, X0, V0, steps: int, relax_s: float = 0.0):
        """Successive impacts run on the device (fibmd_gpu_dose): ion_atoms are
        1-based indices of pre-allocated ions, X0/V0 their (n, 3) start states.
        Returns per impact (lattice atoms removed, ions removed, time, MD steps)
        so far."""
        a = np.ascontiguousarray(ion_atoms, dtype=np.int32)
        n = len(a)
        X0 = _fortran(X0)
        V0 = _fortran(V0)
        rm = np.zeros(n, dtype=np.int32)
        ir = np.zeros(n, dtype=np.int32)
        t = np.zeros(n)
        st = np.zeros(n, dtype=np.int64)
        self._check(self.lib.fibmd_gpu_dose(self.h, n, _ip(a), _dp(X0), _dp(V0), int(steps),
                                            float(relax_s), _ip(rm), _ip(ir), _dp(t),
                                            st.ctypes.data_as(C.POINTER(C.c_longlong))), "dose")
        return rm, ir, t, st

    def impact_stats(self, surface_z, displaced_m: float = 1.0e-10):
        """Per replica (sputtered atoms, displaced lattice atoms, ion depth in
        m or nan), computed on the device (fibmd_gpu_impact_stats)."""
        sz = np.ascontiguousarray(np.atleast_1d(surface_z), dtype=np.float64)
        R = len(sz)
        sp = np.zeros(R, dtype=np.int32)
        dc = np.zeros(R, dtype=np.int32)
        dp = np.zeros(R)
        self._check(self.lib.fibmd_gpu_impact_stats(self.h, _dp(sz), float(displaced_m), _ip(sp),
                                                    _ip(dc), _dp(dp)), "impact_stats")
        return sp, dc, dp

    def xyz_frame(self):
        """writeatoms' columns computed on the device: positions in Angstrom
        (N, 3) and kinetic energies in eV (N)."""
        xyz = np.zeros((self.N, 3), order="F")
        ke = np.zeros(self.N)
        self._check(self.lib.fibmd_gpu_xyz_frame(self.h, _dp(xyz), _dp(ke)), "xyz_frame")
        return xyz, ke

    def temperature(self) -> float:
        T = C.c_double()
        self._check(self.lib.fibmd_gpu_temperature(self.h, C.byref(T)), "temperature")
        return T.value

    def regime(self):
        Ts = C.c_double()
        tic = C.c_int()
        self._check(self.lib.fibmd_gpu_regime(self.h, C.byref(Ts), C.byref(tic)), "regime")
        return Ts.value, tic.value

    def set_option(self, key: str, value: float):
        self._check(self.lib.fibmd_gpu_set_option(self.h, key.encode(), float(value)), "set_option")

    def get_option(self, key: str) -> float:
        v = C.c_double()
        self._check(self.lib.fibmd_gpu_get_option(self.h, key.encode(), C.byref(v)), "get_option")
        return v.value

    def kernel_time(self, reset: bool = False):
        t = C.c_double()
        n = C.c_longlong()
        self._check(self.lib.fibmd_gpu_kernel_time(self.h, C.byref(t), C.byref(n), int(reset)),
                    "kernel_time")
        return t.value, n.value

    PHASES = ("at", "nt", "ds", "f", "force_kernel", "drift", "kick")

    def phase_times(self, reset: bool = False) -> dict:
        t = (C.c_double * 7)()
        n = (C.c_longlong * 7)()
        self._check(self.lib.fibmd_gpu_phase_times(self.h, t, n, int(reset)), "phase_times")
        return {k: (t[i], n[i]) for i, k in enumerate(self.PHASES)}

    @property
    def stream_ptr(self) -> int:
        return int(self.lib.fibmd_gpu_stream(self.h) or 0)

    def timers(self, reset: bool = False):
        v = [C.c_double() for _ in range(4)]
        c = (C.c_longlong * 4)()
        self._check(self.lib.fibmd_gpu_timers(self.h, *[C.byref(x) for x in v], c, int(reset)),
                    "timers")
        return [x.value for x in v], list(c)


class FibMDBatch(FibMD):
    """A batched ensemble of independent spec-mode replicas in one context
    (fibmd_gpu_batch_create). Per-atom arrays have the padded length
    self.N; replica r occupies rows offsets[r] : offsets[r] + natm[r]."""

    def __init__(self, params: Params, replicas):
        """replicas: sequence of (natm, nsg, Lb[3], remove_z)."""
        self.lib = _abi.load()
        self.params = as_params(params)
        R = len(replicas)
        arr = (Replica * R)()
        for r, (natm, nsg, Lb, rz) in enumerate(replicas):
            arr[r].natm, arr[r].nsg = int(natm), int(nsg)
            for d in range(3):
                arr[r].Lb[d] = float(Lb[d])
            arr[r].remove_z = float(rz)
        h = C.c_void_p()
        rc = self.lib.fibmd_gpu_batch_create(C.byref(self.params), R, arr, C.byref(h))
        if rc:
            buf = C.create_string_buffer(512)
            self.lib.fibmd_gpu_last_error(None, buf, 512)
            raise FibmdError(rc, buf.value.decode())
        self.h = h
        self.natm = np.array([int(x[0]) for x in replicas])
        offs = np.zeros(R + 1, dtype=np.int32)
        n = C.c_int()
        self._check(self.lib.fibmd_gpu_batch_layout(self.h, C.byref(n), _ip(offs)), "batch_layout")
        self.nrep = n.value
        self.offsets = offs
        self.N = int(offs[-1])

    def pad(self, parts, fill=0.0, dtype=np.float64):
        """Concatenate per-replica arrays into the padded layout."""
        first = np.asarray(parts[0])
        shape = (self.N,) + first.shape[1:]
        out = np.full(shape, fill, dtype=dtype)
        for r, a in enumerate(parts):
            a = np.asarray(a)
            out[self.offsets[r]:self.offsets[r] + len(a)] = a
        return np.asfortranarray(out) if out.ndim > 1 else out

    def rows(self, r: int) -> slice:
        return slice(int(self.offsets[r]), int(self.offsets[r] + self.natm[r]))

    def scalars(self):
        """Per-replica (time, dt, removed count)."""
        t = np.zeros(self.nrep)
        dt = np.zeros(self.nrep)
        rm = np.zeros(self.nrep, dtype=np.int32)
        self._check(self.lib.fibmd_gpu_batch_scalars(self.h, _dp(t), _dp(dt), _ip(rm)),
                    "batch_scalars")
        return t, dt, rm


class XyzWriter:
    """writeatoms' dump files (fibmd_host_xyz_*): frames appended to `path`
    in the reference's extended-xyz layout and, if given, the snapshot file
    rewritten with each frame, both written by a background thread."""

    def __init__(self, path, snap_path=None):
        self.lib = _abi.load()
        h = C.c_void_p()
        rc = self.lib.fibmd_host_xyz_open(str(path).encode(),
                                          None if snap_path is None else str(snap_path).encode(),
                                          C.byref(h))
        if rc:
            raise FibmdError(rc, f"cannot open {path}")
        self.h = h

    def write(self, time_s, xyz_A, atype, ke_eV, proc=None):
        xyz = _fortran(xyz_A)
        t = np.ascontiguousarray(atype, dtype=np.int32)
        ke = np.ascontiguousarray(ke_eV, dtype=np.float64)
        pr = None if proc is None else np.ascontiguousarray(proc, dtype=np.int32)
        rc = self.lib.fibmd_host_xyz_write(self.h, len(t), float(time_s), _dp(xyz), _ip(t),
                                           _dp(ke), None if pr is None else _ip(pr))
        if rc:
            raise FibmdError(rc, "xyz write")

    def flush(self):
        rc = self.lib.fibmd_host_xyz_flush(self.h)
        if rc:
            raise FibmdError(rc, "xyz flush")

    def close(self):
        if getattr(self, "h", None):
            rc = self.lib.fibmd_host_xyz_close(self.h)
            self.h = None
            if rc:
                raise FibmdError(rc, "xyz close")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def write_restart(path, lt: int, restart_time: float, X, V, mass, atype, impact: int):
    """writerestart (src/out.f90:34-58): Fortran unformatted records."""
    X, V = _fortran(X), _fortran(V)
    m = np.ascontiguousarray(mass, dtype=np.float64)
    t = np.ascontiguousarray(atype, dtype=np.int32)
    rc = _abi.load().fibmd_host_write_restart(str(path).encode(), len(m), int(lt),
                                              float(restart_time), _dp(X), _dp(V), _dp(m),
                                              _ip(t), int(impact))
    if rc:
        raise FibmdError(rc, f"write_restart {path}")


def read_restart(path, natm: int):
    """The records of write_restart: (lt, restart_time, X, V, mass, atype, impact)."""
    X = np.zeros((natm, 3), order="F")
    V = np.zeros((natm, 3), order="F")
    m = np.zeros(natm)
    t = np.zeros(natm, dtype=np.int32)
    lt, imp = C.c_int(), C.c_int()
    rt = C.c_double()
    rc = _abi.load().fibmd_host_read_restart(str(path).encode(), natm, C.byref(lt), C.byref(rt),
                                             _dp(X), _dp(V), _dp(m), _ip(t), C.byref(imp))
    if rc:
        raise FibmdError(rc, f"read_restart {path}")
    return lt.value, rt.value, X, V, m, t, imp.value

