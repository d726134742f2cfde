"""ctypes declarations of libfibmd_gpu.so (include/fibmd_gpu.h, fibmd_host.h).

The library is loaded from this package directory. A missing library is an
error: there is no CPU fallback for the GPU path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfibmd_gpu.so"

ABI_VERSION = 1

# status codes
OK, EINVAL, ECUDA, EOVERFLOW, ENAN, ETIMEOUT, ESTATE, ENOMEM, ETABLE = range(9)
STATUS_NAMES = {0: "OK", 1: "EINVAL", 2: "ECUDA", 3: "EOVERFLOW", 4: "ENAN", 5: "ETIMEOUT",
                6: "ESTATE", 7: "ENOMEM", 8: "ETABLE"}
MODE_REF, MODE_SPEC = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
TAG_FROZEN, TAG_THERMO, TAG_REMOVED = 1, 2, 4
STOP_MAXSTEPS, STOP_DUMP, STOP_DONE, STOP_REGIME = 1, 2, 4, 8

_D = C.c_double
_I = C.c_int


class Params(C.Structure):
    """Mirror of `fibmd_params` (field order and types as in fibmd_gpu.h)."""

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


class Replica(C.Structure):
    """Mirror of `fibmd_replica`: one replica of a batched ensemble."""

    _fields_ = [("natm", _I), ("nsg", _I), ("Lb", _D * 3), ("remove_z", _D),
                ("reserved", _I * 4)]


class Siga(C.Structure):
    """Mirror of `fibmd_siga` (fibmd_host.h)."""

    _fields_ = [
        ("amorcrys", _I), ("whichic", _I), ("startimpact", _I),
        ("eV", _D), ("Nc", _I * 3), ("Npc", _I * 3), ("Nt", _I),
        ("ke_limit_2", _D), ("Uo", _D), ("eng_out", _I), ("tmp_out", _I),
        ("Nrand", _I), ("fwhm", _D), ("phiz", _D), ("phixy", _D),
    ]


class Rng(C.Structure):
    """Mirror of `fibmd_rng`: ran1's shuffle table and state."""

    _fields_ = [("iv", _I * 32), ("iy", _I), ("idum", _I)]


_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LLP = C.POINTER(C.c_longlong)
_VP = C.c_void_p

SIGNATURES = {
    # fibmd_gpu.h
    "fibmd_gpu_params_default": (_I, [C.POINTER(Params)]),
    "fibmd_gpu_abi_version": (_I, []),
    "fibmd_gpu_params_size": (_I, []),
    "fibmd_gpu_create": (_I, [C.POINTER(Params), C.POINTER(_VP)]),
    "fibmd_gpu_destroy": (None, [_VP]),
    "fibmd_gpu_last_error": (_I, [_VP, C.c_char_p, _I]),
    "fibmd_gpu_upload": (_I, [_VP, _DP, _DP, _DP, _DP, _DP, _IP, _IP]),
    "fibmd_gpu_download": (_I, [_VP, _DP, _DP, _DP]),
    "fibmd_gpu_set_tags": (_I, [_VP, C.POINTER(C.c_uint32)]),
    "fibmd_gpu_get_tags": (_I, [_VP, C.POINTER(C.c_uint32)]),
    "fibmd_gpu_set_atom": (_I, [_VP, _I, _DP, _DP]),
    "fibmd_gpu_set_impact": (_I, [_VP, _I]),
    "fibmd_gpu_ionrun": (_I, [_VP, _I]),
    "fibmd_gpu_set_tau": (_I, [_VP, _D]),
    "fibmd_gpu_nlist": (_I, [_VP]),
    "fibmd_gpu_list_counts": (_I, [_VP, _LLP, _LLP, _LLP]),
    "fibmd_gpu_get_pairs": (_I, [_VP, _I, _IP, _IP, _I]),
    "fibmd_gpu_get_triplets": (_I, [_VP, _LLP, _IP, C.c_longlong]),
    "fibmd_gpu_force": (_I, [_VP, _DP, _DP, _DP]),
    "fibmd_gpu_steps": (_I, [_VP, _I, C.c_longlong, _LLP, _DP, _DP, _IP]),
    "fibmd_gpu_temperature": (_I, [_VP, _DP]),
    "fibmd_gpu_regime": (_I, [_VP, _DP, _IP]),
    "fibmd_gpu_timers": (_I, [_VP, _DP, _DP, _DP, _DP, _LLP, _I]),
    "fibmd_gpu_work_counters": (_I, [_VP, _LLP]),
    "fibmd_gpu_virial": (_I, [_VP, _DP, _DP]),
    "fibmd_gpu_stream": (_VP, [_VP]),
    "fibmd_gpu_set_option": (_I, [_VP, C.c_char_p, _D]),
    "fibmd_gpu_get_option": (_I, [_VP, C.c_char_p, _DP]),
    "fibmd_gpu_kernel_time": (_I, [_VP, _DP, _LLP, _I]),
    "fibmd_gpu_phase_times": (_I, [_VP, _DP, _LLP, _I]),
    "fibmd_gpu_pipe_peaks": (_I, [_DP, _DP]),
    "fibmd_gpu_force_noalloc": (_I, [C.POINTER(Params), _VP, _VP, _I, _VP, _VP]),
    "fibmd_gpu_xyz_frame": (_I, [_VP, _DP, _DP]),
    "fibmd_host_xyz_open": (_I, [C.c_char_p, C.c_char_p, C.POINTER(_VP)]),
    "fibmd_host_xyz_write": (_I, [_VP, _I, _D, _DP, _IP, _DP, _IP]),
    "fibmd_host_xyz_flush": (_I, [_VP]),
    "fibmd_host_xyz_close": (_I, [_VP]),
    "fibmd_host_write_restart": (_I, [C.c_char_p, _I, _I, _D, _DP, _DP, _DP, _IP, _I]),
    "fibmd_host_read_restart": (_I, [C.c_char_p, _I, _IP, _DP, _DP, _DP, _DP, _IP, _IP]),
    "fibmd_gpu_dose": (_I, [_VP, _I, _IP, _DP, _DP, C.c_longlong, _D, _IP, _IP, _DP, _LLP]),
    "fibmd_gpu_batch_create": (_I, [C.POINTER(Params), _I, C.POINTER(Replica), C.POINTER(_VP)]),
    "fibmd_gpu_batch_layout": (_I, [_VP, _IP, _IP]),
    "fibmd_gpu_impact_stats": (_I, [_VP, _DP, _D, _IP, _IP, _DP]),
    "fibmd_gpu_batch_scalars": (_I, [_VP, _DP, _DP, _IP]),
    # fibmd_host.h
    "fibmd_host_rng_seed": (None, [C.POINTER(Rng), _I]),
    "fibmd_host_ran1": (_D, [C.POINTER(Rng)]),
    "fibmd_host_read_siga": (_I, [C.c_char_p, C.POINTER(Params), C.POINTER(Siga), C.c_char_p, _I]),
    "fibmd_host_pureepi": (_I, [_I, _I, _I, _DP, _IP, _DP]),
    "fibmd_host_initranions": (None, [C.POINTER(Rng), _I, _D, _DP]),
    "fibmd_host_init_state": (_I, [C.POINTER(Params), C.POINTER(Rng), _D, _DP, _DP, _DP, _DP, _IP]),
    "fibmd_host_knock": (_I, [C.POINTER(Params), C.POINTER(Rng), _I, _D, _D, _D, _DP, _I, _DP, _DP]),
    "fibmd_host_maxwell": (None, [C.POINTER(Rng), _I, _I, _DP, _D, _D, _DP]),
}

_lib: C.CDLL | None = None


def load() -> C.CDLL:
    """Load libfibmd_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(or python fib_md_gb300/build.py); the GPU path has no CPU fallback")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.fibmd_gpu_abi_version() != ABI_VERSION:
        raise RuntimeError("libfibmd_gpu.so ABI version mismatch")
    if lib.fibmd_gpu_params_size() != C.sizeof(Params):
        raise RuntimeError("fibmd_params layout mismatch between Python and the library")
    _lib = lib
    return lib
