"""fib_md_gb300 — GB300 (sm_103a) backend for FIB_MD's per-step hot path.

Cell binning, Verlet lists, the fused Stillinger-Weber/Moliere force and the
velocity-Verlet step run as CUDA kernels in libfibmd_gpu.so behind the C-ABI
of include/fibmd_gpu.h; this package is the Python binding of that ABI.
"""
from . import _abi
from ._abi import (MODE_REF, MODE_SPEC, PREC_FP64, PREC_MIXED, STOP_DONE, STOP_DUMP,
                   STOP_MAXSTEPS, STOP_REGIME, TAG_FROZEN, TAG_REMOVED, TAG_THERMO, Params,
                   Siga)
from .md import (DoseSlab, FibMD, FibMDBatch, FibmdError, Ran1, SpecSlab, System, crystal_system,
                 crater_depth, dose_slab, knock,
                 impact_statistics, params_default, pureepi, read_restart, read_siga, spec_slab,
                 write_restart, XyzWriter)

__all__ = [
    "FibMD", "FibMDBatch", "FibmdError", "Params", "Siga", "Ran1", "SpecSlab", "System",
    "XyzWriter", "read_restart", "write_restart", "crater_depth", "crystal_system", "DoseSlab", "dose_slab", "impact_statistics", "knock", "spec_slab",
    "params_default", "pureepi", "read_siga", "MODE_REF", "MODE_SPEC", "PREC_FP64",
    "PREC_MIXED", "TAG_FROZEN", "TAG_THERMO", "TAG_REMOVED", "STOP_MAXSTEPS", "STOP_DUMP",
    "STOP_DONE", "STOP_REGIME",
]


def library_path():
    return _abi.LIB_PATH
