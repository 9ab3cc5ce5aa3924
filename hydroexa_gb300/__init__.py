"""GB300 (sm_103a) per-level advance of the HydroEXA shallow-water solver.

The compute path is the CUDA library ``libhydroexa_gb300.so`` behind the C ABI
of ``include/hydroexa_gb300.h``; this package holds its build recipe
(``build``), the ctypes binding (``capi``), device-resident level state over
torch CUDA tensors (``level``), a mirror of the reference solver's operator
surface (``solver``) and the seeded synthetic workloads (``workloads``).
"""
from . import build as _build_mod

__version__ = "0.1.0"


def build(force: bool = False, verbose: bool = False):
    """Compile libhydroexa_gb300.so for sm_103a (no-op when up to date)."""
    return _build_mod.build(force=force, verbose=verbose)
