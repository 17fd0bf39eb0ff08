"""GB300-native force path of the Moldy rigid-molecule MD code.

Real-space link-cell forces (force_calc) and reciprocal-space Ewald forces
(ewald) as hand-written sm_103a CUDA kernels behind a C ABI
(libmoldy_gb300.so; include/moldy_gb300.h, include/moldy_ref_abi.h).
"""
from .system import System, Species, Control  # noqa: F401

__all__ = ["System", "Species", "Control", "ForceField", "poteval"]


def __getattr__(name):
    # the GPU binding loads libmoldy_gb300.so lazily, on first use
    if name in ("ForceField", "poteval"):
        from . import forcefield
        return getattr(forcefield, name)
    raise AttributeError(name)
