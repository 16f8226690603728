"""chimera_gb300 -- GB300-native (sm_103a) per-step PIC hot path of CHIMERA.

Drop-in for the reference's Python API (``chimera.moduls``): ``Solver``,
``Specie``, ``ChimeraRun`` and the f2py kernel module ``fimera``, with every
kernel running as hand-written CUDA in libchimera_gb300.so.
"""
from ._lib import ChimeraError  # noqa: F401


def __getattr__(name):
    # the drop-in classes import torch and the CUDA library lazily
    import importlib
    where = {"Solver": ("solvers", "Solver"), "Specie": ("species", "Specie"),
             "ChimeraRun": ("chimera_main", "ChimeraRun")}
    if name in where:
        mod, attr = where[name]
        return getattr(importlib.import_module(f"{__name__}.{mod}"), attr)
    raise AttributeError(name)

__version__ = "0.1.0"


def build(force: bool = False) -> str:
    """Compile libchimera_gb300.so in-tree (nvcc, sm_103a)."""
    from . import buildlib as _b
    return _b.build(force=force)
