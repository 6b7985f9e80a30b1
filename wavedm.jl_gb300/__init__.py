"""wavedm.jl_gb300: GB300-native split-step KDK step for the Schroedinger-Poisson equation.

The compute path is libwavedm.so (hand-written sm_103a CUDA kernels behind a C
ABI, ``include/wavedm.h``).  This package is the host side: a ctypes binding
(``_abi``), a context handle (``core.SPEContext``), the reference-shaped
operator API (``solver``: apply_kick_step, apply_drift_step, parallel_poisson,
SPE3D_waveDM, ...) and the seeded workload generators (``ics``).
"""
from . import _abi, ics  # noqa: F401
from .core import Ensemble, SPEContext, size_supported, weighted_quantiles_grouped  # noqa: F401

__all__ = ["SPEContext", "Ensemble", "size_supported", "weighted_quantiles_grouped", "ics", "build_library",
           "lib_path"]


def build_library(force=False, verbose=False):
    """Compile libwavedm.so for sm_103a in-tree (nvcc); returns its path."""
    import importlib.util
    import os

    spec = importlib.util.spec_from_file_location(
        "_wavedm_build", os.path.join(os.path.dirname(os.path.abspath(__file__)), "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force, verbose=verbose)


def lib_path():
    return _abi.LIB_PATH
