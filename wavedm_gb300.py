"""Import name for the package directory ``wavedm.jl_gb300/``.

A directory whose name contains a dot cannot be imported directly; this module
loads it under the name ``wavedm_gb300`` and replaces itself with it.
"""
import importlib.util
import os
import sys

_pkg_dir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "wavedm.jl_gb300")
_spec = importlib.util.spec_from_file_location(
    __name__, os.path.join(_pkg_dir, "__init__.py"), submodule_search_locations=[_pkg_dir])
_mod = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _mod
_spec.loader.exec_module(_mod)
