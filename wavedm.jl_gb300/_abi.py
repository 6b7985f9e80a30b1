"""ctypes binding of libwavedm (the C ABI declared in include/wavedm.h).

The library is built in-tree (``wavedm.jl_gb300/libwavedm.so``; the environment
variable WDM_LIB_PATH selects another build).  Loading it never falls back to
anything else: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwavedm.so")

WDM_OK = 0
STATUS = {
    0: "WDM_OK",
    1: "WDM_ERR_INVALID",
    2: "WDM_ERR_UNSUPPORTED",
    3: "WDM_ERR_CUDA",
    4: "WDM_ERR_ALLOC",
    5: "WDM_ERR_NONFINITE",
    6: "WDM_ERR_STATE",
}
HOST, DEVICE = 0, 1
STEP_MODES = {"strang": 0, "reference_loop": 1, "lie": 2}
CONVENTIONS = {"periodic": 0, "reference": 1}
PHASE_MODES = {"plain": 0, "precise": 1}
TIDE_CENTERING = {"box_centre": 0, "reference": 1, "density_max": 2}


class WdmDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("convention", C.c_int32),
        ("poisson_coeff", C.c_double),
        ("kerr", C.c_double),
        ("absorb_alpha", C.c_double),
        ("phase_mode", C.c_int32),
        ("batch", C.c_int32),
    ]


# (name, restype, argtypes) for every symbol declared in include/wavedm.h
_vp, _i32, _i64, _d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
SIGNATURES = [
    ("wdm_create", _i32, [C.POINTER(WdmDesc), C.POINTER(_vp)]),
    ("wdm_destroy", _i32, [_vp]),
    ("wdm_last_error", C.c_char_p, [_vp]),
    ("wdm_version", _i32, []),
    ("wdm_size_supported", _i32, [_i32]),
    ("wdm_set_psi", _i32, [_vp, _vp, _i32]),
    ("wdm_get_psi", _i32, [_vp, _vp, _i32]),
    ("wdm_get_rho", _i32, [_vp, _vp, _i32]),
    ("wdm_get_phi", _i32, [_vp, _vp, _i32]),
    ("wdm_set_static_potential", _i32, [_vp, _vp, _i32]),
    ("wdm_set_tidal", _i32, [_vp, _vp, _i32, _i32]),
    ("wdm_set_tidal_clock", _i32, [_vp, _d, _d]),
    ("wdm_set_tidal_centering", _i32, [_vp, _i32]),
    ("wdm_set_particles", _i32, [_vp, _vp, _vp, _i64]),
    ("wdm_step", _i32, [_vp, _i32, _d, _d, _i32]),
    ("wdm_step_async", _i32, [_vp, _i32, _d, _d, _i32]),
    ("wdm_kick", _i32, [_vp, _d, _d]),
    ("wdm_drift", _i32, [_vp, _d]),
    ("wdm_poisson", _i32, [_vp, _vp, _vp, _i32]),
    ("wdm_fft3d", _i32, [_vp, _vp, _i32]),
    ("wdm_poisson_noalloc", _i32, [_vp, _vp, _i32, _i32, _i32, _d, _d, _d, _d, _vp]),
    ("wdm_reduce", _i32, [_vp, _vp]),
    ("wdm_diagnostics", _i32, [_vp, _vp]),
    ("wdm_weighted_quantiles_grouped", _i32, [_vp, _vp, _vp, _i64, _vp, _i32, _vp]),
    ("wdm_interpolate_phi", _i32, [_vp, _vp, _i64, _vp]),
    ("wdm_check_finite", _i32, [_vp, C.POINTER(_i32)]),
    ("wdm_stream", _vp, [_vp]),
    ("wdm_set_profiling", _i32, [_vp, _i32]),
    ("wdm_set_profile_mask", _i32, [_vp, C.c_uint64]),
    ("wdm_get_profile", _i32, [_vp, _vp, _vp, _vp]),
    ("wdm_num_passes", _i32, []),
    ("wdm_pass_name", C.c_char_p, [_i32]),
    ("wdm_launch_count", _i64, [_vp]),
    ("wdm_selftest_sincos", _i32, [_vp, _vp, _i64]),
    ("wdm_selftest_bounded_wait", _i32, [_i64, C.POINTER(_i32), C.POINTER(_i64)]),
    ("wdm_get_line_schedule", _i32, [_vp, _vp, _vp]),
    ("wdm_step_graph", _i32, [_vp, _i32, _d, _i32]),
    ("wdm_adjoint", _i32, [_vp, _i32, _d, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _vp]),
    ("wdm_group_create", _i32, [_vp, _i32, C.POINTER(_vp)]),
    ("wdm_group_destroy", _i32, [_vp]),
    ("wdm_group_step", _i32, [_vp, _i32, _vp, _i32]),
    ("wdm_group_step_async", _i32, [_vp, _i32, _vp, _i32]),
    ("wdm_group_stream", _vp, [_vp]),
    ("wdm_group_schedule", _i32, [_vp, C.POINTER(_i32), _vp]),
    ("wdm_group_launch_count", _i64, [_vp]),
]

_lib = None


class WdmError(RuntimeError):
    """A libwavedm call returned a non-OK status."""

    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def load(path: str | None = None):
    """Load libwavedm.so (once) and declare every entry point's signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("WDM_LIB_PATH") or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            f"libwavedm.so not found at {p}: build it with `python wavedm.jl_gb300/build.py` "
            "(there is no CPU fallback)")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status, ctx=None):
    if status != WDM_OK:
        msg = load().wdm_last_error(ctx)
        raise WdmError(status, msg.decode() if msg else "")
    return status
