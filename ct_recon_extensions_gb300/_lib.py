"""ctypes binding of libctrecon_gb300.so (the C ABI in include/ctrecon_gb300.h).

The library is loaded from this package directory only; there is no other
implementation to fall back to.  ``load()`` raises ``CtrLibraryError`` when it
is missing, which makes every operator fail loudly.
"""
from __future__ import annotations

import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libctrecon_gb300.so")

c_uint = ctypes.c_uint
c_int = ctypes.c_int
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_char_p = ctypes.c_char_p

CTR_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported", 3: "CUDA runtime error",
          4: "no usable sm_103 device", 5: "kernel self-check failed"}


class CtrLibraryError(RuntimeError):
    pass


class CtrError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(status, status)} ({msg})")
        self.status = status


# ---- parameter structs (include/ctrecon_gb300.h) --------------------------
class FanWeightingParam(ctypes.Structure):
    _fields_ = [("ns", c_uint), ("nrow", c_uint), ("ds", c_double), ("offset", c_double),
                ("dso", c_double), ("dsd", c_double), ("type", c_int)]


class FilterParam(ctypes.Structure):
    _fields_ = [("ns", c_uint), ("nrow", c_uint), ("ds", c_double), ("dsd", c_double),
                ("type", c_int), ("window", c_int)]


class FanBpParam(ctypes.Structure):
    _fields_ = [("ns", c_uint), ("na", c_uint), ("ds", c_double), ("orbit", c_double),
                ("offset_s", c_double), ("orbit_start", c_double), ("nx", c_uint),
                ("ny", c_uint), ("dx", c_double), ("dy", c_double), ("offset_x", c_double),
                ("offset_y", c_double), ("dso", c_double), ("dsd", c_double), ("fov", c_double)]


class FanBpAngleParam(ctypes.Structure):
    _fields_ = [("ns", c_uint), ("na", c_uint), ("ds", c_double), ("offset_s", c_double),
                ("nx", c_uint), ("ny", c_uint), ("dx", c_double), ("dy", c_double),
                ("offset_x", c_double), ("offset_y", c_double), ("dso", c_double),
                ("dsd", c_double), ("fov", c_double)]


class ParParam(ctypes.Structure):
    _fields_ = [("ns", c_uint), ("na", c_uint), ("ds", c_double), ("orbit", c_double),
                ("offset_s", c_double), ("orbit_start", c_double), ("nx", c_uint),
                ("ny", c_uint), ("dx", c_double), ("dy", c_double), ("offset_x", c_double),
                ("offset_y", c_double), ("fov", c_double)]


class HelicalParam(ctypes.Structure):
    _fields_ = [("ns", c_uint), ("nt", c_uint), ("na", c_uint), ("ds", c_double), ("dt", c_double),
                ("offset_s", c_double), ("offset_t", c_double), ("orbit_start", c_double),
                ("orbit", c_double), ("couch_begin", c_double), ("couch_mov", c_double),
                ("view_per_rot", c_uint), ("nz", c_uint), ("dz", c_double), ("z0", c_double),
                ("thickness", c_double), ("dso", c_double), ("dsd", c_double)]


CTR_HELICAL_360, CTR_HELICAL_180 = 0, 1
CTR_HELICAL_NO_ROWS, CTR_HELICAL_OUTSIDE, CTR_HELICAL_BAD_TABLE, CTR_HELICAL_NO_VIEWS = 1, 2, 4, 8


class PlanInfo(ctypes.Structure):
    _fields_ = [("n_items", c_int), ("work_items", ctypes.c_longlong), ("tile_rows", c_int),
                ("view_block", c_int), ("ctas", c_int), ("autotuned", c_int),
                ("tuned_ms", c_double), ("graph", c_int), ("workspace_bytes", ctypes.c_ulonglong),
                ("launches_per_run", ctypes.c_longlong)]


CTR_PLAN_AUTOTUNE = 1
CTR_PLAN_GRAPH = 2

_P = c_void_p  # device pointers and the stream travel as void*
_S = ctypes.POINTER

# name -> argument types (return type is int unless listed in _RESTYPES)
PROTOTYPES = {
    "ctr_status_string": [c_int],
    "ctr_last_error": [],
    "ctr_version": [],
    "ctr_device_check": [],
    "ctr_kernel_flags": [ctypes.POINTER(c_uint), c_int],
    "ctr_selftest_wait_timeout": [ctypes.c_ulonglong, _P],
    "ctr_ramp_filter_prep": [_S(FilterParam), _P, _P],
    "ctr_bp_fan_2d_prep": [_S(FanBpParam), _P, _P, _P, _P],
    "ctr_bp_fan_2d_angle_prep": [_S(FanBpAngleParam), _P, _P, _P, _P, _P],
    "ctr_bp_par_2d_prep": [_S(ParParam), _P, _P, _P, _P],
    "ctr_fp_par_2d_prep": [_S(ParParam), _P, _P, _P, _P],
    "ctr_fp_par_2d_grad_prep": [_S(ParParam), _P, _P, _P, _P],
    "ctr_fbp_fan_plan_create": [_S(FanBpParam), c_int, c_int, c_int, ctypes.POINTER(c_void_p)],
    "ctr_fbp_fan_plan_run": [c_void_p, ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p), _P],
    "ctr_fbp_fan_plan_info": [c_void_p, _S(PlanInfo)],
    "ctr_fbp_fan_plan_destroy": [c_void_p],
    "ctr_fp_par_2d_f32_noalloc": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
    "ctr_fp_par_2d_plan_create": [_S(ParParam), _P, _P, _P, c_int, ctypes.POINTER(c_void_p), _P],
    "ctr_fp_par_2d_plan_run": [c_void_p, _P, _P, c_int, _P],
    "ctr_fp_par_2d_plan_destroy": [c_void_p],
    "ctr_bp_par_2d_plan_create": [_S(ParParam), _P, _P, c_int, ctypes.POINTER(c_void_p), _P],
    "ctr_bp_fan_2d_plan_create": [_S(FanBpParam), _P, _P, _P, c_int, ctypes.POINTER(c_void_p), _P],
    "ctr_bp_plan_run": [c_void_p, _P, _P, c_int, _P],
    "ctr_bp_plan_run_grad": [c_void_p, _P, _P, c_int, _P],
    "ctr_bp_plan_destroy": [c_void_p],
    "ctr_fp_par_2d_cast_prep": [_S(ParParam), c_double, _P, _P, _P, _P],
    "ctr_fp_par_2d_dd_prep": [_S(ParParam), _P, _P, _P, _P],
    "ctr_fp_par_2d_dd_grad_prep": [_S(ParParam), _P, _P, _P, _P],
    "ctr_ramp_filter_tc_create": [_S(FilterParam), _P, _S(FanWeightingParam), c_int, c_int, c_int,
                                  ctypes.POINTER(c_void_p), _P],
    "ctr_ramp_filter_tc_run": [c_void_p, c_int, _P, _P, c_int, _P],
    "ctr_ramp_filter_tc_info": [c_void_p, ctypes.POINTER(ctypes.c_ulonglong),
                                ctypes.POINTER(ctypes.c_ulonglong)],
    "ctr_ramp_filter_tc_destroy": [c_void_p],
    "ctr_helical_interpolation_table_bytes": [_S(HelicalParam)],
    "ctr_helical_interpolation_prep": [_S(HelicalParam), c_int, _P, _P],
}

# storage types of ctr_ramp_filter_tc_run's input
CTR_DTYPE_F32, CTR_DTYPE_BF16, CTR_DTYPE_F16 = 0, 1, 2
for _t in ("f32", "f64"):
    PROTOTYPES.update({
        f"ctr_fan_weighting_{_t}": [_S(FanWeightingParam), _P, _P, c_int, _P],
        f"ctr_fan_weighting_grad_{_t}": [_S(FanWeightingParam), _P, _P, c_int, _P],
        f"ctr_ramp_filter_{_t}": [_S(FilterParam), _P, _P, _P, c_int, _P],
        f"ctr_ramp_filter_grad_{_t}": [_S(FilterParam), _P, _P, _P, c_int, _P],
        f"ctr_bp_fan_2d_{_t}": [_S(FanBpParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_bp_fan_2d_grad_{_t}": [_S(FanBpParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_bp_fan_2d_angle_{_t}": [_S(FanBpAngleParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_bp_fan_2d_angle_grad_{_t}": [_S(FanBpAngleParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_bp_par_2d_{_t}": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_bp_par_2d_grad_{_t}": [_S(ParParam), _P, _P, _P, _P, c_int, _P],
        f"ctr_bp_par_2d_sv_{_t}": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_fp_par_2d_{_t}": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_fp_par_2d_grad_{_t}": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_fp_par_2d_cast_{_t}": [_S(ParParam), c_double, _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_fp_par_2d_dd_{_t}": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_fp_par_2d_dd_grad_{_t}": [_S(ParParam), _P, _P, _P, _P, _P, c_int, _P],
        f"ctr_helical_interpolation_360_{_t}": [_S(HelicalParam), _P, _P, _P, _P, c_int, _P],
        f"ctr_helical_interpolation_180_{_t}": [_S(HelicalParam), _P, _P, _P, _P, c_int, _P],
    })
_RESTYPES = {"ctr_status_string": c_char_p, "ctr_last_error": c_char_p,
             "ctr_helical_interpolation_table_bytes": ctypes.c_size_t}

_lock = threading.Lock()
_lib = None


def load() -> ctypes.CDLL:
    """Load the library (once) and attach the prototypes."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise CtrLibraryError(
                f"{LIB_PATH} is missing: build it with `python -m ct_recon_extensions_gb300.build` "
                "(there is no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, args in PROTOTYPES.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = _RESTYPES.get(name, c_int)
        _lib = lib
    return _lib


def exported_names():
    return list(PROTOTYPES)


def check(status: int, where: str) -> None:
    if status != CTR_OK:
        msg = load().ctr_last_error()
        raise CtrError(status, where, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    """Call an entry point and raise CtrError on a nonzero status."""
    check(getattr(load(), name)(*args), name)
