"""numpy front end over the numpy-extension ABI of libctrecon_gb300.

Mirrors the reference's numpy_ext/np_ctrecon.py: the same ctypes prototypes
(with ``restype`` set, so the bools come back as bools; the reference sets a
misspelled ``rettype`` attribute, np_ctrecon.py:24) and the same
``FanFBP2DAngle`` class -- fan weighting (in place on the caller's array, as
the reference does), equiangular ramp filter and angle-list backprojection,
the result scaled by the orbit step (np_ctrecon.py:85-99).  Arrays are float64
host arrays; the work runs on the GPU chosen by ``param["device"]`` (>= 0).
"""
from __future__ import annotations

import numpy as np
import numpy.ctypeslib as npct

from ._lib import LIB_PATH, CtrLibraryError

_array1dd = npct.ndpointer(np.double, 1, flags="C")
_array2dd = npct.ndpointer(np.double, 2, flags="C")
_uint = npct.ctypes.c_uint
_int = npct.ctypes.c_int
_double = npct.ctypes.c_double
_bool = npct.ctypes.c_bool

_lib = None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    import os
    if not os.path.exists(LIB_PATH):
        raise CtrLibraryError(f"{LIB_PATH} is missing: build it with `python -m ct_recon_extensions_gb300.build`")
    lib = npct.load_library(os.path.basename(LIB_PATH), os.path.dirname(LIB_PATH))
    sig = {
        "set_device": (_bool, [_int]),
        "clear": (_bool, []),
        "fan_weighting_create": (_int, [_uint, _uint, _double, _double, _double, _double, _int]),
        "fan_weighting_run": (_bool, [_int, _array2dd, _array2dd]),
        "fan_weighting_destroy": (_bool, [_int]),
        "ramp_filter_create": (_int, [_uint, _uint, _double, _double, _int]),
        "ramp_filter_run": (_bool, [_int, _array2dd, _array2dd]),
        "ramp_filter_destroy": (_bool, [_int]),
        "fan_bp_2d_angle_create": (_int, [_array1dd, _uint, _uint, _double, _double, _uint, _uint,
                                          _double, _double, _double, _double, _double, _double,
                                          _double]),
        "fan_bp_2d_angle_run": (_bool, [_int, _array2dd, _array2dd]),
        "fan_bp_2d_angle_destroy": (_bool, [_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib.ctr_last_error.restype = npct.ctypes.c_char_p
    _lib = lib
    return lib


def last_error() -> str:
    return _load().ctr_last_error().decode()


class FanFBP2DAngle:
    """Fan-beam FBP over an explicit angle list (reference np_ctrecon.py:66-99).

    param keys: device, ns, na, ds, offset_s, dso, dsd, angles (float64[na]),
    nx, ny, dx, dy, offset_x, offset_y, fov, orbit.
    """

    def __init__(self, param: dict):
        lib = _load()
        self._param = param
        itype = 1
        if not lib.set_device(param["device"]):
            raise RuntimeError(f"set_device failed: {last_error()}")
        self._fw_handle = lib.fan_weighting_create(param["ns"], param["na"], param["ds"],
                                                   param["offset_s"], param["dso"], param["dsd"],
                                                   itype)
        self._flt_handle = lib.ramp_filter_create(param["ns"], param["na"], param["ds"],
                                                  param["dsd"], itype)
        angles = np.ascontiguousarray(param["angles"], dtype=np.double)
        self._bp_handle = lib.fan_bp_2d_angle_create(angles, param["ns"], param["na"],
                                                     param["ds"], param["offset_s"], param["nx"],
                                                     param["ny"], param["dx"], param["dy"],
                                                     param["offset_x"], param["offset_y"],
                                                     param["dso"], param["dsd"], param["fov"])
        if self._bp_handle < 0:
            raise RuntimeError(f"fan_bp_2d_angle_create failed: {last_error()}")

    def __del__(self):
        lib = _lib
        if lib is None:
            return
        for f, h in ((lib.fan_weighting_destroy, "_fw_handle"), (lib.ramp_filter_destroy, "_flt_handle"),
                     (lib.fan_bp_2d_angle_destroy, "_bp_handle")):
            if hasattr(self, h):
                f(getattr(self, h))

    def run(self, proj):
        lib = _load()
        if proj.dtype != np.double:
            proj = proj.astype(np.double)
        proj = np.ascontiguousarray(proj)
        recon = np.zeros([self._param["ny"], self._param["nx"]], dtype=np.double)
        na, ns = proj.shape
        if na != self._param["na"] or ns != self._param["ns"]:
            raise RuntimeError("Input shape not available!")
        filtered = np.zeros([self._param["na"], self._param["ns"]], dtype=np.double)
        if not lib.fan_weighting_run(self._fw_handle, proj, proj):
            raise RuntimeError(f"Fan weighting failed! {last_error()}")
        if not lib.ramp_filter_run(self._flt_handle, proj, filtered):
            raise RuntimeError(f"Ramp filter failed! {last_error()}")
        if not lib.fan_bp_2d_angle_run(self._bp_handle, filtered, recon):
            raise RuntimeError(f"Backprojection failed! {last_error()}")
        return recon * self._param["orbit"]
