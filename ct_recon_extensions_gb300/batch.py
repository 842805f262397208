"""Batched uneven fan-beam FBP (ctr_fbp_fan_plan_* of the C ABI).

``FanFBPBatch`` reconstructs a list of fan-beam sinograms whose geometries all
differ (image size, views, channels): fan weighting -> ramp filter -> bp_fan_2d
for every item in one batched filter launch plus one persistent
backprojection launch, replayed from a CUDA graph; the tile shape and
view-block depth are chosen by timing the candidates on the batch at creation.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import FanBpParam, PlanInfo


class FanFBPBatch:
    def __init__(self, geoms, weighting: str = "fan", autotune: bool = True, graph: bool = True):
        """geoms: list of dicts with the FanBackprojection2DParam fields
        (ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
        offset_y, dso, dsd[, fov])."""
        self.geoms = [dict(g) for g in geoms]
        arr = (FanBpParam * len(geoms))()
        for i, g in enumerate(geoms):
            arr[i] = FanBpParam(g["ns"], g["na"], g["ds"], g["orbit"], g.get("offset_s", 0.0),
                                g.get("orbit_start", 0.0), g["nx"], g["ny"], g["dx"], g["dy"],
                                g.get("offset_x", 0.0), g.get("offset_y", 0.0), g["dso"], g["dsd"],
                                g.get("fov", -1.0))
        flags = (_lib.CTR_PLAN_AUTOTUNE if autotune else 0) | (_lib.CTR_PLAN_GRAPH if graph else 0)
        wt = {"fan": 1, "flat": 2}[weighting]
        self._plan = ctypes.c_void_p()
        _lib.call("ctr_fbp_fan_plan_create", arr, len(geoms), wt, flags, ctypes.byref(self._plan))
        self._ptr_in = (ctypes.c_void_p * len(geoms))()
        self._ptr_out = (ctypes.c_void_p * len(geoms))()

    def info(self) -> dict:
        inf = PlanInfo()
        _lib.call("ctr_fbp_fan_plan_info", self._plan, ctypes.byref(inf))
        return {f: getattr(inf, f) for f, _ in PlanInfo._fields_}

    def run(self, sinos, out=None):
        """sinos: list of CUDA float32 tensors [na][ns]; returns (or fills) a
        list of [ny][nx] images."""
        if len(sinos) != len(self.geoms):
            raise ValueError("one sinogram per plan item")
        if out is None:
            out = [torch.empty((g["ny"], g["nx"]), dtype=torch.float32, device=s.device)
                   for g, s in zip(self.geoms, sinos)]
        for i, (s, o, g) in enumerate(zip(sinos, out, self.geoms)):
            if s.dtype != torch.float32 or not s.is_cuda or not s.is_contiguous():
                raise ValueError("sinograms must be contiguous float32 CUDA tensors")
            if tuple(s.shape[-2:]) != (g["na"], g["ns"]) or tuple(o.shape[-2:]) != (g["ny"], g["nx"]):
                raise ValueError(f"item {i}: shape does not match its geometry")
            self._ptr_in[i] = s.data_ptr()
            self._ptr_out[i] = o.data_ptr()
        _lib.call("ctr_fbp_fan_plan_run", self._plan, self._ptr_in, self._ptr_out,
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        return out

    def close(self):
        if self._plan:
            _lib.load().ctr_fbp_fan_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
