"""PyTorch front end of the GB300 CT reconstruction path.

Mirrors the reference's TensorFlow front end (python/tf_ctrecon.py): the same
function names, argument names, defaults and tensor layout (NHWC with C = 1,
i.e. [batch, height, width, 1]; [batch, H, W] and [H, W] are accepted too),
and the same gradient wiring (tf_ctrecon.py:29-108): every forward operator
is a ``torch.autograd.Function`` whose backward runs the operator's
hand-written adjoint kernel.

Each distinct set of attributes builds one operator object that owns its
FP64 geometry tables on the device, as the reference's TF op kernels keep
persistent buffers (tensorflow/bp_fan_2d_ops.cu:167-169).  Computation goes
through the C ABI of libctrecon_gb300.so on the current CUDA stream;
float32 tensors take the FP32 kernels, float64 tensors the FP64 kernels.
There is no CPU implementation: CPU tensors are rejected.
"""
from __future__ import annotations

import ctypes
import math
from functools import lru_cache

import torch

from . import _lib
from ._lib import (FanBpAngleParam, FanBpParam, FanWeightingParam, FilterParam, HelicalParam,
                   ParParam, call)

_FILTER_TYPES = {"par": 0, "fan": 1, "flat": 2}
_WEIGHT_TYPES = {"fan": 1, "flat": 2}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


def _sfx(t: torch.Tensor) -> str:
    if t.dtype == torch.float32:
        return "f32"
    if t.dtype == torch.float64:
        return "f64"
    raise TypeError(f"ct_recon operators take float32 or float64 tensors, got {t.dtype}")


def _as_batch(x: torch.Tensor, h: int, w: int, what: str):
    """[B,H,W,1] / [B,H,W] / [H,W] -> contiguous [B,H,W] and a function that
    restores the caller's layout for an output of shape [B,h2,w2]."""
    if not x.is_cuda:
        raise ValueError(f"{what}: input must be a CUDA tensor (no CPU implementation)")
    shape = tuple(x.shape)
    if x.dim() == 4:
        if shape[3] != 1:
            raise ValueError(f"{what}: channel dimension must be 1, got {shape}")
        xb = x.reshape(shape[0], shape[1], shape[2])
        restore = lambda y: y.unsqueeze(-1)  # noqa: E731
    elif x.dim() == 3:
        xb = x
        restore = lambda y: y  # noqa: E731
    elif x.dim() == 2:
        xb = x.unsqueeze(0)
        restore = lambda y: y[0]  # noqa: E731
    else:
        raise ValueError(f"{what}: expected [B,H,W,1], [B,H,W] or [H,W], got {shape}")
    if xb.shape[1] != h or xb.shape[2] != w:
        raise ValueError(f"{what}: expected height {h} and width {w}, got {shape}")
    return xb.contiguous(), restore


class _Tables:
    """Device FP64 tables of one operator, built once per device."""

    def __init__(self):
        self._per_device = {}

    def get(self, device, build):
        key = device.index if device.index is not None else torch.cuda.current_device()
        t = self._per_device.get(key)
        if t is None:
            with torch.cuda.device(key):
                t = build(torch.device("cuda", key))
            self._per_device[key] = t
        return t


# ---------------------------------------------------------------------------
# operator objects
# ---------------------------------------------------------------------------

class FanWeightingOp:
    """FanWeighting / FanWeightingGrad (reference include/fan_weighting.h)."""

    def __init__(self, ns, nrow, ds, offset=0.0, dso=-1.0, dsd=-1.0, type=1):
        if type not in (1, 2):
            raise ValueError("fan weighting type must be 1 ('fan') or 2 ('flat')")
        self.p = FanWeightingParam(ns, nrow, ds, offset, dso, dsd, type)
        self.ns, self.nrow = ns, nrow

    def _run(self, name, x):
        xb, restore = _as_batch(x, self.nrow, self.ns, name)
        out = torch.empty_like(xb)
        call(f"ctr_{name}_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(out), xb.shape[0],
             _stream())
        return restore(out)

    def forward(self, x):
        return self._run("fan_weighting", x)

    def adjoint(self, y):
        return self._run("fan_weighting_grad", y)


class RampFilterOp:
    """RampFilterPrep + RampFilter / RampFilterGrad (reference include/filter.h)."""

    def __init__(self, ns, nrow, ds, dsd=-1.0, type=0, window=0):
        if type not in (0, 1, 2):
            raise ValueError("ramp filter type must be 0 ('par'), 1 ('fan') or 2 ('flat')")
        self.p = FilterParam(ns, nrow, ds, dsd, type, window)
        self.ns, self.nrow = ns, nrow
        self._tables = _Tables()

    def taps(self, device):
        def build(dev):
            f = torch.empty(2 * self.ns + 1, dtype=torch.float64, device=dev)
            call("ctr_ramp_filter_prep", ctypes.byref(self.p), _ptr(f), _stream())
            return f
        return self._tables.get(device, build)

    def _run(self, name, x):
        xb, restore = _as_batch(x, self.nrow, self.ns, name)
        out = torch.empty_like(xb)
        call(f"ctr_{name}_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(self.taps(xb.device)),
             _ptr(out), xb.shape[0], _stream())
        return restore(out)

    def forward(self, x):
        return self._run("ramp_filter", x)

    def adjoint(self, y):
        return self._run("ramp_filter_grad", y)


class RampFilterTCOp:
    """The ramp filter, optionally after fan weighting, as a Toeplitz GEMM on
    the BF16 tensor cores with split operands and FP32 accumulation:
    splits=3 (hi/mid/lo, six term products; FP32-grade) or splits=2 (hi/lo,
    three products; ~16 bits per operand).

    Input: float32, bfloat16 or float16 sinograms [B,nrow,ns]; output float32.
    No reference counterpart: it is the reduced-precision form of RampFilter
    (src/filter.cc:67-91), with FanWeighting (src/fan_weighting.cc:19-38)
    fused in front when `weighting` (a FanWeightingOp) is given.  One plan per
    (device, direction), grown to the largest batch seen."""

    _DTYPES = {torch.float32: _lib.CTR_DTYPE_F32, torch.bfloat16: _lib.CTR_DTYPE_BF16,
               torch.float16: _lib.CTR_DTYPE_F16}

    def __init__(self, ns, nrow, ds, dsd=-1.0, type=0, weighting=None, splits=3):
        if splits not in (2, 3):
            raise ValueError("splits must be 2 (hi/lo) or 3 (hi/mid/lo)")
        self.splits = splits
        self.ramp = RampFilterOp(ns, nrow, ds, dsd, type)
        if weighting is not None and (weighting.ns != ns or weighting.nrow != nrow):
            raise ValueError("weighting must have the filter's ns and nrow")
        self.weighting = weighting
        self.ns, self.nrow = ns, nrow
        self._plans = {}
        self._lib = _lib.load()

    def plan(self, device, grad=False, batch=1):
        dev = device.index if device.index is not None else torch.cuda.current_device()
        key = (dev, bool(grad))
        cur = self._plans.get(key)
        if cur is None or cur[1] < batch:
            with torch.cuda.device(dev):
                if cur is not None:
                    torch.cuda.current_stream().synchronize()
                    self._lib.ctr_ramp_filter_tc_destroy(cur[0])
                    del self._plans[key]
                h = ctypes.c_void_p()
                w = ctypes.byref(self.weighting.p) if self.weighting is not None else None
                call("ctr_ramp_filter_tc_create", ctypes.byref(self.ramp.p),
                     _ptr(self.ramp.taps(torch.device("cuda", dev))), w, int(grad), self.splits,
                     int(batch), ctypes.byref(h), _stream())
                self._plans[key] = (h, batch)
        return self._plans[key][0]

    def info(self, device):
        ws, fl = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        call("ctr_ramp_filter_tc_info", self.plan(device), ctypes.byref(ws), ctypes.byref(fl))
        return {"workspace_bytes": ws.value, "mma_flops_per_row": fl.value}

    def _run(self, x, grad):
        if x.dtype not in self._DTYPES:
            raise TypeError(f"ramp_filter_tc takes float32, bfloat16 or float16, got {x.dtype}")
        xb, restore = _as_batch(x, self.nrow, self.ns, "ramp_filter_tc")
        out = torch.empty(xb.shape, dtype=torch.float32, device=xb.device)
        h = self.plan(xb.device, grad, xb.shape[0])
        call("ctr_ramp_filter_tc_run", h, self._DTYPES[xb.dtype], _ptr(xb), _ptr(out), xb.shape[0],
             _stream())
        return restore(out)

    def forward(self, x):
        return self._run(x, False)

    def adjoint(self, y):
        if self.weighting is not None:
            raise ValueError("the adjoint of the fused weighting + filter is not provided; "
                             "use RampFilterTCOp without weighting and FanWeightingOp.adjoint")
        return self._run(y, True)

    def close(self):
        for h, _ in self._plans.values():
            self._lib.ctr_ramp_filter_tc_destroy(h)
        self._plans.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _BpPlans:
    """Per-device FP32 backprojection plans (ctr_bp_*_plan_create: the tables,
    the stream-split scratch and the per-(tile, view) constants kept), grown to
    the largest batch seen."""

    def __init__(self, create):
        self._create = create  # (device, max_batch) -> plan handle
        self._plans = {}
        self._lib = _lib.load()

    def get(self, device, batch):
        dev = device.index if device.index is not None else torch.cuda.current_device()
        cur = self._plans.get(dev)
        if cur is None or cur[1] < batch:
            with torch.cuda.device(dev):
                if cur is not None:
                    torch.cuda.current_stream().synchronize()
                    self._lib.ctr_bp_plan_destroy(cur[0])
                    del self._plans[dev]
                self._plans[dev] = (self._create(torch.device("cuda", dev), batch), batch)
        return self._plans[dev][0]

    def close(self):
        for h, _ in self._plans.values():
            self._lib.ctr_bp_plan_destroy(h)
        self._plans.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FanBackprojection2DOp:
    """FanBackprojection2DPixDriven{Prep,,GradPrep,Grad} (reference
    include/bp_fan_2d.h:151-225).  FP32 calls (forward and adjoint) run
    through a per-geometry plan (ctr_bp_fan_2d_plan_*)."""

    def __init__(self, ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                 offset_y, dso, dsd, fov=-1.0):
        self.p = FanBpParam(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                            offset_y, dso, dsd, fov)
        self.ns, self.na, self.nx, self.ny = ns, na, nx, ny
        self._tables = _Tables()
        self._plans = _BpPlans(self._make_plan)

    def _make_plan(self, device, batch):
        h = ctypes.c_void_p()
        call("ctr_bp_fan_2d_plan_create", ctypes.byref(self.p), *map(_ptr, self.tables(device)), int(batch),
             ctypes.byref(h), _stream())
        return h

    def plan(self, device, batch=1):
        """The FP32 forward's plan handle on `device` (for the C ABI)."""
        return self._plans.get(device, batch)

    def tables(self, device):
        def build(dev):
            xpos = torch.empty(self.nx, dtype=torch.float64, device=dev)
            ypos = torch.empty(self.ny, dtype=torch.float64, device=dev)
            sc = torch.empty(2 * self.na, dtype=torch.float64, device=dev)
            call("ctr_bp_fan_2d_prep", ctypes.byref(self.p), _ptr(xpos), _ptr(ypos), _ptr(sc),
                 _stream())
            return xpos, ypos, sc
        return self._tables.get(device, build)

    _fwd, _adj = "bp_fan_2d", "bp_fan_2d_grad"

    def forward(self, proj):
        xb, restore = _as_batch(proj, self.na, self.ns, self._fwd)
        img = torch.empty((xb.shape[0], self.ny, self.nx), dtype=xb.dtype, device=xb.device)
        if self._fwd == "bp_fan_2d" and xb.dtype == torch.float32:
            call("ctr_bp_plan_run", self._plans.get(xb.device, xb.shape[0]), _ptr(xb), _ptr(img),
                 xb.shape[0], _stream())
            return restore(img)
        t = self.tables(xb.device)
        call(f"ctr_{self._fwd}_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(img),
             *map(_ptr, t), xb.shape[0], _stream())
        return restore(img)

    def adjoint(self, img):
        xb, restore = _as_batch(img, self.ny, self.nx, self._adj)
        grad = torch.empty((xb.shape[0], self.na, self.ns), dtype=xb.dtype, device=xb.device)
        if self._adj == "bp_fan_2d_grad" and xb.dtype == torch.float32:
            call("ctr_bp_plan_run_grad", self._plans.get(xb.device, xb.shape[0]), _ptr(xb), _ptr(grad),
                 xb.shape[0], _stream())
            return restore(grad)
        t = self.tables(xb.device)
        call(f"ctr_{self._adj}_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(grad),
             *map(_ptr, t), xb.shape[0], _stream())
        return restore(grad)


class FanBackprojection2DAngleOp(FanBackprojection2DOp):
    """FanBackprojection2DAnglePixDriven{Prep,} (reference include/bp_fan_2d_angle.h):
    explicit view angles, no output scale."""

    _fwd, _adj = "bp_fan_2d_angle", "bp_fan_2d_angle_grad"

    def __init__(self, angles, ns, ds, offset_s, nx, ny, dx, dy, offset_x, offset_y, dso, dsd,
                 fov=-1.0):
        angles = torch.as_tensor(angles, dtype=torch.float64).flatten().cpu()
        na = int(angles.numel())
        self.angles = angles
        self.p = FanBpAngleParam(ns, na, ds, offset_s, nx, ny, dx, dy, offset_x, offset_y, dso,
                                 dsd, fov)
        self.ns, self.na, self.nx, self.ny = ns, na, nx, ny
        self._tables = _Tables()
        self._plans = None  # no plan form: the angle op's forward is unscaled

    def tables(self, device):
        def build(dev):
            ang = self.angles.to(dev)
            xpos = torch.empty(self.nx, dtype=torch.float64, device=dev)
            ypos = torch.empty(self.ny, dtype=torch.float64, device=dev)
            sc = torch.empty(2 * self.na, dtype=torch.float64, device=dev)
            call("ctr_bp_fan_2d_angle_prep", ctypes.byref(self.p), _ptr(ang), _ptr(xpos),
                 _ptr(ypos), _ptr(sc), _stream())
            return xpos, ypos, sc
        return self._tables.get(device, build)


class ParallelBackprojection2DOp:
    """ParallelBackprojection2DPixDriven (reference include/bp_par_2d.h) and its
    exact adjoint.  FP32 calls (forward and adjoint) run through a
    per-geometry plan (ctr_bp_par_2d_plan_*)."""

    def __init__(self, ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                 offset_y, fov=-1.0):
        self.p = ParParam(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                          offset_y, fov)
        self.ns, self.na, self.nx, self.ny = ns, na, nx, ny
        self._tables = _Tables()
        self._plans = _BpPlans(self._make_plan)

    def _make_plan(self, device, batch):
        h = ctypes.c_void_p()
        xcos, ysin = self.tables(device)
        call("ctr_bp_par_2d_plan_create", ctypes.byref(self.p), _ptr(xcos), _ptr(ysin), int(batch),
             ctypes.byref(h), _stream())
        return h

    def plan(self, device, batch=1):
        """The FP32 forward's plan handle on `device` (for the C ABI)."""
        return self._plans.get(device, batch)

    def tables(self, device):
        def build(dev):
            xcos = torch.empty((self.nx, self.na), dtype=torch.float64, device=dev)
            ysin = torch.empty((self.ny, self.na), dtype=torch.float64, device=dev)
            call("ctr_bp_par_2d_prep", ctypes.byref(self.p), _ptr(xcos), _ptr(ysin), None,
                 _stream())
            return xcos, ysin
        return self._tables.get(device, build)

    def forward(self, proj):
        xb, restore = _as_batch(proj, self.na, self.ns, "bp_par_2d")
        img = torch.empty((xb.shape[0], self.ny, self.nx), dtype=xb.dtype, device=xb.device)
        if xb.dtype == torch.float32:
            call("ctr_bp_plan_run", self._plans.get(xb.device, xb.shape[0]), _ptr(xb), _ptr(img),
                 xb.shape[0], _stream())
            return restore(img)
        xcos, ysin = self.tables(xb.device)
        call(f"ctr_bp_par_2d_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(img), _ptr(xcos),
             _ptr(ysin), None, xb.shape[0], _stream())
        return restore(img)

    def adjoint(self, img):
        xb, restore = _as_batch(img, self.ny, self.nx, "bp_par_2d_grad")
        grad = torch.empty((xb.shape[0], self.na, self.ns), dtype=xb.dtype, device=xb.device)
        if xb.dtype == torch.float32:
            call("ctr_bp_plan_run_grad", self._plans.get(xb.device, xb.shape[0]), _ptr(xb), _ptr(grad),
                 xb.shape[0], _stream())
            return restore(grad)
        xcos, ysin = self.tables(xb.device)
        call(f"ctr_bp_par_2d_grad_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(grad),
             _ptr(xcos), _ptr(ysin), xb.shape[0], _stream())
        return restore(grad)

    def single_view(self, proj):
        """ParallelSingleViewBp2DPixDriven: [B,na,ns] -> [B,ny,nx,na]."""
        xb, _ = _as_batch(proj, self.na, self.ns, "bp_par_2d_sv")
        img = torch.empty((xb.shape[0], self.ny, self.nx, self.na), dtype=xb.dtype,
                          device=xb.device)
        xcos, ysin = self.tables(xb.device)
        call(f"ctr_bp_par_2d_sv_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(img),
             _ptr(xcos), _ptr(ysin), None, xb.shape[0], _stream())
        return img


class ParallelProjection2DOp:
    """Parallel-beam forward projection, `method` as the reference op's attr:
    "raydriven" (ParallelProjection2DRayDriven{Prepare,,GradPrep,Grad},
    reference include/fp_par_2d.h:209-278), "raycasting"
    (ParallelProjection2DRayCasting{Prepare,}, include/fp_par_2d.h:155-203,
    step_size pixels per sample, rays bounded by the FoV circle of radius fov;
    no gradient, as in the reference) or "disdriven"
    (ParallelProjection2DDisDriven{Prep,,GradPrep,Grad},
    include/fp_par_2d.h:283-352; its adjoint is the reference's distance-driven
    grad, which the reference op registers as the gradient).  FP32 ray-driven
    calls run through a per-geometry plan (ctr_fp_par_2d_plan_*): the ray
    set-up runs once per device; a one-image call is one projector launch
    (which makes its own transposed copy), a batch the transposed copy and the
    projector."""

    def __init__(self, ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                 offset_y, fov=-1.0, method="raydriven", step_size=0.125):
        if method not in ("raydriven", "raycasting", "disdriven"):
            raise ValueError(f"projection method {method!r}: 'raydriven', 'raycasting' or "
                             "'disdriven'")
        if method == "raydriven" and nx != ny:
            raise ValueError("Image should have same width and height for raydriven projection.")
        if method == "disdriven" and nx != ny:
            raise ValueError("Image should have same width and height for distance-driven "
                             "projection.")
        self.method, self.step_size = method, float(step_size)
        self.p = ParParam(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                          offset_y, fov)
        self.ns, self.na, self.nx, self.ny = ns, na, nx, ny
        self._fwd_tables = _Tables()
        self._adj_tables = _Tables()
        self._plans = {}  # device -> (ctr_fp_plan handle, max batch): FP32 ray driven
        self._lib = _lib.load()

    def plan(self, device, batch=1):
        """The FP32 ray-driven projector's per-geometry plan on `device` (its
        ray tables built once from this op's tables), grown to the largest
        batch seen."""
        dev = device.index if device.index is not None else torch.cuda.current_device()
        cur = self._plans.get(dev)
        if cur is None or cur[1] < batch:
            with torch.cuda.device(dev):
                if cur is not None:
                    torch.cuda.current_stream().synchronize()
                    self._lib.ctr_fp_par_2d_plan_destroy(cur[0])
                    del self._plans[dev]
                h = ctypes.c_void_p()
                call("ctr_fp_par_2d_plan_create", ctypes.byref(self.p),
                     *map(_ptr, self.tables(torch.device("cuda", dev))), int(batch), ctypes.byref(h),
                     _stream())
                self._plans[dev] = (h, batch)
        return self._plans[dev][0]

    def close(self):
        for h, _ in self._plans.values():
            self._lib.ctr_fp_par_2d_plan_destroy(h)
        self._plans.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tables(self, device):
        if self.method == "raycasting":
            def build_cast(dev):
                sc = torch.empty((self.na, 2), dtype=torch.float64, device=dev)
                bg = torch.empty((self.na, self.ns, 2), dtype=torch.float64, device=dev)
                nst = torch.empty((self.na, self.ns), dtype=torch.int32, device=dev)
                call("ctr_fp_par_2d_cast_prep", ctypes.byref(self.p), self.step_size, _ptr(sc),
                     _ptr(bg), _ptr(nst), _stream())
                return sc, bg, nst
            return self._fwd_tables.get(device, build_cast)
        if self.method == "disdriven":
            def build_dd(dev):
                sc = torch.empty((self.na, 2), dtype=torch.float64, device=dev)
                bo = torch.empty((self.na, self.ns, 3), dtype=torch.float64, device=dev)
                ux = torch.empty(self.na, dtype=torch.int32, device=dev)
                call("ctr_fp_par_2d_dd_prep", ctypes.byref(self.p), _ptr(sc), _ptr(bo), _ptr(ux),
                     _stream())
                return sc, bo, ux
            return self._fwd_tables.get(device, build_dd)

        def build(dev):
            sc = torch.empty((self.na, 2), dtype=torch.float64, device=dev)
            bo = torch.empty((self.na, self.ns, 2), dtype=torch.float64, device=dev)
            ux = torch.empty(self.na, dtype=torch.int32, device=dev)
            call("ctr_fp_par_2d_prep", ctypes.byref(self.p), _ptr(sc), _ptr(bo), _ptr(ux),
                 _stream())
            return sc, bo, ux
        return self._fwd_tables.get(device, build)

    def grad_tables(self, device):
        name = "ctr_fp_par_2d_dd_grad_prep" if self.method == "disdriven" else "ctr_fp_par_2d_grad_prep"

        def build(dev):
            w = torch.empty(self.na, dtype=torch.float64, device=dev)
            pos = torch.empty((self.na, self.nx, 2), dtype=torch.float64, device=dev)
            ux = torch.empty(self.na, dtype=torch.int32, device=dev)
            call(name, ctypes.byref(self.p), _ptr(w), _ptr(pos), _ptr(ux), _stream())
            return w, pos, ux
        return self._adj_tables.get(device, build)

    def forward(self, img):
        xb, restore = _as_batch(img, self.ny, self.nx, "fp_par_2d")
        proj = torch.empty((xb.shape[0], self.na, self.ns), dtype=xb.dtype, device=xb.device)
        if self.method == "raycasting":
            call(f"ctr_fp_par_2d_cast_{_sfx(xb)}", ctypes.byref(self.p), self.step_size, _ptr(xb),
                 _ptr(proj), *map(_ptr, self.tables(xb.device)), xb.shape[0], _stream())
        elif self.method == "disdriven":
            call(f"ctr_fp_par_2d_dd_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(proj),
                 *map(_ptr, self.tables(xb.device)), xb.shape[0], _stream())
        elif xb.dtype == torch.float32 and xb.data_ptr() % 16 == 0 and self.nx <= 8192:
            call("ctr_fp_par_2d_plan_run", self.plan(xb.device, xb.shape[0]), _ptr(xb), _ptr(proj),
                 xb.shape[0], _stream())
        else:
            call(f"ctr_fp_par_2d_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(proj),
                 *map(_ptr, self.tables(xb.device)), xb.shape[0], _stream())
        return restore(proj)

    def adjoint(self, proj):
        if self.method == "raycasting":
            raise NotImplementedError("Gradient is not yet implemented for raycasting forward "
                                      "projector.")
        xb, restore = _as_batch(proj, self.na, self.ns, "fp_par_2d_grad")
        img = torch.empty((xb.shape[0], self.ny, self.nx), dtype=xb.dtype, device=xb.device)
        kind = "dd_grad" if self.method == "disdriven" else "grad"
        call(f"ctr_fp_par_2d_{kind}_{_sfx(xb)}", ctypes.byref(self.p), _ptr(xb), _ptr(img),
             *map(_ptr, self.grad_tables(xb.device)), xb.shape[0], _stream())
        return restore(img)


class HelicalInterpolationOp:
    """HelicalInterpolation360 / HelicalInterpolation180 (reference
    include/helical_interpolation.h:17-116, src/helical_interpolation.cc:80-370;
    CPU-only there): helical sinograms ``[na][nt][ns]`` (view, detector row,
    channel; optionally with a leading batch dimension) to one fan-beam
    sinogram per slice, ``[nz][view_per_rot][ns]``.  Bit-identical to the
    reference.  Raises RuntimeError with the reference's messages where it
    throws ("View not enough for this slice!", "No row data available!")."""

    _METHODS = {"360": _lib.CTR_HELICAL_360, "180": _lib.CTR_HELICAL_180}

    def __init__(self, ns, nt, na, ds, dt, offset_s, offset_t, orbit_start, orbit, couch_begin,
                 couch_mov, view_per_rot, nz, dz, z0, thickness, dso, dsd, method="360"):
        if str(method) not in self._METHODS:
            raise ValueError("helical interpolation method must be '360' or '180'")
        self.method = str(method)
        self.p = HelicalParam(ns, nt, na, ds, dt, offset_s, offset_t, orbit_start, orbit,
                              couch_begin, couch_mov, view_per_rot, nz, dz, z0, thickness, dso,
                              dsd)
        self.shape_in = (na, nt, ns)
        self.shape_out = (nz, view_per_rot, ns)
        self._tables = _Tables()

    def table(self, device):
        def build(dev):
            n = _lib.load().ctr_helical_interpolation_table_bytes(ctypes.byref(self.p))
            t = torch.empty(n, dtype=torch.uint8, device=dev)
            call("ctr_helical_interpolation_prep", ctypes.byref(self.p),
                 self._METHODS[self.method], _ptr(t), _stream())
            return t
        return self._tables.get(device, build)

    def launch(self, proj, out, status):
        """Stream-ordered launch of ``proj`` [B, na, nt, ns] into ``out``
        [B, nz, vpr, ns]; ORs the CTR_HELICAL_* bits into the int32 device tensor
        ``status`` of B*nz words, one per item and slice."""
        call(f"ctr_helical_interpolation_{self.method}_{_sfx(proj)}", ctypes.byref(self.p),
             _ptr(proj), _ptr(out), _ptr(self.table(proj.device)), _ptr(status), proj.shape[0],
             _stream())

    @staticmethod
    def raise_status(words):
        """The reference's exception for one item's per-slice status words: it
        processes slices in order and throws at the first problem."""
        for w in words:
            if w & _lib.CTR_HELICAL_BAD_TABLE:
                raise RuntimeError("helical_interpolation: table prepared for another geometry")
            if w & _lib.CTR_HELICAL_NO_VIEWS:
                raise RuntimeError("View not enough for this slice!")
            if w & _lib.CTR_HELICAL_NO_ROWS:
                raise RuntimeError("No row data available!")

    def forward(self, proj):
        if not proj.is_cuda:
            raise ValueError("helical_interpolation: input must be a CUDA tensor (no CPU implementation)")
        single = proj.dim() == 3
        xb = (proj.unsqueeze(0) if single else proj).contiguous()
        if xb.dim() != 4 or tuple(xb.shape[1:]) != self.shape_in:
            raise ValueError(f"helical_interpolation: expected [B,] {self.shape_in}, got {tuple(proj.shape)}")
        nz = self.shape_out[0]
        out = torch.empty((xb.shape[0],) + self.shape_out, dtype=xb.dtype, device=xb.device)
        status = torch.zeros(xb.shape[0] * nz, dtype=torch.int32, device=xb.device)
        self.launch(xb, out, status)
        words = status.cpu().tolist()
        for b in range(xb.shape[0]):
            self.raise_status(words[b * nz:(b + 1) * nz])
        if any(w & _lib.CTR_HELICAL_OUTSIDE for w in words):
            import warnings
            warnings.warn("helical_interpolation: a 180LI complementary sample lies before the "
                          "first view and was read as 0 (the reference reads out of bounds)")
        return out[0] if single else out


def helical_interpolation(proj, ns, nt, na, ds, dt, view_per_rot, couch_mov, nz, dz, z0,
                          thickness, dso, dsd, offset_s=0.0, offset_t=0.0, orbit_start=0.0,
                          orbit=None, couch_begin=0.0, method="360"):
    """Rebin a helical sinogram into per-slice fan sinograms (360LI or 180LI);
    ``orbit`` defaults to 2*pi / view_per_rot."""
    if orbit is None:
        orbit = 2 * math.pi / view_per_rot
    op = HelicalInterpolationOp(ns, nt, na, ds, dt, offset_s, offset_t, orbit_start, orbit,
                                couch_begin, couch_mov, view_per_rot, nz, dz, z0, thickness, dso,
                                dsd, method)
    return op.forward(proj)


# ---------------------------------------------------------------------------
# autograd: forward op + adjoint kernel as backward
# ---------------------------------------------------------------------------

class _LinearOp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        ctx.op = op
        return op.forward(x)

    @staticmethod
    def backward(ctx, g):
        return ctx.op.adjoint(g.contiguous()), None


class _AdjointOp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        ctx.op = op
        return op.adjoint(x)

    @staticmethod
    def backward(ctx, g):
        return ctx.op.forward(g.contiguous()), None


def apply(op, x):
    """Differentiable forward of an operator object."""
    return _LinearOp.apply(x, op)


def apply_adjoint(op, x):
    """Differentiable adjoint of an operator object."""
    return _AdjointOp.apply(x, op)


# ---------------------------------------------------------------------------
# tf_ctrecon.py-compatible functions (attributes are (y, x) ordered there)
# ---------------------------------------------------------------------------

@lru_cache(maxsize=256)
def _fan_weighting_op(ns, nrow, ds, offset, dso, dsd, tp):
    return FanWeightingOp(ns, nrow, ds, offset, dso, dsd, _WEIGHT_TYPES[tp])


@lru_cache(maxsize=256)
def _ramp_op(ns, nrow, ds, dsd, ftype):
    return RampFilterOp(ns, nrow, ds, dsd, _FILTER_TYPES[ftype])


@lru_cache(maxsize=256)
def _fan_bp_op(*args):
    return FanBackprojection2DOp(*args)


@lru_cache(maxsize=256)
def _par_bp_op(*args):
    return ParallelBackprojection2DOp(*args)


@lru_cache(maxsize=256)
def _par_fp_op(*args):
    return ParallelProjection2DOp(*args)


def _par_args(img_shape, img_space, img_offset, proj_shape, channel_space, channel_offset,
              orbit_start, orbit, fov):
    # reference tensorflow/bp_par_2d_ops.cu: (nx, ny) = (img_shape[1], img_shape[0])
    return (int(proj_shape[1]), int(proj_shape[0]), float(channel_space), float(orbit),
            float(channel_offset), float(orbit_start), int(img_shape[1]), int(img_shape[0]),
            float(img_space[1]), float(img_space[0]), float(img_offset[1]), float(img_offset[0]),
            float(fov))


def ramp_filter(proj, n_channel, n_row, channel_space, dsd=-1, type="par", window="None"):
    """Ramp filter (tf_ctrecon.py:112-129); differentiable, backward = correlation."""
    if type not in _FILTER_TYPES:
        raise ValueError("Unrecognised geometry type. Only par, fan or flat are available for ramp filter.")
    return apply(_ramp_op(int(n_channel), int(n_row), float(channel_space), float(dsd), type), proj)


def ramp_filter_grad(grad_in, n_channel, n_row, channel_space, dsd=-1, type="par", window="None"):
    return apply_adjoint(_ramp_op(int(n_channel), int(n_row), float(channel_space), float(dsd), type),
                         grad_in)


def fan_weighting(proj, proj_shape, channel_space, channel_offset=0, dso=1000, dsd=1500, tp="fan"):
    """Fan / flat pre-weighting (tf_ctrecon.py:268-281)."""
    if tp not in _WEIGHT_TYPES:
        raise ValueError("fan weighting tp must be 'fan' or 'flat'")
    op = _fan_weighting_op(int(proj_shape[1]), int(proj_shape[0]), float(channel_space),
                           float(channel_offset), float(dso), float(dsd), tp)
    return apply(op, proj)


def fan_weighting_grad(grad_in, proj_shape, channel_space, channel_offset=0, dso=1000, dsd=1500,
                       tp="fan"):
    op = _fan_weighting_op(int(proj_shape[1]), int(proj_shape[0]), float(channel_space),
                           float(channel_offset), float(dso), float(dsd), tp)
    return apply_adjoint(op, grad_in)


def parallel_backprojection_2d(proj, img_shape, img_space, proj_shape, channel_space,
                               img_offset=(0, 0), channel_offset=0, orbit_start=0,
                               orbit=math.pi / 180, fov=-1, method="pixdriven"):
    """Pixel-driven parallel BP (tf_ctrecon.py:149-170)."""
    if method != "pixdriven":
        raise ValueError("Unrecognised backprojection method. Only pixdriven is available now.")
    op = _par_bp_op(*_par_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, fov))
    return apply(op, proj)


def parallel_backprojection_2d_grad(grad_in, img_shape, img_space, proj_shape, channel_space,
                                    img_offset=(0, 0), channel_offset=0, orbit_start=0,
                                    orbit=math.pi / 180, fov=-1, method="pixdriven"):
    op = _par_bp_op(*_par_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, fov))
    return apply_adjoint(op, grad_in)


def parallel_projection_2d(img, img_shape, img_space, proj_shape, channel_space,
                           img_offset=(0, 0), channel_offset=0, orbit_start=0,
                           orbit=math.pi / 180, fov=-1, method="raydriven"):
    """Ray-driven parallel forward projection (tf_ctrecon.py:173-195)."""
    op = _par_fp_op(*_par_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, fov), method)
    return apply(op, img)


def parallel_projection_2d_grad(grad_in, img_shape, img_space, proj_shape, channel_space,
                                img_offset=(0, 0), channel_offset=0, orbit_start=0,
                                orbit=math.pi / 180, fov=-1, method="raydriven"):
    op = _par_fp_op(*_par_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, fov), method)
    return apply_adjoint(op, grad_in)


def parallel_single_view_bp_2d(proj, img_shape, img_space, proj_shape, channel_space,
                               img_offset=(0, 0), channel_offset=0, orbit_start=0,
                               orbit=math.pi / 180, fov=-1, method="pixdriven"):
    """Single-view BP (tf_ctrecon.py:198-219): [B,na,ns(,1)] -> [B,ny,nx,na]."""
    if method != "pixdriven":
        raise ValueError("Unrecognised backprojection method. Only pixdriven is available now.")
    op = _par_bp_op(*_par_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, fov))
    return op.single_view(proj)


def _fan_args(img_shape, img_space, img_offset, proj_shape, channel_space, channel_offset,
              orbit_start, orbit, dso, dsd, fov):
    # reference tensorflow/bp_fan_2d_ops.cu:156-159
    return (int(proj_shape[1]), int(proj_shape[0]), float(channel_space), float(orbit),
            float(channel_offset), float(orbit_start), int(img_shape[1]), int(img_shape[0]),
            float(img_space[1]), float(img_space[0]), float(img_offset[1]), float(img_offset[0]),
            float(dso), float(dsd), float(fov))


def fan_backprojection_2d(proj, img_shape, img_space, proj_shape, channel_space,
                          img_offset=(0, 0), channel_offset=0, orbit_start=0,
                          orbit=math.pi / 180, dso=1000, dsd=1500, fov=-1, method="pixdriven"):
    """Pixel-driven fan BP (tf_ctrecon.py:221-244)."""
    if method != "pixdriven":
        raise ValueError("Unrecognised backprojection method. Only pixdriven is available for fan geometry now.")
    op = _fan_bp_op(*_fan_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, dso, dsd, fov))
    return apply(op, proj)


def fan_backprojection_2d_grad(grad_in, img_shape, img_space, proj_shape, channel_space,
                               img_offset=(0, 0), channel_offset=0, orbit_start=0,
                               orbit=math.pi / 180, dso=1000, dsd=1500, fov=-1,
                               method="pixdriven"):
    """Adjoint of fan_backprojection_2d (tf_ctrecon.py:246-266)."""
    op = _fan_bp_op(*_fan_args(img_shape, img_space, img_offset, proj_shape, channel_space,
                               channel_offset, orbit_start, orbit, dso, dsd, fov))
    return apply_adjoint(op, grad_in)


def fan_projection_2d(img, img_shape, img_space, proj_shape, channel_space, img_offset=(0, 0),
                      channel_offset=0, orbit_start=0, orbit=math.pi / 180, dso=1000, dsd=1500,
                      fov=-1):
    """Matched fan-beam forward projector (the reference has no fan projector):
    the exact adjoint of the pixel-driven fan_backprojection_2d, so that
    (fan_projection_2d, fan_backprojection_2d) is an exact A / A^T pair for
    fan-beam iterative reconstruction.  Differentiable; its backward is the
    backprojection.  img: [B, ny, nx, 1] -> [B, na, ns, 1]."""
    return fan_backprojection_2d_grad(img, img_shape, img_space, proj_shape, channel_space,
                                      img_offset, channel_offset, orbit_start, orbit, dso, dsd, fov)


def fan_backprojection_2d_angle(proj, angles, img_shape, img_space, proj_shape, channel_space,
                                img_offset=(0, 0), channel_offset=0, dso=1000, dsd=1500, fov=-1):
    """Fan BP over an explicit angle list, unscaled (the reference's numpy
    FanFBP2DAngle path, numpy_ext/np_ctrecon.py:66-99)."""
    op = FanBackprojection2DAngleOp(angles, int(proj_shape[1]), float(channel_space),
                                    float(channel_offset), int(img_shape[1]), int(img_shape[0]),
                                    float(img_space[1]), float(img_space[0]),
                                    float(img_offset[1]), float(img_offset[0]), float(dso),
                                    float(dsd), float(fov))
    return apply(op, proj)


# ---- the reference's PyTorch extension functions (pytorch/bp_par_2d_ops.cc) ----

_BPPAR2D_METHOD_ERROR = "Unrecognised backprojection method. Only pixdriven is available now."


def bppar2d_prep_forward(method, ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy,
                         offset_x, offset_y, fov, device=None):
    """ParallelBackprojection2DPixDrivenPrep as the reference's PyTorch
    extension exposes it (pytorch/bp_par_2d_ops.cc:17-48): returns [buffer1,
    buffer2, buffer3] = [x cos(t) double [nx][na], y sin(t) double [ny][na],
    the prep's unused int buffer (one int)].  Same arguments and the same error
    for any method other than "pixdriven".  The buffers are built on the CUDA
    device (`device`, default the current one): this library has no CPU
    implementation, where the reference extension ran the prep on the CPU."""
    if method != "pixdriven":
        raise RuntimeError(_BPPAR2D_METHOD_ERROR)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    p = ParParam(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x, offset_y, fov)
    buf1 = torch.empty((nx, na), dtype=torch.float64, device=dev)
    buf2 = torch.empty((ny, na), dtype=torch.float64, device=dev)
    buf3 = torch.zeros((1,), dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        call("ctr_bp_par_2d_prep", ctypes.byref(p), _ptr(buf1), _ptr(buf2), _ptr(buf3), _stream())
    return [buf1, buf2, buf3]


def bppar2d_forward(input, buffer1, buffer2, buffer3, method, ns, na, ds, orbit, offset_s,
                    orbit_start, nx, ny, dx, dy, offset_x, offset_y, fov):
    """ParallelBackprojection2DPixDriven through the reference's PyTorch
    extension signature (pytorch/bp_par_2d_ops.cc:50-73): `input` is a
    sinogram [na][ns] or a batch [B][na][ns] (float32 or float64, CUDA), the
    buffers are bppar2d_prep_forward's; returns the image [ny][nx] (or
    [B][ny][nx]).  Raises RuntimeError for a method other than "pixdriven"."""
    if method != "pixdriven":
        raise RuntimeError(_BPPAR2D_METHOD_ERROR)
    p = ParParam(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x, offset_y, fov)
    xb, restore = _as_batch(input, na, ns, "bppar2d_forward")
    for b, shape in ((buffer1, (nx, na)), (buffer2, (ny, na))):
        if (b.dtype != torch.float64 or tuple(b.shape) != shape or b.device != xb.device
                or not b.is_contiguous()):
            raise ValueError(f"bppar2d_forward: buffer of shape {tuple(b.shape)} {b.dtype} on "
                             f"{b.device}; expected a contiguous {shape} float64 on {xb.device}")
    img = torch.empty((xb.shape[0], ny, nx), dtype=xb.dtype, device=xb.device)
    call(f"ctr_bp_par_2d_{_sfx(xb)}", ctypes.byref(p), _ptr(xb), _ptr(img), _ptr(buffer1),
         _ptr(buffer2), _ptr(buffer3), xb.shape[0], _stream())
    return restore(img)
