"""CPU oracle for the CT reconstruction hot path -- TEST INFRASTRUCTURE ONLY.

Two interchangeable back ends with one numpy API:

* ``Oracle("port")`` loads ``oracle/libctr_oracle.so``, the plain-C
  restatement of the reference's CPU code (``ctr_oracle.c``).  It builds on any
  host and is what the GPU-side tests and the CPU baseline use.
* ``Oracle("reference")`` loads ``oracle/_ref/libctr_ref.so``, the reference's
  own ``src`` sources compiled unmodified with ``ref_shim.cc``.  It exists only
  where the reference checkout was available at build time and is used to pin
  the port (tests/golden/make_golden.py, tests/test_oracle_golden.py).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm may import this package, and only as the checker.

Array conventions follow the reference: sinograms ``[na][ns]`` (view-major),
images ``[ny][nx]`` with row 0 at the top (y = +centy*dy), single-view stacks
``[ny][nx][na]``.  float32 inputs run the reference's ``T=float`` code,
float64 inputs ``T=double``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(_HERE, "libctr_oracle.so")
REF_LIB = os.path.join(_HERE, "_ref", "libctr_ref.so")

_c_uint = ctypes.c_uint
_c_double = ctypes.c_double
_c_int = ctypes.c_int
_ptr = ctypes.c_void_p


class Geom(ctypes.Structure):
    """Mirror of ``orc_geom`` (ctr_oracle.h)."""

    _fields_ = [
        ("ns", _c_uint), ("na", _c_uint),
        ("ds", _c_double), ("orbit", _c_double), ("offset_s", _c_double),
        ("orbit_start", _c_double),
        ("nx", _c_uint), ("ny", _c_uint),
        ("dx", _c_double), ("dy", _c_double), ("offset_x", _c_double),
        ("offset_y", _c_double),
        ("dso", _c_double), ("dsd", _c_double), ("fov", _c_double),
    ]

    @classmethod
    def make(cls, ns, na, ds, orbit, nx, ny, dx, dy, offset_s=0.0, orbit_start=0.0,
             offset_x=0.0, offset_y=0.0, dso=-1.0, dsd=-1.0, fov=-1.0):
        return cls(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x,
                   offset_y, dso, dsd, fov)


class Heli(ctypes.Structure):
    """Mirror of ``orc_heli`` (ctr_oracle.h): HelicalInterpolationParam's fields
    in its order (reference include/helical_interpolation.h:17-64)."""

    _fields_ = [
        ("ns", _c_uint), ("nt", _c_uint), ("na", _c_uint),
        ("ds", _c_double), ("dt", _c_double), ("offset_s", _c_double), ("offset_t", _c_double),
        ("orbit_start", _c_double), ("orbit", _c_double), ("couch_begin", _c_double),
        ("couch_mov", _c_double),
        ("view_per_rot", _c_uint), ("nz", _c_uint),
        ("dz", _c_double), ("z0", _c_double), ("thickness", _c_double), ("dso", _c_double),
        ("dsd", _c_double),
    ]

    @classmethod
    def make(cls, ns, nt, na, ds, dt, view_per_rot, couch_mov, nz, dz, z0, thickness, dso, dsd,
             offset_s=0.0, offset_t=0.0, orbit_start=0.0, orbit=None, couch_begin=0.0):
        if orbit is None:
            orbit = 2 * math.pi / view_per_rot
        return cls(ns, nt, na, ds, dt, offset_s, offset_t, orbit_start, orbit, couch_begin,
                   couch_mov, view_per_rot, nz, dz, z0, thickness, dso, dsd)


# the reference's std::runtime_error messages (src/helical_interpolation.cc:87-148)
HELI_ERRORS = {-1: "View not enough for this slice!", -2: "No row data available!"}


class HelicalError(RuntimeError):
    def __init__(self, code: int):
        super().__init__(HELI_ERRORS.get(code, f"helical status {code}"))
        self.code = code


def build(ref_src: str | None = None, quiet: bool = True) -> None:
    """Compile the port (always) and, when ``ref_src`` (default: the
    environment variable CTR_REFERENCE_SRC) names a reference checkout with its
    ``src/`` directory, the reference build from that checkout."""
    if ref_src is None:
        ref_src = os.environ.get("CTR_REFERENCE_SRC")
    targets = ["all"]
    if ref_src and os.path.isdir(os.path.join(ref_src, "src")):
        targets += ["ref", f"REF={ref_src}"]
    out = subprocess.run(["make", "-C", _HERE, *targets], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_ptr)


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f32"
    if dt == np.float64:
        return "f64"
    raise TypeError(f"oracle supports float32/float64, got {dt}")


def _chunks(n: int, parts: int):
    parts = max(1, min(parts, n))
    step = (n + parts - 1) // parts
    return [(i, min(n, i + step)) for i in range(0, n, step)]


class Oracle:
    """numpy front end over the port or the reference build."""

    def __init__(self, kind: str = "port", threads: int = 1):
        if kind not in ("port", "reference"):
            raise ValueError(kind)
        path = PORT_LIB if kind == "port" else REF_LIB
        if not os.path.exists(path):
            if kind == "port":
                build(ref=False)
            else:
                raise FileNotFoundError(
                    f"{path} missing: the reference build needs the reference checkout")
        self.kind = kind
        self.lib = ctypes.CDLL(path)
        self.threads = max(1, int(threads))
        self._pfx = "orc_" if kind == "port" else "ref_"

    # -- plumbing ----------------------------------------------------------
    def _fn(self, name):
        f = getattr(self.lib, self._pfx + name)
        f.restype = _c_int
        return f

    def _run_ranges(self, n, call):
        """Run call(lo, hi) over [0, n) split across the worker threads (port
        only; the reference functions take whole arrays)."""
        ranges = _chunks(n, self.threads)
        if len(ranges) == 1:
            ok = call(*ranges[0])
            if not ok:
                raise RuntimeError("oracle call failed")
            return
        with ThreadPoolExecutor(len(ranges)) as ex:
            res = list(ex.map(lambda r: call(*r), ranges))
        if not all(res):
            raise RuntimeError("oracle call failed")

    @staticmethod
    def _c(a, dtype=None):
        return np.ascontiguousarray(a, dtype=dtype)

    # -- fan weighting (src/fan_weighting.cc:19-59) -------------------------
    def fan_weighting(self, proj, ds, offset=0.0, dso=-1.0, dsd=-1.0, type=1, grad=False):
        proj = self._c(proj)
        nrow, ns = proj.shape
        out = np.empty_like(proj)
        f = self._fn(("fan_weighting_grad_" if grad else "fan_weighting_") + _sfx(proj.dtype))
        ok = f(_c_uint(ns), _c_uint(nrow), _c_double(ds), _c_double(offset), _c_double(dso),
               _c_double(dsd), _c_int(type), _p(proj), _p(out))
        if not ok:
            raise ValueError("fan weighting rejected the parameters (type must be 1 or 2)")
        return out

    # -- ramp filter (src/filter.cc:18-124) --------------------------------
    def ramp_taps(self, ns, ds, dsd=-1.0, type=0):
        taps = np.empty(2 * ns + 1, dtype=np.float64)
        ok = self._fn("ramp_filter_prep")(_c_uint(ns), _c_double(ds), _c_double(dsd),
                                          _c_int(type), _p(taps))
        if not ok:
            raise ValueError("ramp filter rejected the type (must be 0, 1 or 2)")
        return taps

    def ramp_filter(self, proj, ds, dsd=-1.0, type=0, grad=False, taps=None):
        proj = self._c(proj)
        nrow, ns = proj.shape
        if taps is None:
            taps = self.ramp_taps(ns, ds, dsd, type)
        out = np.empty_like(proj)
        name = ("ramp_filter_grad_" if grad else "ramp_filter_") + ("" if self.kind == "reference" else "rows_")
        f = self._fn(name + _sfx(proj.dtype))
        if self.kind == "reference":
            if not f(_c_uint(ns), _c_uint(nrow), _c_double(ds), _p(proj), _p(taps), _p(out)):
                raise RuntimeError("reference ramp filter failed")
        else:
            self._run_ranges(nrow, lambda a, b: f(_c_uint(ns), _c_uint(a), _c_uint(b),
                                                  _c_double(ds), _p(proj), _p(taps), _p(out)))
        return out

    # -- fan BP (src/bp_fan_2d.cc) -----------------------------------------
    def bp_fan_2d_tables(self, g: Geom):
        xpos = np.empty(g.nx); ypos = np.empty(g.ny); sc = np.empty(2 * g.na)
        self._fn("bp_fan_2d_prep")(ctypes.byref(g), _p(xpos), _p(ypos), _p(sc))
        return xpos, ypos, sc

    def bp_fan_2d_angle_tables(self, g: Geom, angles):
        angles = self._c(angles, np.float64)
        xpos = np.empty(g.nx); ypos = np.empty(g.ny); sc = np.empty(2 * g.na)
        self._fn("bp_fan_2d_angle_prep")(ctypes.byref(g), _p(angles), _p(xpos), _p(ypos), _p(sc))
        return xpos, ypos, sc

    def _fan_bp(self, kind, proj, g, tables):
        proj = self._c(proj)
        assert proj.shape == (g.na, g.ns), (proj.shape, g.na, g.ns)
        xpos, ypos, sc = tables
        img = np.empty((g.ny, g.nx), dtype=proj.dtype)
        if self.kind == "reference":
            f = self._fn(f"{kind}_{_sfx(proj.dtype)}")
            f(ctypes.byref(g), _p(proj), _p(img), _p(xpos), _p(ypos), _p(sc))
        else:
            f = self._fn(f"{kind}_rows_{_sfx(proj.dtype)}")
            self._run_ranges(g.ny, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b),
                                                  _p(proj), _p(img), _p(xpos), _p(ypos), _p(sc)))
        return img

    def bp_fan_2d(self, proj, g: Geom):
        return self._fan_bp("bp_fan_2d", proj, g, self.bp_fan_2d_tables(g))

    def bp_fan_2d_angle(self, proj, g: Geom, angles):
        return self._fan_bp("bp_fan_2d_angle", proj, g, self.bp_fan_2d_angle_tables(g, angles))

    def bp_fan_2d_grad(self, img, g: Geom):
        img = self._c(img)
        xpos, ypos, sc = self.bp_fan_2d_tables(g)
        grad = np.empty((g.na, g.ns), dtype=img.dtype)
        self._fn(f"bp_fan_2d_grad_{_sfx(img.dtype)}")(ctypes.byref(g), _p(img), _p(grad),
                                                      _p(xpos), _p(ypos), _p(sc))
        return grad

    def bp_fan_2d_angle_grad(self, img, g: Geom, angles):
        if self.kind == "reference":
            raise NotImplementedError("the reference fan-angle grad is not well defined")
        img = self._c(img)
        xpos, ypos, sc = self.bp_fan_2d_angle_tables(g, angles)
        grad = np.empty((g.na, g.ns), dtype=img.dtype)
        self._fn(f"bp_fan_2d_angle_grad_{_sfx(img.dtype)}")(ctypes.byref(g), _p(img), _p(grad),
                                                            _p(xpos), _p(ypos), _p(sc))
        return grad

    # -- parallel BP (src/bp_par_2d.cc, src/bp_par_2d_sv.cc) ---------------
    def bp_par_2d_tables(self, g: Geom):
        xcos = np.empty((g.nx, g.na)); ysin = np.empty((g.ny, g.na))
        self._fn("bp_par_2d_prep")(ctypes.byref(g), _p(xcos), _p(ysin))
        return xcos, ysin

    def _par_bp(self, kind, proj, g, out_shape):
        proj = self._c(proj)
        assert proj.shape == (g.na, g.ns), (proj.shape, g.na, g.ns)
        xcos, ysin = self.bp_par_2d_tables(g)
        img = np.empty(out_shape, dtype=proj.dtype)
        if self.kind == "reference":
            self._fn(f"{kind}_{_sfx(proj.dtype)}")(ctypes.byref(g), _p(proj), _p(img),
                                                   _p(xcos), _p(ysin))
        else:
            f = self._fn(f"{kind}_rows_{_sfx(proj.dtype)}")
            self._run_ranges(g.ny, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b),
                                                  _p(proj), _p(img), _p(xcos), _p(ysin)))
        return img

    def bp_par_2d(self, proj, g: Geom):
        return self._par_bp("bp_par_2d", proj, g, (g.ny, g.nx))

    def bp_par_2d_sv(self, proj, g: Geom):
        return self._par_bp("bp_par_2d_sv", proj, g, (g.ny, g.nx, g.na))

    def bp_par_2d_grad(self, img, g: Geom):
        if self.kind == "reference":
            raise NotImplementedError("the reference parallel-BP grad is not well defined")
        img = self._c(img)
        xcos, ysin = self.bp_par_2d_tables(g)
        grad = np.empty((g.na, g.ns), dtype=img.dtype)
        self._fn(f"bp_par_2d_grad_{_sfx(img.dtype)}")(ctypes.byref(g), _p(img), _p(grad),
                                                      _p(xcos), _p(ysin))
        return grad

    # -- parallel ray-driven FP (src/fp_par_2d.cc:149-391) ------------------
    def fp_par_2d_tables(self, g: Geom):
        sc = np.empty((g.na, 2)); bo = np.empty((g.na, g.ns, 2)); usex = np.empty(g.na, np.int32)
        self._fn("fp_par_2d_prep")(ctypes.byref(g), _p(sc), _p(bo), _p(usex))
        return sc, bo, usex

    def fp_par_2d_grad_tables(self, g: Geom):
        if g.nx != g.ny:
            raise ValueError("ray-driven projection needs nx == ny")
        w = np.empty(g.na); pos = np.empty((g.na, g.nx, 2)); usex = np.empty(g.na, np.int32)
        self._fn("fp_par_2d_grad_prep")(ctypes.byref(g), _p(w), _p(pos), _p(usex))
        return w, pos, usex

    def fp_par_2d(self, img, g: Geom, tables=None):
        """Ray-driven projection; `tables` = (sincos, beginoffset, usex) in
        place of the prep's own (a caller's table, as the reference's op takes)."""
        img = self._c(img)
        assert img.shape == (g.ny, g.nx)
        sc, bo, usex = self.fp_par_2d_tables(g) if tables is None else (
            self._c(tables[0], np.float64), self._c(tables[1], np.float64), self._c(tables[2], np.int32))
        proj = np.empty((g.na, g.ns), dtype=img.dtype)
        if self.kind == "reference":
            self._fn(f"fp_par_2d_{_sfx(img.dtype)}")(ctypes.byref(g), _p(img), _p(proj), _p(sc),
                                                     _p(bo), _p(usex))
        else:
            f = self._fn(f"fp_par_2d_views_{_sfx(img.dtype)}")
            self._run_ranges(g.na, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b),
                                                  _p(img), _p(proj), _p(sc), _p(bo), _p(usex)))
        return proj

    def fp_par_2d_grad(self, proj, g: Geom):
        proj = self._c(proj)
        assert proj.shape == (g.na, g.ns)
        w, pos, usex = self.fp_par_2d_grad_tables(g)
        img = np.empty((g.ny, g.nx), dtype=proj.dtype)
        if self.kind == "reference":
            self._fn(f"fp_par_2d_grad_{_sfx(proj.dtype)}")(ctypes.byref(g), _p(proj), _p(img),
                                                           _p(w), _p(pos), _p(usex))
        else:
            f = self._fn(f"fp_par_2d_grad_rows_{_sfx(proj.dtype)}")
            self._run_ranges(g.ny, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b),
                                                  _p(proj), _p(img), _p(w), _p(pos), _p(usex)))
        return img

    # -- parallel ray-casting FP (src/fp_par_2d.cc:18-145) -----------------
    def fp_par_2d_cast_tables(self, g: Geom, step_size: float = 0.125):
        sc = np.empty((g.na, 2)); begins = np.empty((g.na, g.ns, 2))
        nsteps = np.empty((g.na, g.ns), np.int32)
        self._fn("fp_par_2d_cast_prep")(ctypes.byref(g), ctypes.c_double(step_size), _p(sc),
                                        _p(begins), _p(nsteps))
        return sc, begins, nsteps

    def fp_par_2d_cast(self, img, g: Geom, step_size: float = 0.125):
        img = self._c(img)
        assert img.shape == (g.ny, g.nx)
        sc, begins, nsteps = self.fp_par_2d_cast_tables(g, step_size)
        proj = np.empty((g.na, g.ns), dtype=img.dtype)
        st = ctypes.c_double(step_size)
        if self.kind == "reference":
            self._fn(f"fp_par_2d_cast_{_sfx(img.dtype)}")(ctypes.byref(g), st, _p(img), _p(proj),
                                                          _p(sc), _p(begins), _p(nsteps))
        else:
            f = self._fn(f"fp_par_2d_cast_views_{_sfx(img.dtype)}")
            self._run_ranges(g.na, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b), st,
                                                  _p(img), _p(proj), _p(sc), _p(begins),
                                                  _p(nsteps)))
        return proj

    # -- parallel distance-driven FP and its grad (src/fp_par_2d.cc:396-653) ----
    def fp_par_2d_dd_tables(self, g: Geom):
        sc = np.empty((g.na, 2)); bo = np.empty((g.na, g.ns, 3)); usex = np.empty(g.na, np.int32)
        self._fn("fp_par_2d_dd_prep")(ctypes.byref(g), _p(sc), _p(bo), _p(usex))
        return sc, bo, usex

    def fp_par_2d_dd_grad_tables(self, g: Geom):
        if g.nx != g.ny:
            raise ValueError("distance-driven projection needs nx == ny")
        w = np.empty(g.na); pos = np.empty((g.na, g.nx, 2)); usex = np.empty(g.na, np.int32)
        self._fn("fp_par_2d_dd_grad_prep")(ctypes.byref(g), _p(w), _p(pos), _p(usex))
        return w, pos, usex

    def fp_par_2d_dd(self, img, g: Geom):
        img = self._c(img)
        assert img.shape == (g.ny, g.nx)
        sc, bo, usex = self.fp_par_2d_dd_tables(g)
        proj = np.empty((g.na, g.ns), dtype=img.dtype)
        if self.kind == "reference":
            self._fn(f"fp_par_2d_dd_{_sfx(img.dtype)}")(ctypes.byref(g), _p(img), _p(proj), _p(sc),
                                                        _p(bo), _p(usex))
        else:
            f = self._fn(f"fp_par_2d_dd_views_{_sfx(img.dtype)}")
            self._run_ranges(g.na, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b),
                                                  _p(img), _p(proj), _p(sc), _p(bo), _p(usex)))
        return proj

    def fp_par_2d_dd_grad(self, proj, g: Geom):
        proj = self._c(proj)
        assert proj.shape == (g.na, g.ns)
        w, pos, usex = self.fp_par_2d_dd_grad_tables(g)
        img = np.empty((g.ny, g.nx), dtype=proj.dtype)
        if self.kind == "reference":
            self._fn(f"fp_par_2d_dd_grad_{_sfx(proj.dtype)}")(ctypes.byref(g), _p(proj), _p(img),
                                                              _p(w), _p(pos), _p(usex))
        else:
            f = self._fn(f"fp_par_2d_dd_grad_rows_{_sfx(proj.dtype)}")
            self._run_ranges(g.ny, lambda a, b: f(ctypes.byref(g), _c_uint(a), _c_uint(b),
                                                  _p(proj), _p(img), _p(w), _p(pos), _p(usex)))
        return img

    # -- helical rebinning (src/helical_interpolation.cc:80-370) -----------
    def helical(self, proj, h: Heli, method: str = "360"):
        """HelicalInterpolation360 / 180 ``calculate_on_cpu``: [na][nt][ns] ->
        [nz][view_per_rot][ns].  Returns (out, outside): ``outside`` is True when a
        180LI corresponding-view sample fell outside the scan's views (read as 0
        here, an out-of-bounds read in the reference).  Raises HelicalError where
        the reference throws."""
        if method not in ("360", "180"):
            raise ValueError(method)
        proj = self._c(proj)
        assert proj.shape == (h.na, h.nt, h.ns)
        out = np.zeros((h.nz, h.view_per_rot, h.ns), dtype=proj.dtype)
        sfx = _sfx(proj.dtype)
        if self.kind == "reference":
            st = self._fn(f"helical_{method}_{sfx}")(ctypes.byref(h), _p(proj), _p(out))
            if st < 0:
                raise HelicalError(st)
            return out, False
        f = self._fn(f"helical_{method}_slices_{sfx}")
        ranges = _chunks(h.nz, self.threads) if h.nz else []
        call = lambda r: f(ctypes.byref(h), _c_uint(r[0]), _c_uint(r[1]), _p(proj), _p(out))  # noqa: E731
        if len(ranges) > 1:
            with ThreadPoolExecutor(len(ranges)) as ex:
                res = list(ex.map(call, ranges))
        else:
            res = [call(r) for r in ranges]
        for st in res:  # slice order: the first failing slice is the reference's throw
            if st < 0:
                raise HelicalError(st)
        return out, any(st == 3 for st in res)

    # -- composed FBP -------------------------------------------------------
    def fbp_fan(self, proj, g: Geom, weighting_type=1):
        """fan_weighting -> ramp(fan) -> bp_fan_2d, as the reference's CPU
        drivers chain them."""
        w = self.fan_weighting(proj, g.ds, g.offset_s, g.dso, g.dsd, weighting_type)
        f = self.ramp_filter(w, g.ds, g.dsd, 1 if weighting_type == 1 else 2)
        return self.bp_fan_2d(f, g)

    def fbp_par(self, proj, g: Geom):
        return self.bp_par_2d(self.ramp_filter(proj, g.ds, -1.0, 0), g)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))
