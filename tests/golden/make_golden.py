"""Generate the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs the reference's own CPU operators (its src/ sources compiled unmodified
by ``make -C oracle ref`` into oracle/_ref/libctr_ref.so) on small seeded
inputs and stores inputs, geometry and outputs for T=float and T=double.  The
fixtures pin the oracle port (tests/test_oracle_golden.py) and the CUDA path
(tests/test_parity_gpu.py).  Needs the reference checkout, so it runs only
where that exists:

    python tests/golden/make_golden.py [case ...]

Operators whose reference code is not well defined (the parallel-BP grad and
the fan-angle grad) have no reference fixture; their oracle is pinned by the
adjoint dot test against the pinned forward operator instead.
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ct_recon_extensions_gb300 import synthetic as syn  # noqa: E402
from oracle import Geom, Oracle, build  # noqa: E402

GEOM_KEYS = [f for f, _ in Geom._fields_]

# Small geometries.  Phantoms are the benchmark's 100 mm ellipses scaled to
# each field of view; several cases carry offsets, reversed orbits, partial
# scans, non-square images and positions that land exactly on channels.  The
# forward-projection cases use detectors that cover the image diagonal plus a
# channel: the reference grad reads channels without a bounds check
# (src/fp_par_2d.cc:375), so outside that domain its output is undefined.
CASES = {
    "fan_full": dict(kind="fan", g=dict(ns=80, na=72, ds=1.2858 * 736 / 80, orbit=2 * math.pi / 72,
                                        nx=48, ny=40, dx=256 / 48, dy=256 / 48, offset_s=0.3,
                                        offset_x=0.2, offset_y=-0.4, dso=595.0, dsd=1085.6)),
    "fan_short_cw": dict(kind="fan", g=dict(ns=64, na=50, ds=1.6, orbit=-math.pi / 50,
                                            orbit_start=0.7, nx=32, ny=32, dx=6.0, dy=6.0,
                                            dso=595.0, dsd=1085.6)),
    "fan_angle": dict(kind="fan_angle", g=dict(ns=70, na=60, ds=1.2858 * 736 / 70,
                                               orbit=2 * math.pi / 60, nx=40, ny=40,
                                               dx=6.4, dy=6.4, offset_s=-0.2, dso=595.0,
                                               dsd=1085.6)),
    "par": dict(kind="par", g=dict(ns=91, na=60, ds=4.0, orbit=math.pi / 60, nx=64, ny=64,
                                   dx=4.0, dy=4.0, offset_s=0.25)),
    "par_rect_cw": dict(kind="par", g=dict(ns=75, na=45, ds=3.0, orbit=-math.pi / 45,
                                           orbit_start=0.4, nx=40, ny=56, dx=4.0, dy=3.5,
                                           offset_x=0.5, offset_y=-0.25)),
    "par_exact": dict(kind="par", g=dict(ns=16, na=4, ds=1.0, orbit=math.pi / 2, nx=16, ny=16,
                                         dx=1.0, dy=1.0)),
    "sv": dict(kind="sv", g=dict(ns=45, na=24, ds=8.0, orbit=math.pi / 24, nx=24, ny=20,
                                 dx=10.0, dy=10.0, offset_s=-0.5)),
    "fp_half": dict(kind="fp", g=dict(ns=91, na=60, ds=4.5, orbit=math.pi / 60, nx=64, ny=64,
                                      dx=4.0, dy=4.0, offset_s=0.25)),
    "fp_full_wrap": dict(kind="fp", g=dict(ns=67, na=72, ds=7.0, orbit=2 * math.pi / 72,
                                           orbit_start=-0.2, nx=48, ny=48, dx=6.0, dy=6.0,
                                           offset_x=0.3, offset_y=0.1)),
    # distance driven (src/fp_par_2d.cc:396-653); detectors cover the image
    # diagonal plus a channel, like the ray-driven cases (unchecked channels)
    "dd_half": dict(kind="dd", g=dict(ns=91, na=60, ds=4.5, orbit=math.pi / 60, nx=64, ny=64,
                                      dx=4.0, dy=4.0, offset_s=0.25)),
    "dd_full_wrap": dict(kind="dd", g=dict(ns=67, na=72, ds=7.0, orbit=2 * math.pi / 72,
                                           orbit_start=-0.2, nx=48, ny=48, dx=6.0, dy=6.0,
                                           offset_x=0.3, offset_y=0.1)),
    # ray casting (src/fp_par_2d.cc:18-145): the FoV radius bounds the rays
    "cast_half": dict(kind="cast", step=0.125,
                      g=dict(ns=91, na=60, ds=4.5, orbit=math.pi / 60, nx=64, ny=64, dx=4.0,
                             dy=4.0, offset_s=0.25, fov=120.0)),
    "cast_full_rect": dict(kind="cast", step=0.25,
                           g=dict(ns=67, na=72, ds=7.0, orbit=-2 * math.pi / 72, orbit_start=0.3,
                                  nx=48, ny=40, dx=6.0, dy=6.0, offset_x=0.3, offset_y=-0.2,
                                  fov=150.0)),
}

# Helical rebinning (src/helical_interpolation.cc:80-370).  Rows map to z as
# z * dsd / dso (the reference's implied 1 mm rows), so a pitch-p scan moves
# p * nt * dso / dsd per rotation.  Slices keep every needed view >= 1 (the
# 180LI complementary rays of a slice whose first view is 0 make the reference
# read before its input).  "expect" is the reference's status: 1, or the
# oracle codes of its two runtime_errors.
_P1 = 8 * 500.0 / 1000.0 / 60  # pitch 1: couch step per view for nt=8, dso/dsd=0.5, 60 views/rotation
HELI_CASES = {
    "heli_p1": dict(h=dict(ns=48, nt=8, na=170, ds=1.0, dt=1.0, view_per_rot=60, couch_mov=_P1,
                           nz=6, dz=0.3, z0=5.2, thickness=1.0, dso=500.0, dsd=1000.0,
                           offset_s=0.25, offset_t=-0.3), expect=1),
    # clockwise rotation, couch moving towards -z, pitch 1.2, thick slices
    "heli_cw_back": dict(h=dict(ns=40, nt=12, na=180, ds=1.3, dt=1.0, view_per_rot=50,
                                couch_mov=-12 * 600.0 / 1100.0 * 1.2 / 50, couch_begin=40.0,
                                orbit=-2 * math.pi / 50, nz=7, dz=0.35,
                                z0=40.0 - 12 * 600.0 / 1100.0 * 1.2 / 50 * 120, thickness=1.5,
                                dso=600.0, dsd=1100.0, offset_s=-0.35, offset_t=0.4), expect=1),
    # pitch 2.6: samples where both rays miss the detector rows
    "heli_norows": dict(h=dict(ns=32, nt=6, na=120, ds=1.0, dt=1.0, view_per_rot=40,
                               couch_mov=6 * 0.5 * 2.6 / 40, nz=3, dz=0.5, z0=7.8 * 2.0,
                               thickness=0.5, dso=500.0, dsd=1000.0), expect=-2),
    # the first slice needs views before view 0
    "heli_views": dict(h=dict(ns=32, nt=6, na=120, ds=1.0, dt=1.0, view_per_rot=40,
                              couch_mov=6 * 0.5 / 40, nz=3, dz=0.5, z0=1.0, thickness=0.5,
                              dso=500.0, dsd=1000.0), expect=-1),
}


def heli(d):
    from oracle import Heli
    return Heli.make(**d)


def make_heli_case(name, spec, ref: Oracle):
    from oracle import HelicalError
    h = heli(spec["h"])
    rng = np.random.default_rng(9000 + sum(map(ord, name)))
    v, t, s = np.meshgrid(np.arange(h.na), np.arange(h.nt), np.arange(h.ns), indexing="ij")
    x = (1.5 + np.sin(0.07 * v + 0.5 * t) * np.cos(0.13 * s) + 0.2 * np.cos(0.011 * v * t)
         + 0.05 * rng.standard_normal(v.shape))
    x = np.round(x * 4096) / 4096  # 12 fractional bits: compresses, and exact in float32
    out = dict(params=json.dumps(dict(kind="heli", heli={f: getattr(h, f) for f, _ in h._fields_},
                                      expect=spec["expect"])))
    out["in_f64"] = x  # the float input is its exact cast, x.astype(float32)
    for sfx, dt in (("f32", np.float32), ("f64", np.float64)):
        for m in ("360", "180"):
            try:
                res, _ = ref.helical(x.astype(dt), h, m)
                st = 1
            except HelicalError as e:
                res, st = np.zeros((h.nz, h.view_per_rot, h.ns), dt), e.code
            assert st == spec["expect"], (name, m, st)
            out[f"out{m}_{sfx}"] = res
            out[f"status{m}"] = np.int32(st)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def geom(d):
    full = dict(offset_s=0.0, orbit_start=0.0, offset_x=0.0, offset_y=0.0, dso=-1.0, dsd=-1.0,
                fov=-1.0)
    full.update(d)
    return Geom.make(**full)


def gdict(g):
    return {k: getattr(g, k) for k in GEOM_KEYS}


def make_case(name, spec, ref: Oracle):
    g = geom(spec["g"])
    kind = spec["kind"]
    seed = 7000 + sum(map(ord, name))
    rng = np.random.default_rng(seed)
    fov = min(g.nx * g.dx, g.ny * g.dy) / 2
    ph = syn.scaled(syn.random_ellipses(seed), 0.8 * fov / 180.0)
    out = dict(params=json.dumps(dict(kind=kind, geom=gdict(g))))
    if kind in ("fan", "fan_angle"):
        angles = None
        if kind == "fan_angle":
            angles = np.sort(rng.uniform(0.0, 2 * math.pi, g.na))
            out["angles"] = angles
        sino = syn.fan_sinogram(ph, g.na, g.ns, g.ds, g.orbit, g.dso, g.dsd, g.orbit_start,
                                g.offset_s, angles=angles, dtype=np.float64)
        sino += 0.01 * rng.standard_normal(sino.shape) * sino.max()
        img_in = rng.standard_normal((g.ny, g.nx))
        out["taps_fan"] = ref.ramp_taps(g.ns, g.ds, g.dsd, 1)
        out["taps_flat"] = ref.ramp_taps(g.ns, g.ds, g.dsd, 2)
        for sfx, dt in (("f32", np.float32), ("f64", np.float64)):
            p = sino.astype(dt)
            out[f"sino_{sfx}"] = p
            for wt in (1, 2):
                w = ref.fan_weighting(p, g.ds, g.offset_s, g.dso, g.dsd, wt)
                out[f"weighted{wt}_{sfx}"] = w
                out[f"weighted{wt}_grad_{sfx}"] = ref.fan_weighting(p, g.ds, g.offset_s, g.dso,
                                                                    g.dsd, wt, grad=True)
            filt = ref.ramp_filter(out[f"weighted1_{sfx}"], g.ds, g.dsd, 1)
            out[f"filtered_{sfx}"] = filt
            out[f"filtered_grad_{sfx}"] = ref.ramp_filter(p, g.ds, g.dsd, 1, grad=True)
            out[f"filtered_flat_{sfx}"] = ref.ramp_filter(out[f"weighted2_{sfx}"], g.ds, g.dsd, 2)
            if kind == "fan":
                out[f"bp_{sfx}"] = ref.bp_fan_2d(filt, g)
                out[f"bp_grad_{sfx}"] = ref.bp_fan_2d_grad(img_in.astype(dt), g)
                out[f"img_in_{sfx}"] = img_in.astype(dt)
            else:
                out[f"bp_{sfx}"] = ref.bp_fan_2d_angle(filt, g, angles)
    elif kind in ("par", "sv"):
        sino = syn.parallel_sinogram(ph, g.na, g.ns, g.ds, g.orbit, g.orbit_start, g.offset_s,
                                     dtype=np.float64)
        sino += 0.01 * rng.standard_normal(sino.shape) * sino.max()
        out["taps_par"] = ref.ramp_taps(g.ns, g.ds, -1.0, 0)
        for sfx, dt in (("f32", np.float32), ("f64", np.float64)):
            p = sino.astype(dt)
            out[f"sino_{sfx}"] = p
            filt = ref.ramp_filter(p, g.ds, -1.0, 0)
            out[f"filtered_{sfx}"] = filt
            if kind == "par":
                out[f"bp_{sfx}"] = ref.bp_par_2d(filt, g)
            else:
                out[f"sv_{sfx}"] = ref.bp_par_2d_sv(p, g)
    elif kind == "fp":
        img = syn.rasterize(ph, g.nx, g.ny, g.dx, g.dy, g.offset_x, g.offset_y, dtype=np.float64)
        img += 0.001 * rng.standard_normal(img.shape)
        proj_in = rng.standard_normal((g.na, g.ns))
        for sfx, dt in (("f32", np.float32), ("f64", np.float64)):
            out[f"img_{sfx}"] = img.astype(dt)
            out[f"fp_{sfx}"] = ref.fp_par_2d(img.astype(dt), g)
            out[f"proj_in_{sfx}"] = proj_in.astype(dt)
            out[f"fp_grad_{sfx}"] = ref.fp_par_2d_grad(proj_in.astype(dt), g)
    elif kind == "dd":
        img = syn.rasterize(ph, g.nx, g.ny, g.dx, g.dy, g.offset_x, g.offset_y, dtype=np.float64)
        img += 0.001 * rng.standard_normal(img.shape)
        proj_in = rng.standard_normal((g.na, g.ns))
        for sfx, dt in (("f32", np.float32), ("f64", np.float64)):
            out[f"img_{sfx}"] = img.astype(dt)
            out[f"dd_{sfx}"] = ref.fp_par_2d_dd(img.astype(dt), g)
            out[f"proj_in_{sfx}"] = proj_in.astype(dt)
            out[f"dd_grad_{sfx}"] = ref.fp_par_2d_dd_grad(proj_in.astype(dt), g)
    elif kind == "cast":
        img = syn.rasterize(ph, g.nx, g.ny, g.dx, g.dy, g.offset_x, g.offset_y, dtype=np.float64)
        img += 0.001 * rng.standard_normal(img.shape)
        out["step"] = np.float64(spec["step"])
        for sfx, dt in (("f32", np.float32), ("f64", np.float64)):
            out[f"img_{sfx}"] = img.astype(dt)
            out[f"cast_{sfx}"] = ref.fp_par_2d_cast(img.astype(dt), g, spec["step"])
    else:
        raise ValueError(kind)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def main(names=None):
    build(ref=True)
    ref = Oracle("reference")
    for name, spec in CASES.items():
        if names and name not in names:
            continue
        make_case(name, spec, ref)
        print("wrote", name)
    for name, spec in HELI_CASES.items():
        if names and name not in names:
            continue
        make_heli_case(name, spec, ref)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1:])
