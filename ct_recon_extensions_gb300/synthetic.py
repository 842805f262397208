"""Seeded synthetic CT inputs: random-ellipse phantoms and their analytic
line integrals, in the geometry conventions of the reference operators.

Conventions (reference src/bp_fan_2d.cc:22-42, src/bp_par_2d.cc:70):

* image ``[ny][nx]``, pixel centre ``x = (ix - centx)*dx``,
  ``y = (centy - iy)*dy`` with ``centx = (nx-1)/2 + offset_x`` (row 0 on top);
* parallel view ``theta = orbit_start + ia*orbit``, channel coordinate
  ``s = x*cos(theta) + y*sin(theta)`` at ``s = (is - cents)*ds``;
* equiangular fan view ``beta``: source at ``(-dso*sin(beta), dso*cos(beta))``,
  channel fan angle ``gamma = (is - cents)*ds/dsd`` (``ds`` is the arc pitch
  at the detector in mm).  A fan ray is the parallel ray
  ``theta = beta + gamma``, ``s = dso*sin(gamma)``.

The ellipse parameters follow the benchmark description: centres uniform in a
disk of radius 100 mm, semi-axes U[5, 80] mm, orientation U[0, pi),
attenuation U[0.01, 0.03] /mm.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Ellipses:
    cx: np.ndarray
    cy: np.ndarray
    a: np.ndarray
    b: np.ndarray
    phi: np.ndarray
    mu: np.ndarray


def random_ellipses(seed: int, n: int = 10, radius: float = 100.0,
                    axes=(5.0, 80.0), mu=(0.01, 0.03)) -> Ellipses:
    rng = np.random.default_rng(seed)
    r = radius * np.sqrt(rng.uniform(0.0, 1.0, n))
    t = rng.uniform(0.0, 2 * math.pi, n)
    return Ellipses(cx=r * np.cos(t), cy=r * np.sin(t),
                    a=rng.uniform(*axes, n), b=rng.uniform(*axes, n),
                    phi=rng.uniform(0.0, math.pi, n), mu=rng.uniform(*mu, n))


def scaled(e: Ellipses, f: float) -> Ellipses:
    """The same phantom magnified by f (for small test geometries)."""
    return Ellipses(e.cx * f, e.cy * f, e.a * f, e.b * f, e.phi, e.mu / f)


def rasterize(e: Ellipses, nx: int, ny: int, dx: float, dy: float,
              offset_x: float = 0.0, offset_y: float = 0.0, dtype=np.float32) -> np.ndarray:
    """Pixel-centre sampling of the phantom on the reference image grid."""
    centx = (nx - 1) / 2 + offset_x
    centy = (ny - 1) / 2 + offset_y
    x = (np.arange(nx) - centx) * dx
    y = (centy - np.arange(ny)) * dy
    X, Y = np.meshgrid(x, y)
    img = np.zeros((ny, nx), dtype=np.float64)
    for i in range(len(e.mu)):
        c, s = math.cos(e.phi[i]), math.sin(e.phi[i])
        u = (X - e.cx[i]) * c + (Y - e.cy[i]) * s
        v = -(X - e.cx[i]) * s + (Y - e.cy[i]) * c
        img += e.mu[i] * ((u / e.a[i]) ** 2 + (v / e.b[i]) ** 2 <= 1.0)
    return img.astype(dtype)


def _line_integrals(e: Ellipses, theta: np.ndarray, s: np.ndarray) -> np.ndarray:
    """Line integrals along {p : p . (cos theta, sin theta) = s} (broadcast)."""
    out = np.zeros(np.broadcast(theta, s).shape, dtype=np.float64)
    ct, st = np.cos(theta), np.sin(theta)
    for i in range(len(e.mu)):
        al = theta - e.phi[i]
        r2 = (e.a[i] * np.cos(al)) ** 2 + (e.b[i] * np.sin(al)) ** 2
        sp = s - (e.cx[i] * ct + e.cy[i] * st)
        arg = r2 - sp * sp
        val = 2.0 * e.mu[i] * e.a[i] * e.b[i] * np.sqrt(np.maximum(arg, 0.0)) / r2
        out += np.where(arg > 0, val, 0.0)
    return out


def parallel_sinogram(e: Ellipses, na: int, ns: int, ds: float, orbit: float,
                      orbit_start: float = 0.0, offset_s: float = 0.0,
                      dtype=np.float32) -> np.ndarray:
    cents = (ns - 1) / 2 + offset_s
    theta = orbit_start + np.arange(na)[:, None] * orbit
    s = (np.arange(ns)[None, :] - cents) * ds
    return _line_integrals(e, theta, s).astype(dtype)


def fan_sinogram(e: Ellipses, na: int, ns: int, ds: float, orbit: float, dso: float,
                 dsd: float, orbit_start: float = 0.0, offset_s: float = 0.0,
                 angles=None, dtype=np.float32) -> np.ndarray:
    cents = (ns - 1) / 2 + offset_s
    beta = (orbit_start + np.arange(na) * orbit) if angles is None else np.asarray(angles)
    gamma = (np.arange(ns) - cents) * ds / dsd
    theta = beta[:, None] + gamma[None, :]
    s = dso * np.sin(gamma)[None, :]
    return _line_integrals(e, theta, s).astype(dtype)


# ---------------------------------------------------------------------------
# The benchmark workloads (sizes of the reference's headline configurations)
# ---------------------------------------------------------------------------

FAN_DSO = 595.0
FAN_DSD = 1085.6


def fan_config_1():
    """Plain fan FBP: 720 views over 2pi, 736 channels at 1.2858 mm arc pitch,
    512x512 image at 0.5 mm."""
    return dict(ns=736, na=720, ds=1.2858, orbit=2 * math.pi / 720, offset_s=0.0,
                orbit_start=0.0, nx=512, ny=512, dx=0.5, dy=0.5, offset_x=0.0, offset_y=0.0,
                dso=FAN_DSO, dsd=FAN_DSD, fov=-1.0)


def parallel_config_2():
    """Parallel drop-in: 512x512 image at 0.5 mm, 720 views over pi, 729 bins
    at 0.5 mm."""
    return dict(ns=729, na=720, ds=0.5, orbit=math.pi / 720, offset_s=0.0, orbit_start=0.0,
                nx=512, ny=512, dx=0.5, dy=0.5, offset_x=0.0, offset_y=0.0, fov=-1.0)


def batched_config_3(n_items: int = 64, seed_base: int = 3000):
    """Uneven fan batch: per item image n in [256, 1024] with dx = 256/n mm
    (constant FOV), views in [360, 2304] over 2pi, channels in [512, 1024]
    with ds = 1.2858*736/ns (constant fan angle).  Item i draws its sizes and
    phantom from seed seed_base + i."""
    items = []
    for i in range(n_items):
        rng = np.random.default_rng(seed_base + i)
        n = int(rng.integers(256, 1025))
        na = int(rng.integers(360, 2305))
        ns = int(rng.integers(512, 1025))
        items.append(dict(ns=ns, na=na, ds=1.2858 * 736 / ns, orbit=2 * math.pi / na,
                          offset_s=0.0, orbit_start=0.0, nx=n, ny=n, dx=256.0 / n,
                          dy=256.0 / n, offset_x=0.0, offset_y=0.0, dso=FAN_DSO,
                          dsd=FAN_DSD, fov=-1.0, seed=seed_base + i))
    return items


def large_config_5():
    """Reduced-precision large slice: 2048x2048 at 0.25 mm, 2304 views over
    2pi, 1472 channels at 0.6429 mm arc pitch."""
    return dict(ns=1472, na=2304, ds=0.6429, orbit=2 * math.pi / 2304, offset_s=0.0,
                orbit_start=0.0, nx=2048, ny=2048, dx=0.25, dy=0.25, offset_x=0.0,
                offset_y=0.0, dso=FAN_DSO, dsd=FAN_DSD, fov=-1.0)


def fan_sinogram_torch(e: Ellipses, na: int, ns: int, ds: float, orbit: float, dso: float,
                       dsd: float, device, orbit_start: float = 0.0, offset_s: float = 0.0):
    """fan_sinogram computed with torch on `device` (FP32), for large batches."""
    import torch
    f32 = dict(dtype=torch.float32, device=device)
    cents = (ns - 1) / 2 + offset_s
    beta = orbit_start + torch.arange(na, **f32) * orbit
    gamma = (torch.arange(ns, **f32) - cents) * (ds / dsd)
    theta = beta[:, None] + gamma[None, :]
    s = dso * torch.sin(gamma)[None, :]
    ct, st = torch.cos(theta), torch.sin(theta)
    out = torch.zeros((na, ns), **f32)
    for i in range(len(e.mu)):
        al = theta - float(e.phi[i])
        r2 = (float(e.a[i]) * torch.cos(al)) ** 2 + (float(e.b[i]) * torch.sin(al)) ** 2
        sp = s - (float(e.cx[i]) * ct + float(e.cy[i]) * st)
        arg = r2 - sp * sp
        out += torch.where(arg > 0, 2.0 * float(e.mu[i] * e.a[i] * e.b[i]) *
                           torch.sqrt(torch.clamp(arg, min=0.0)) / r2, torch.zeros_like(arg))
    return out
