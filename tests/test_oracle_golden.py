"""Pin the oracle port (oracle/ctr_oracle.c) to the reference's own outputs.

The fixtures were produced by the reference's src/ code compiled unmodified
(tests/golden/make_golden.py); the port must reproduce them bit for bit.  The
two adjoints without a reference fixture are pinned by the dot test against
their pinned forward operators.
"""
import math

import numpy as np
import pytest

import golden_cases as gc

SFX = [("f32", np.float32), ("f64", np.float64)]


@pytest.mark.parametrize("name", gc.names(("fan", "fan_angle")))
@pytest.mark.parametrize("sfx,dt", SFX)
def test_fan_chain(port, name, sfx, dt):
    c = gc.load(name)
    g = gc.geom(c)
    p = c[f"sino_{sfx}"]
    for wt in (1, 2):
        w = port.fan_weighting(p, g.ds, g.offset_s, g.dso, g.dsd, wt)
        assert np.array_equal(w, c[f"weighted{wt}_{sfx}"])
        wg = port.fan_weighting(p, g.ds, g.offset_s, g.dso, g.dsd, wt, grad=True)
        assert np.array_equal(wg, c[f"weighted{wt}_grad_{sfx}"])
    assert np.array_equal(port.ramp_taps(g.ns, g.ds, g.dsd, 1), c["taps_fan"])
    assert np.array_equal(port.ramp_taps(g.ns, g.ds, g.dsd, 2), c["taps_flat"])
    filt = port.ramp_filter(c[f"weighted1_{sfx}"], g.ds, g.dsd, 1)
    assert np.array_equal(filt, c[f"filtered_{sfx}"])
    assert np.array_equal(port.ramp_filter(p, g.ds, g.dsd, 1, grad=True), c[f"filtered_grad_{sfx}"])
    assert np.array_equal(port.ramp_filter(c[f"weighted2_{sfx}"], g.ds, g.dsd, 2),
                          c[f"filtered_flat_{sfx}"])
    if c["kind"] == "fan":
        assert np.array_equal(port.bp_fan_2d(filt, g), c[f"bp_{sfx}"])
        assert np.array_equal(port.bp_fan_2d_grad(c[f"img_in_{sfx}"], g), c[f"bp_grad_{sfx}"])
    else:
        assert np.array_equal(port.bp_fan_2d_angle(filt, g, c["angles"]), c[f"bp_{sfx}"])


@pytest.mark.parametrize("name", gc.names("par"))
@pytest.mark.parametrize("sfx,dt", SFX)
def test_par_bp(port, name, sfx, dt):
    c = gc.load(name)
    g = gc.geom(c)
    assert np.array_equal(port.ramp_taps(g.ns, g.ds, -1.0, 0), c["taps_par"])
    filt = port.ramp_filter(c[f"sino_{sfx}"], g.ds, -1.0, 0)
    assert np.array_equal(filt, c[f"filtered_{sfx}"])
    assert np.array_equal(port.bp_par_2d(filt, g), c[f"bp_{sfx}"])


@pytest.mark.parametrize("sfx,dt", SFX)
def test_single_view(port, sfx, dt):
    c = gc.load("sv")
    g = gc.geom(c)
    assert np.array_equal(port.bp_par_2d_sv(c[f"sino_{sfx}"], g), c[f"sv_{sfx}"])


@pytest.mark.parametrize("name", gc.names("fp"))
@pytest.mark.parametrize("sfx,dt", SFX)
def test_fp_ray_driven(port, name, sfx, dt):
    c = gc.load(name)
    g = gc.geom(c)
    assert np.array_equal(port.fp_par_2d(c[f"img_{sfx}"], g), c[f"fp_{sfx}"])
    assert np.array_equal(port.fp_par_2d_grad(c[f"proj_in_{sfx}"], g), c[f"fp_grad_{sfx}"])


@pytest.mark.parametrize("name", gc.names("cast"))
@pytest.mark.parametrize("sfx,dt", SFX)
def test_fp_ray_casting(port, name, sfx, dt):
    c = gc.load(name)
    g = gc.geom(c)
    assert np.array_equal(port.fp_par_2d_cast(c[f"img_{sfx}"], g, float(c["step"])), c[f"cast_{sfx}"])


@pytest.mark.parametrize("name", gc.names("dd"))
@pytest.mark.parametrize("sfx,dt", SFX)
def test_fp_distance_driven(port, name, sfx, dt):
    c = gc.load(name)
    g = gc.geom(c)
    assert np.array_equal(port.fp_par_2d_dd(c[f"img_{sfx}"], g), c[f"dd_{sfx}"])
    assert np.array_equal(port.fp_par_2d_dd_grad(c[f"proj_in_{sfx}"], g), c[f"dd_grad_{sfx}"])


@pytest.mark.parametrize("name", gc.names("heli"))
@pytest.mark.parametrize("sfx,dt", SFX)
@pytest.mark.parametrize("method", ["360", "180"])
def test_helical(port, name, sfx, dt, method):
    """Helical rebinning, bit for bit, including where the reference throws
    (the status codes of its two runtime_errors)."""
    from oracle import HelicalError
    c = gc.load(name)
    h = gc.heli(c)
    x = c["in_f64"].astype(dt)
    want = int(c[f"status{method}"])
    try:
        out, outside = port.helical(x, h, method)
        got = 1
    except HelicalError as e:
        got = e.code
    assert got == want
    if want == 1:
        assert not outside
        assert np.array_equal(out, c[f"out{method}_{sfx}"])


def test_helical_first_view_zero_reads_zero():
    """180LI slice whose first view is 0: the complementary rays just before it
    read as 0 and are reported (the reference reads out of bounds there, so
    this case has no reference fixture).  Pitch 0.5, so that the rays half a
    rotation away still reach the detector rows."""
    from oracle import Heli, Oracle
    h = Heli.make(ns=32, nt=6, na=80, ds=1.0, dt=1.0, view_per_rot=40, couch_mov=3 * 0.5 / 40,
                  nz=1, dz=0.5, z0=20 * 3 * 0.5 / 40, thickness=0.5, dso=500.0, dsd=1000.0)
    x = np.ones((h.na, h.nt, h.ns))
    out, outside = Oracle("port").helical(x, h, "180")
    assert outside and np.isfinite(out).all()
    out360, outside360 = Oracle("port").helical(np.ones((120, 6, 32)), Heli.make(
        ns=32, nt=6, na=120, ds=1.0, dt=1.0, view_per_rot=40, couch_mov=6 * 0.5 / 40, nz=1,
        dz=0.5, z0=40 * 6 * 0.5 / 40, thickness=0.5, dso=500.0, dsd=1000.0), "360")
    assert not outside360 and np.allclose(out360, 1.0)


def _dot_rel(a_x, y, x, at_y):
    lhs = float(np.vdot(a_x.astype(np.float64), y.astype(np.float64)))
    rhs = float(np.vdot(x.astype(np.float64), at_y.astype(np.float64)))
    return abs(lhs - rhs) / abs(lhs)


@pytest.mark.parametrize("name", gc.names("par"))
def test_par_bp_adjoint_dot(port, name):
    c = gc.load(name)
    g = gc.geom(c)
    rng = np.random.default_rng(5)
    x = rng.standard_normal((g.na, g.ns))
    y = rng.standard_normal((g.ny, g.nx))
    assert _dot_rel(port.bp_par_2d(x, g), y, x, port.bp_par_2d_grad(y, g)) < 1e-12


def test_fan_angle_adjoint_dot(port):
    c = gc.load("fan_angle")
    g = gc.geom(c)
    rng = np.random.default_rng(6)
    x = rng.standard_normal((g.na, g.ns))
    y = rng.standard_normal((g.ny, g.nx))
    lhs = port.bp_fan_2d_angle(x, g, c["angles"])
    assert _dot_rel(lhs, y, x, port.bp_fan_2d_angle_grad(y, g, c["angles"])) < 1e-12


@pytest.mark.parametrize("name", gc.names("fan"))
def test_fan_bp_adjoint_dot(port, name):
    c = gc.load(name)
    g = gc.geom(c)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((g.na, g.ns))
    y = rng.standard_normal((g.ny, g.nx))
    assert _dot_rel(port.bp_fan_2d(x, g), y, x, port.bp_fan_2d_grad(y, g)) < 1e-12


def test_row_threads_identical():
    from oracle import Oracle
    c = gc.load("fan_full")
    g = gc.geom(c)
    one = Oracle("port", threads=1).bp_fan_2d(c["filtered_f32"], g)
    many = Oracle("port", threads=7).bp_fan_2d(c["filtered_f32"], g)
    assert np.array_equal(one, many)


def test_invalid_types_rejected(port):
    p = np.zeros((3, 8), np.float32)
    with pytest.raises(ValueError):
        port.fan_weighting(p, 1.0, 0.0, 500.0, 1000.0, 3)
    with pytest.raises(ValueError):
        port.ramp_taps(8, 1.0, 1000.0, 5)
