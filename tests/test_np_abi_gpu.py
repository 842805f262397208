"""The reference's numpy front end (FanFBP2DAngle over the numpy-extension ABI)
against the reference's own T=double outputs for the same inputs."""
import numpy as np
import pytest

import golden_cases as gc
from gpu_helpers import rel_l2


def test_set_device_cpu_mode_refused():
    from ct_recon_extensions_gb300 import np_ctrecon, build
    build.build()
    lib = np_ctrecon._load()
    assert lib.set_device(-1) is False
    assert "CPU" in np_ctrecon.last_error()


@pytest.mark.gpu
def test_fan_fbp_2d_angle_numpy_path():
    from ct_recon_extensions_gb300 import np_ctrecon
    from oracle import Oracle
    c = gc.load("fan_angle")
    g = c["geom"]
    param = dict(device=0, ns=g["ns"], na=g["na"], ds=g["ds"], offset_s=g["offset_s"], dso=g["dso"],
                 dsd=g["dsd"], angles=c["angles"], nx=g["nx"], ny=g["ny"], dx=g["dx"], dy=g["dy"],
                 offset_x=g["offset_x"], offset_y=g["offset_y"], fov=g["fov"], orbit=0.5)
    fbp = np_ctrecon.FanFBP2DAngle(param)
    sino = c["sino_f64"].copy()
    out = fbp.run(sino)
    # the reference weights in place, filters, backprojects and scales by orbit
    assert np.allclose(sino, c["weighted1_f64"], rtol=1e-14, atol=0)
    expect = c["bp_f64"] * 0.5
    assert rel_l2(out, expect) <= 1e-11
    port = Oracle("port")
    from oracle import Geom
    ref = port.bp_fan_2d_angle(port.ramp_filter(c["weighted1_f64"], g["ds"], g["dsd"], 1),
                               Geom(**g), c["angles"]) * 0.5
    assert rel_l2(out, ref) <= 1e-11
