"""The FP32 backprojectors on launches split across the SMs (stream-K: a
tile's views shared by several CTAs and summed in segment order): a batch of
sinograms equals per-item calls, results repeat bit for bit run to run, and
odd image sizes (partial tiles) agree with the oracle."""
import math

import numpy as np
import pytest

from gpu_helpers import TOL_F32, cuda, fan_op, host, par_op, rel_l2

pytestmark = pytest.mark.gpu

# batch vs items: same taps, different split of the views over CTAs
TOL_SPLIT = 1e-6


def _geoms():
    from ct_recon_extensions_gb300 import synthetic as syn
    par = dict(syn.parallel_config_2())
    fan = dict(syn.fan_config_1())
    odd = dict(ns=301, na=250, ds=1.0, orbit=math.pi / 250, offset_s=0.3, orbit_start=0.1, nx=97,
               ny=97, dx=1.2, dy=1.2, offset_x=0.0, offset_y=0.0, fov=-1.0)
    return [("par", par), ("fan", fan), ("par_odd", odd)]


@pytest.mark.parametrize("name,g", _geoms(), ids=[n for n, _ in _geoms()])
def test_batch_equals_items_and_repeats(name, g):
    op = fan_op(g) if name == "fan" else par_op(g)
    rng = np.random.default_rng(11)
    sino = rng.random((3, g["na"], g["ns"]), dtype=np.float32)
    x = cuda(sino)
    batch = host(op.forward(x))
    again = host(op.forward(x))
    assert np.array_equal(batch, again)  # deterministic
    for b in range(3):
        one = host(op.forward(x[b:b + 1]))[0]
        assert rel_l2(batch[b], one) <= TOL_SPLIT


def test_odd_size_against_oracle():
    from oracle import Geom, Oracle
    name, g = _geoms()[2]
    op = par_op(g)
    rng = np.random.default_rng(12)
    sino = rng.random((g["na"], g["ns"]), dtype=np.float32)
    y = host(op.forward(cuda(sino)))
    G = Geom.make(g["ns"], g["na"], g["ds"], g["orbit"], g["nx"], g["ny"], g["dx"], g["dy"],
                  g["offset_s"], g["orbit_start"], g["offset_x"], g["offset_y"])
    ref = Oracle("port", threads=8).bp_par_2d(sino, G)
    assert rel_l2(y, ref) <= TOL_F32
