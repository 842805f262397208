"""Batched uneven fan FBP (one persistent launch, CUDA graph, autotuned)
against the single-geometry path and the oracle."""
import math

import numpy as np
import pytest

from gpu_helpers import cuda, fan_op, host, ramp_op, rel_l2, weight_op

TOL_PATHS = 1e-5  # the FP32 parity bound

pytestmark = pytest.mark.gpu


def _items(n, seed=11, small=True):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nx = int(rng.integers(24, 90)) if small else int(rng.integers(256, 1025))
        ny = nx if i % 3 else int(rng.integers(20, 80))
        na = int(rng.integers(30, 140)) if small else int(rng.integers(360, 2305))
        ns = int(rng.integers(40, 130)) if small else int(rng.integers(512, 1025))
        out.append(dict(ns=ns, na=na, ds=1.2858 * 736 / ns, orbit=2 * math.pi / na,
                        offset_s=float(rng.uniform(-0.5, 0.5)), orbit_start=float(rng.uniform(0, 1)),
                        nx=nx, ny=ny, dx=256.0 / nx, dy=256.0 / nx, offset_x=0.0, offset_y=0.0,
                        dso=595.0, dsd=1085.6, fov=-1.0))
    return out


@pytest.mark.parametrize("autotune,graph", [(False, False), (True, True)])
def test_batch_matches_single_item_path(autotune, graph):
    import torch
    from ct_recon_extensions_gb300.batch import FanFBPBatch
    from oracle import Geom, Oracle
    port = Oracle("port", threads=8)
    geoms = _items(7)
    rng = np.random.default_rng(3)
    sinos = [cuda(rng.standard_normal((g["na"], g["ns"])).astype(np.float32)) for g in geoms]
    plan = FanFBPBatch(geoms, autotune=autotune, graph=graph)
    info = plan.info()
    assert info["n_items"] == 7 and info["graph"] == int(graph) and info["autotuned"] == int(autotune)
    outs = plan.run(sinos)
    outs2 = plan.run(sinos)  # graph replay with the same pointers
    for g, s, o, o2 in zip(geoms, sinos, outs, outs2):
        w = weight_op(g, g["na"], 1).forward(s)
        f = ramp_op(g, g["na"], 1).forward(w)
        ref = host(fan_op(g).forward(f))
        # the plan's tiles differ from the single-item kernel's, and fast-path
        # channel positions are rounded relative to each tile's window start
        # (to ulp(W)): on these white-noise sinograms the two agree to <= 4.3e-6,
        # and each is within 7.4e-6 of the FP64 oracle
        assert rel_l2(host(o), ref) <= TOL_PATHS
        ref64 = port.fbp_fan(host(s).astype(np.float64), Geom(**g))
        assert rel_l2(host(o), ref64) <= TOL_PATHS
        assert rel_l2(ref, ref64) <= TOL_PATHS
        assert np.array_equal(host(o), host(o2))
    # new output buffers: descriptors are updated, the graph is reused
    fresh = [torch.empty_like(o) for o in outs]
    plan.run(sinos, fresh)
    for o, f in zip(outs, fresh):
        assert np.array_equal(host(o), host(f))


def test_batch_against_oracle():
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.batch import FanFBPBatch
    from oracle import Geom, Oracle
    port = Oracle("port", threads=8)
    geoms = _items(4, seed=5)
    sinos, refs = [], []
    for k, g in enumerate(geoms):
        e = syn.scaled(syn.random_ellipses(100 + k), 0.7)
        s = syn.fan_sinogram(e, g["na"], g["ns"], g["ds"], g["orbit"], g["dso"], g["dsd"],
                             g["orbit_start"], g["offset_s"])
        sinos.append(cuda(s))
        refs.append(port.fbp_fan(s, Geom(**g)))
    outs = FanFBPBatch(geoms).run(sinos)
    for o, r in zip(outs, refs):
        assert rel_l2(host(o), r) <= 1e-5


def test_batch_config3_sizes():
    """The plan at the batched benchmark's sizes (items of syn.batched_config_3:
    image 256^2-1024^2, 360-2304 views, 512-1024 channels): the largest item,
    the smallest and three others, each against the oracle's T=float FBP on two
    strips of 16 image rows and against the single-item path on the whole
    image."""
    import os
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.batch import FanFBPBatch
    from oracle import Geom, Oracle
    port = Oracle("port", threads=os.cpu_count() or 1)
    items = syn.batched_config_3()
    cost = [it["nx"] * it["ny"] * it["na"] for it in items]
    pick = sorted({int(np.argmax(cost)), int(np.argmin(cost)), 7, 23, 41})
    geoms = [{k: v for k, v in items[i].items() if k != "seed"} for i in pick]
    hosts = [syn.fan_sinogram(syn.random_ellipses(items[i]["seed"]), g["na"], g["ns"], g["ds"],
                              g["orbit"], g["dso"], g["dsd"]) for i, g in zip(pick, geoms)]
    outs = FanFBPBatch(geoms).run([cuda(s) for s in hosts])
    for g, s, o in zip(geoms, hosts, outs):
        img = host(o)
        w = weight_op(g, g["na"], 1).forward(cuda(s))
        single = host(fan_op(g).forward(ramp_op(g, g["na"], 1).forward(w)))
        assert rel_l2(img, single) <= TOL_PATHS
        f = port.ramp_filter(port.fan_weighting(s, g["ds"], g["offset_s"], g["dso"], g["dsd"], 1),
                             g["ds"], g["dsd"], 1)
        for r0 in (g["ny"] // 4, (3 * g["ny"]) // 4):
            k = 16
            off_y = (g["ny"] - 1) / 2 + g["offset_y"] - r0 - (k - 1) / 2
            gs = Geom.make(g["ns"], g["na"], g["ds"], g["orbit"], g["nx"], k, g["dx"], g["dy"],
                           g["offset_s"], g["orbit_start"], g["offset_x"], off_y, g["dso"],
                           g["dsd"], g["fov"])
            assert rel_l2(img[r0:r0 + k], port.bp_fan_2d(f, gs)) <= TOL_PATHS
