"""Autograd: every differentiable operator's backward is the hand-written
adjoint kernel.  Checked by central finite differences in FP64
(torch.autograd.gradcheck) on small geometries, through the fan chain
(fan_weighting -> ramp filter -> bp_fan_2d) with respect to the sinogram, and
by a few steps of gradient descent on ||A x - y||^2 for the parallel pair with
a noisy sinogram (batch of images, FP32)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FAN = dict(ns=20, na=12, ds=12.0, orbit=2 * math.pi / 12, offset_s=0.3, orbit_start=0.1,
           nx=16, ny=14, dx=8.0, dy=8.0, offset_x=0.5, offset_y=-0.25, dso=595.0,
           dsd=1085.6, fov=-1.0)
PAR = dict(ns=23, na=10, ds=6.0, orbit=math.pi / 10, offset_s=-0.2, orbit_start=0.05,
           nx=16, ny=16, dx=6.0, dy=6.0, offset_x=0.0, offset_y=0.0, fov=-1.0)


def _ops():
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    f = FAN
    p = PAR
    fan = tc.FanBackprojection2DOp(f["ns"], f["na"], f["ds"], f["orbit"], f["offset_s"],
                                   f["orbit_start"], f["nx"], f["ny"], f["dx"], f["dy"],
                                   f["offset_x"], f["offset_y"], f["dso"], f["dsd"], f["fov"])
    par = tc.ParallelBackprojection2DOp(p["ns"], p["na"], p["ds"], p["orbit"], p["offset_s"],
                                        p["orbit_start"], p["nx"], p["ny"], p["dx"], p["dy"],
                                        p["offset_x"], p["offset_y"], p["fov"])
    fp = tc.ParallelProjection2DOp(p["ns"], p["na"], p["ds"], p["orbit"], p["offset_s"],
                                   p["orbit_start"], p["nx"], p["ny"], p["dx"], p["dy"],
                                   p["offset_x"], p["offset_y"], p["fov"])
    weight = tc.FanWeightingOp(f["ns"], f["na"], f["ds"], f["offset_s"], f["dso"], f["dsd"], 1)
    ramp_fan = tc.RampFilterOp(f["ns"], f["na"], f["ds"], f["dsd"], 1)
    ramp_par = tc.RampFilterOp(p["ns"], p["na"], p["ds"], -1.0, 0)
    return dict(fan=fan, par=par, fp=fp, weight=weight, ramp_fan=ramp_fan, ramp_par=ramp_par)


def _x(shape, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    return torch.randn(shape, generator=g, dtype=torch.float64).cuda().requires_grad_(True)


@pytest.mark.parametrize("name", ["fan", "par", "fp", "weight", "ramp_fan", "ramp_par"])
def test_gradcheck_fp64(name):
    import torch
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    op = _ops()[name]
    shape = (PAR["ny"], PAR["nx"]) if name == "fp" else (
        (FAN["na"], FAN["ns"]) if name in ("fan", "weight", "ramp_fan") else (PAR["na"], PAR["ns"]))
    x = _x(shape, 7)
    assert torch.autograd.gradcheck(lambda t: tc.apply(op, t), (x,), eps=1e-6, atol=1e-7, rtol=1e-6)
    # and the adjoint as a differentiable op of its own
    y = _x(tuple(tc.apply(op, x).shape), 8)
    assert torch.autograd.gradcheck(lambda t: tc.apply_adjoint(op, t), (y,), eps=1e-6, atol=1e-7,
                                    rtol=1e-6)


def test_gradcheck_fan_chain_wrt_sinogram():
    import torch
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    ops = _ops()

    def chain(s):
        return tc.apply(ops["fan"], tc.apply(ops["ramp_fan"], tc.apply(ops["weight"], s)))

    s = _x((FAN["na"], FAN["ns"]), 9)
    assert torch.autograd.gradcheck(chain, (s,), eps=1e-6, atol=1e-7, rtol=1e-6)


def test_gradient_descent_parallel_pair():
    # the differentiable-pair workload on a small batch: y = A x_true + 1 % noise,
    # GD on ||A x - y||^2 from x = 0 (step 1/L with L from power iteration)
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    d = syn.parallel_config_2()
    d.update(nx=128, ny=128, dx=2.0, dy=2.0, na=180, ns=183, ds=2.0, orbit=math.pi / 180)
    op = tc.ParallelProjection2DOp(d["ns"], d["na"], d["ds"], d["orbit"], d["offset_s"],
                                   d["orbit_start"], d["nx"], d["ny"], d["dx"], d["dy"],
                                   d["offset_x"], d["offset_y"], d["fov"])
    xt = torch.from_numpy(np.stack([syn.rasterize(syn.random_ellipses(4000 + i), 128, 128, 2.0, 2.0)
                                    for i in range(4)])).float().cuda()
    y = op.forward(xt)
    g = torch.Generator(device="cuda").manual_seed(3)
    y = y + 0.01 * y.max() * torch.randn(y.shape, generator=g, device="cuda")
    v = torch.ones_like(xt)
    for _ in range(20):  # power iteration for ||A^T A||
        v = op.adjoint(op.forward(v))
        L = float(v.norm() / math.sqrt(v.numel()))
        v = v / v.norm() * math.sqrt(v.numel())
    x = torch.zeros_like(xt, requires_grad=True)
    losses = []
    for _ in range(15):
        loss = 0.5 * (tc.apply(op, x) - y).pow(2).sum()
        loss.backward()
        with torch.no_grad():
            x -= x.grad / L
            x.grad = None
        losses.append(float(loss.detach()))
    assert all(b < a for a, b in zip(losses, losses[1:]))
    assert losses[-1] < 0.2 * losses[0]


def test_gradient_descent_fan_matched_pair():
    """Fan-beam GD through the matched projector fan_projection_2d (the exact
    adjoint of fan_backprojection_2d): its backward is the backprojection, the
    pair passes the dot test, and the loss falls monotonically."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    n, na, ns, dx, ds, dso, dsd = 96, 120, 128, 2.0, 2.6, 595.0, 1085.6
    args = dict(img_shape=(n, n), img_space=(dx, dx), proj_shape=(na, ns), channel_space=ds,
                orbit=2 * math.pi / na, dso=dso, dsd=dsd)
    xt = torch.from_numpy(np.stack([syn.rasterize(syn.random_ellipses(4200 + i), n, n, dx, dx)
                                    for i in range(2)])).float().cuda()[..., None]
    g = torch.Generator(device="cuda").manual_seed(5)
    yr = torch.randn((2, na, ns, 1), generator=g, device="cuda")
    ax = tc.fan_projection_2d(xt, **args)
    aty = tc.fan_backprojection_2d(yr, **args)
    lhs, rhs = float((ax * yr).sum()), float((xt * aty).sum())
    assert abs(lhs - rhs) <= 1e-5 * float((ax.abs() * yr.abs()).sum())
    y = ax + 0.01 * ax.max() * torch.randn(ax.shape, generator=g, device="cuda")
    v = torch.ones_like(xt)
    for _ in range(20):  # power iteration for ||A^T A||
        v = tc.fan_backprojection_2d(tc.fan_projection_2d(v, **args), **args)
        L = float(v.norm() / math.sqrt(v.numel()))
        v = v / v.norm() * math.sqrt(v.numel())
    x = torch.zeros_like(xt, requires_grad=True)
    losses = []
    for _ in range(12):
        loss = 0.5 * (tc.fan_projection_2d(x, **args) - y).pow(2).sum()
        loss.backward()
        with torch.no_grad():
            x -= x.grad / L
            x.grad = None
        losses.append(float(loss.detach()))
    assert all(b < a for a, b in zip(losses, losses[1:]))
    assert losses[-1] < 0.3 * losses[0]
