"""Parity of the CUDA path (through the C ABI) with the reference.

* small cases: every operator against the fixtures the reference's own CPU
  code produced (tests/golden), T=float kernels at rel-L2 <= 1e-5 and
  T=double kernels at rel-L2 <= 1e-11;
* full benchmark sizes: the FP32 FBP chains against the oracle port, at
  rel-L2 <= 1e-5 against its T=float output and <= 1e-4 against FP64;
* adjoint dot tests, batching and the kernels' self-check flags.
"""
import ctypes
import math

import numpy as np
import pytest

import golden_cases as gc
from gpu_helpers import (angle_op, cuda, dot_rel, fan_op, fp_op, host, par_op, ramp_op,
                         rel_l2, tol, weight_op)

pytestmark = pytest.mark.gpu

DT = [("f32", np.float32), ("f64", np.float64)]


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    import torch
    from ct_recon_extensions_gb300 import build, _lib
    build.build()
    assert torch.cuda.is_available()
    assert _lib.load().ctr_device_check() == 0, _lib.load().ctr_last_error()
    flags = ctypes.c_uint(0)
    _lib.load().ctr_kernel_flags(ctypes.byref(flags), 1)
    yield
    _lib.load().ctr_kernel_flags(ctypes.byref(flags), 1)
    assert flags.value == 0, f"kernel self-check flags raised: {flags.value:#x}"


@pytest.mark.parametrize("name", gc.names(("fan", "fan_angle")))
@pytest.mark.parametrize("sfx,dt", DT)
def test_fan_chain(name, sfx, dt):
    c = gc.load(name)
    g = c["geom"]
    p = cuda(c[f"sino_{sfx}"])
    for wt in (1, 2):
        op = weight_op(g, g["na"], wt)
        w = host(op.forward(p))
        assert rel_l2(w, c[f"weighted{wt}_{sfx}"]) <= 1e-7
        assert rel_l2(host(op.adjoint(p)), c[f"weighted{wt}_grad_{sfx}"]) <= 1e-7
    filt = host(ramp_op(g, g["na"], 1).forward(cuda(c[f"weighted1_{sfx}"])))
    assert rel_l2(filt, c[f"filtered_{sfx}"]) <= tol(dt)
    assert rel_l2(host(ramp_op(g, g["na"], 1).adjoint(p)), c[f"filtered_grad_{sfx}"]) <= tol(dt)
    flat = host(ramp_op(g, g["na"], 2).forward(cuda(c[f"weighted2_{sfx}"])))
    assert rel_l2(flat, c[f"filtered_flat_{sfx}"]) <= tol(dt)
    if c["kind"] == "fan":
        op = fan_op(g)
        assert rel_l2(host(op.forward(cuda(c[f"filtered_{sfx}"]))), c[f"bp_{sfx}"]) <= tol(dt)
        assert rel_l2(host(op.adjoint(cuda(c[f"img_in_{sfx}"]))), c[f"bp_grad_{sfx}"]) <= tol(dt)
    else:
        op = angle_op(g, c["angles"])
        assert rel_l2(host(op.forward(cuda(c[f"filtered_{sfx}"]))), c[f"bp_{sfx}"]) <= tol(dt)


@pytest.mark.parametrize("name", gc.names("par"))
@pytest.mark.parametrize("sfx,dt", DT)
def test_par_bp(name, sfx, dt):
    c = gc.load(name)
    g = c["geom"]
    filt = host(ramp_op(g, g["na"], 0, dsd=-1.0).forward(cuda(c[f"sino_{sfx}"])))
    assert rel_l2(filt, c[f"filtered_{sfx}"]) <= tol(dt)
    img = host(par_op(g).forward(cuda(c[f"filtered_{sfx}"])))
    assert rel_l2(img, c[f"bp_{sfx}"]) <= tol(dt)


@pytest.mark.parametrize("sfx,dt", DT)
def test_bppar2d_torch_binding(sfx, dt):
    """The reference's PyTorch extension functions (pytorch/bp_par_2d_ops.cc):
    bppar2d_prep_forward's buffers into bppar2d_forward, against the golden
    backprojection; any method but "pixdriven" raises its error."""
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    c = gc.load("par")
    g = c["geom"]
    args = (g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"], g["orbit_start"], g["nx"],
            g["ny"], g["dx"], g["dy"], g["offset_x"], g["offset_y"], g["fov"])
    bufs = tc.bppar2d_prep_forward("pixdriven", *args)
    assert tuple(bufs[0].shape) == (g["nx"], g["na"]) and tuple(bufs[1].shape) == (g["ny"], g["na"])
    img = tc.bppar2d_forward(cuda(c[f"filtered_{sfx}"]), *bufs, "pixdriven", *args)
    assert rel_l2(host(img), c[f"bp_{sfx}"]) <= tol(dt)
    with pytest.raises(RuntimeError, match="Only pixdriven is available now"):
        tc.bppar2d_prep_forward("raydriven", *args)
    with pytest.raises(RuntimeError, match="Only pixdriven is available now"):
        tc.bppar2d_forward(cuda(c[f"filtered_{sfx}"]), *bufs, "raydriven", *args)


@pytest.mark.parametrize("sfx,dt", DT)
def test_single_view(sfx, dt):
    c = gc.load("sv")
    g = c["geom"]
    out = host(par_op(g).single_view(cuda(c[f"sino_{sfx}"])))[0]
    assert out.shape == c[f"sv_{sfx}"].shape
    assert rel_l2(out, c[f"sv_{sfx}"]) <= tol(dt)


@pytest.mark.parametrize("name", gc.names("fp"))
@pytest.mark.parametrize("sfx,dt", DT)
def test_fp_ray_driven(name, sfx, dt):
    c = gc.load(name)
    g = c["geom"]
    op = fp_op(g)
    assert rel_l2(host(op.forward(cuda(c[f"img_{sfx}"]))), c[f"fp_{sfx}"]) <= tol(dt)
    assert rel_l2(host(op.adjoint(cuda(c[f"proj_in_{sfx}"]))), c[f"fp_grad_{sfx}"]) <= tol(dt)


def _cast_op(g, step):
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    return tc.ParallelProjection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                     g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                     g["offset_x"], g["offset_y"], g["fov"], method="raycasting",
                                     step_size=step)


@pytest.mark.parametrize("name", gc.names("cast"))
@pytest.mark.parametrize("sfx,dt", DT)
def test_fp_ray_casting(name, sfx, dt):
    c = gc.load(name)
    g = c["geom"]
    op = _cast_op(g, float(c["step"]))
    assert rel_l2(host(op.forward(cuda(c[f"img_{sfx}"]))), c[f"cast_{sfx}"]) <= tol(dt)
    with pytest.raises(NotImplementedError):
        op.adjoint(cuda(np.zeros((g["na"], g["ns"]), dt)))


def _dd_op(g):
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    return tc.ParallelProjection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                     g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                     g["offset_x"], g["offset_y"], g["fov"], method="disdriven")


@pytest.mark.parametrize("name", gc.names("dd"))
@pytest.mark.parametrize("sfx,dt", DT)
def test_fp_distance_driven(name, sfx, dt):
    c = gc.load(name)
    g = c["geom"]
    op = _dd_op(g)
    assert rel_l2(host(op.forward(cuda(c[f"img_{sfx}"]))), c[f"dd_{sfx}"]) <= tol(dt)
    assert rel_l2(host(op.adjoint(cuda(c[f"proj_in_{sfx}"]))), c[f"dd_grad_{sfx}"]) <= tol(dt)


# ---- adjoint dot tests --------------------------------------------------------

def _smooth_signed(shape, rng, sigma=6.0):
    """A smooth random field of both signs (white noise low-passed by a
    Gaussian of `sigma` samples), unit standard deviation."""
    f = np.fft.rfft2(rng.standard_normal(shape))
    ky = np.fft.fftfreq(shape[0])[:, None]
    kx = np.fft.rfftfreq(shape[1])[None, :]
    f *= np.exp(-2.0 * (np.pi * sigma) ** 2 * (kx ** 2 + ky ** 2))
    v = np.fft.irfft2(f, s=shape)
    return v / v.std()


def _dot(op, x_shape, y_shape, dt, seed=0, kind="positive"):
    """|<Ax,y> - <x,A^T y>| / |<Ax,y>|, both inner products in FP64.
    kind: "positive" (values in [0.5, 1.5): no cancellation in the inner
    products, so the ratio isolates the operators' mismatch), "smooth" (smooth
    fields of both signs) or "signed" (white noise of both signs: the FP32
    rounding of the kernels themselves then shows, about 1e-6 of the terms).
    Exact transposition entry by entry is checked in test_adjoint_matrix_gpu.py."""
    rng = np.random.default_rng(seed)
    if kind == "positive":
        x = (0.5 + rng.random(x_shape)).astype(dt)
        y = (0.5 + rng.random(y_shape)).astype(dt)
    elif kind == "smooth":
        x = _smooth_signed(x_shape, rng).astype(dt)
        y = _smooth_signed(y_shape, rng).astype(dt)
    else:
        x = rng.standard_normal(x_shape).astype(dt)
        y = rng.standard_normal(y_shape).astype(dt)
    ax = host(op.forward(cuda(x)))
    aty = host(op.adjoint(cuda(y)))
    if kind == "signed":
        # <Ax, y> of independent signed fields is ~ |Ax| |y| / sqrt(size) and may
        # come near zero by chance: normalise by |Ax| |y| instead
        lhs = float(np.vdot(ax.astype(np.float64), y.astype(np.float64)))
        rhs = float(np.vdot(x.astype(np.float64), aty.astype(np.float64)))
        return abs(lhs - rhs) / (np.linalg.norm(ax.astype(np.float64)) * np.linalg.norm(y.astype(np.float64)))
    return dot_rel(ax, y, x, aty)


@pytest.mark.parametrize("sfx,dt", DT)
def test_adjoint_dot(sfx, dt):
    lim = 1e-6 if dt == np.float32 else 1e-12
    c = gc.load("fan_full")["geom"]
    assert _dot(fan_op(c), (c["na"], c["ns"]), (c["ny"], c["nx"]), dt) < lim
    p = gc.load("par_rect_cw")["geom"]
    assert _dot(par_op(p), (p["na"], p["ns"]), (p["ny"], p["nx"]), dt) < lim
    f = gc.load("fp_half")["geom"]
    assert _dot(fp_op(f), (f["ny"], f["nx"]), (f["na"], f["ns"]), dt) < lim
    assert _dot(ramp_op(c, c["na"], 1), (c["na"], c["ns"]), (c["na"], c["ns"]), dt) < lim
    assert _dot(weight_op(c, c["na"], 1), (c["na"], c["ns"]), (c["na"], c["ns"]), dt) < lim


# Signed inputs at the benchmark sizes.  Smooth signed fields: FP32 kernels to
# 1e-6 of <Ax, y>.  White noise of both signs, normalised by |Ax| |y|: FP64
# kernels to 1e-13, FP32 to 1e-7 (the forward backprojector's interpolation
# pairs hold p - (k - kc - 1/2) d in FP32, which rounds at up to W/2 = 40 times
# the size of a white-noise difference d: about 1e-6 of <Ax, y>, 2e-8 of
# |Ax| |y|).  An adjoint that is wrong by a sign or an offset is off by more
# than 1e-3 in either measure.
SIGNED_CASES = [
    ("fan", lambda: __import__("ct_recon_extensions_gb300.synthetic", fromlist=["x"]).fan_config_1(), fan_op, False),
    ("par", lambda: __import__("ct_recon_extensions_gb300.synthetic", fromlist=["x"]).parallel_config_2(), par_op, False),
    ("fp", lambda: __import__("ct_recon_extensions_gb300.synthetic", fromlist=["x"]).parallel_config_2(), fp_op, True),
]


@pytest.mark.parametrize("name,geom,mk,image_in", SIGNED_CASES, ids=[c[0] for c in SIGNED_CASES])
def test_adjoint_dot_signed(name, geom, mk, image_in):
    d = geom()
    sino = (d["na"], d["ns"])
    img = (d["ny"], d["nx"])
    xs, ys = (img, sino) if image_in else (sino, img)
    op = mk(d)
    assert _dot(op, xs, ys, np.float64, seed=1, kind="signed") < 1e-13
    assert _dot(op, xs, ys, np.float32, seed=2, kind="smooth") < 1e-6
    assert _dot(op, xs, ys, np.float32, seed=3, kind="signed") < 1e-7


# ---- batching ----------------------------------------------------------------

def test_batch_matches_items():
    import torch
    c = gc.load("fan_full")
    g = c["geom"]
    op = fan_op(g)
    rng = np.random.default_rng(3)
    stack = np.stack([c["filtered_f32"], rng.standard_normal(c["filtered_f32"].shape).astype(np.float32),
                      np.zeros_like(c["filtered_f32"])])
    out = host(op.forward(cuda(stack)[..., None]))[..., 0]
    for i in range(3):
        one = host(op.forward(cuda(stack[i])))
        assert np.array_equal(out[i], one)
    assert np.all(out[2] == 0)


# ---- full benchmark sizes against the oracle ---------------------------------

@pytest.fixture(scope="module")
def oracle_port():
    import os
    from oracle import Oracle
    return Oracle("port", threads=os.cpu_count() or 1)


def test_fan_fbp_config1(oracle_port):
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.fan_config_1()
    g = Geom.make(**d)
    e = syn.random_ellipses(1000)
    sino = syn.fan_sinogram(e, g.na, g.ns, g.ds, g.orbit, g.dso, g.dsd)
    ref32 = oracle_port.fbp_fan(sino, g)
    ref64 = oracle_port.fbp_fan(sino.astype(np.float64), g)
    w = weight_op(d, d["na"], 1).forward(cuda(sino))
    f = ramp_op(d, d["na"], 1).forward(w)
    img = host(fan_op(d).forward(f))
    assert rel_l2(img, ref32) <= 1e-5
    assert rel_l2(img, ref64) <= 1e-4


def test_parallel_config2(oracle_port):
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    g = Geom.make(**d)
    img0 = syn.rasterize(syn.random_ellipses(2000), 512, 512, 0.5, 0.5)
    sino_ref = oracle_port.fp_par_2d(img0, g)
    sino = fp_op(d).forward(cuda(img0))
    assert rel_l2(host(sino), sino_ref) <= 1e-5
    filt_ref = oracle_port.ramp_filter(sino_ref, g.ds, -1.0, 0)
    rec_ref = oracle_port.bp_par_2d(filt_ref, g)
    filt = ramp_op(d, d["na"], 0, dsd=-1.0).forward(cuda(sino_ref))
    rec = host(par_op(d).forward(filt))
    assert rel_l2(rec, rec_ref) <= 1e-5
    rec64 = oracle_port.bp_par_2d(oracle_port.ramp_filter(sino_ref.astype(np.float64), g.ds, -1.0, 0), g)
    assert rel_l2(rec, rec64) <= 1e-4


def test_fan_config1_white_noise(oracle_port):
    """Fan weighting + ramp(fan) + bp_fan_2d at config 1 (720 views x 736
    channels -> 512^2) on a white-noise sinogram (detector differences as large
    as the values: the worst case for FP32 channel positions) against the
    reference's CPU algorithm, T=float and FP64."""
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.fan_config_1()
    g = Geom.make(**d)
    sino = np.random.default_rng(17).standard_normal((d["na"], d["ns"])).astype(np.float32)
    w = weight_op(d, d["na"], 1).forward(cuda(sino))
    rec = host(fan_op(d).forward(ramp_op(d, d["na"], 1).forward(w)))
    assert rel_l2(rec, oracle_port.fbp_fan(sino, g)) <= 1e-5  # measured ~2.5e-6
    assert rel_l2(rec, oracle_port.fbp_fan(sino.astype(np.float64), g)) <= 1e-5


def test_ramp_filter_f32_config5(oracle_port):
    """The FP32 ramp filter (fan) of a config-5 sinogram (2304 views x 1472
    channels, analytic ellipses) against the oracle in FP64; its taps nearly
    cancel on smooth data, the case that FP32 partial sums lose."""
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.large_config_5()
    g = Geom.make(**d)
    e = syn.random_ellipses(5000)
    sino = syn.fan_sinogram(e, d["na"], d["ns"], d["ds"], d["orbit"], d["dso"], d["dsd"])
    w = weight_op(d, d["na"], 1).forward(cuda(sino))
    out = host(ramp_op(d, d["na"], 1).forward(w))
    # the reference's T=float filter sums in double (src/filter.cc:77-89): FP64
    # on the same FP32 weighted sinogram
    ref = oracle_port.ramp_filter(host(w).astype(np.float64), g.ds, g.dsd, 1)
    assert rel_l2(out, ref) <= 1e-5  # measured ~1e-6 (1.3e-5 with uncentred FP32 sums)
    grad = host(ramp_op(d, d["na"], 1).adjoint(w))
    gref = oracle_port.ramp_filter(host(w).astype(np.float64), g.ds, g.dsd, 1, grad=True)
    assert rel_l2(grad, gref) <= 1e-5


def test_parallel_config2_white_noise(oracle_port):
    """Ramp + bp_par_2d at 512^2 x 720 views x 729 bins on a white-noise sinogram
    (detector differences as large as the values: the worst case for the FP32
    channel positions) against the reference's CPU algorithm."""
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    g = Geom.make(**d)
    sino = np.random.default_rng(7).standard_normal((d["na"], d["ns"])).astype(np.float32)
    rec = host(par_op(d).forward(ramp_op(d, d["na"], 0, dsd=-1.0).forward(cuda(sino))))
    ref = oracle_port.bp_par_2d(oracle_port.ramp_filter(sino, g.ds, -1.0, 0), g)
    assert rel_l2(rec, ref) <= 1e-5  # measured ~1.5e-6


def test_single_view_config2_strips(oracle_port):
    """bp_par_2d_sv at config 2 (720 views x 729 bins -> 512 x 512 x 720) on a
    white-noise sinogram: two strips of 8 image rows against the reference's
    CPU algorithm (T=float), plus the image's outer rows, where pixels reach
    the detector ends."""
    import torch
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    sino = np.random.default_rng(19).standard_normal((d["na"], d["ns"])).astype(np.float32)
    out = par_op(d).single_view(cuda(sino))[0]
    for r0 in (0, 200, 504):
        k = 8
        off_y = (d["ny"] - 1) / 2 + d["offset_y"] - r0 - (k - 1) / 2
        gs = Geom.make(d["ns"], d["na"], d["ds"], d["orbit"], d["nx"], k, d["dx"], d["dy"], d["offset_s"],
                       d["orbit_start"], d["offset_x"], off_y, -1.0, -1.0, d["fov"])
        ref = oracle_port.bp_par_2d_sv(sino, gs)
        got = out[r0:r0 + k].cpu().numpy()
        assert got.shape == ref.shape
        assert rel_l2(got, ref) <= 1e-5
    del out
    torch.cuda.empty_cache()


def test_fp_ray_casting_config2(oracle_port):
    """Ray casting at 512^2 (0.5 mm) -> 720 views x 729 bins over pi, FoV radius
    128 mm, step 0.125 pixel, against the oracle (~1.7e9 samples), and a batch
    of 3 equal to its items."""
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = dict(syn.parallel_config_2(), fov=128.0)
    g = Geom.make(**d)
    img0 = syn.rasterize(syn.random_ellipses(2200), 512, 512, 0.5, 0.5)
    op = _cast_op(d, 0.125)
    out = host(op.forward(cuda(img0)))
    assert rel_l2(out, oracle_port.fp_par_2d_cast(img0, g, 0.125)) <= 1e-5
    rng = np.random.default_rng(5)
    stack = np.stack([img0, rng.random((512, 512)).astype(np.float32), np.zeros((512, 512), np.float32)])
    outs = host(op.forward(cuda(stack)))
    assert np.array_equal(outs[0], out)
    assert np.array_equal(outs[1], host(op.forward(cuda(stack[1]))))
    assert np.all(outs[2] == 0)


def test_fp_distance_driven_config2(oracle_port):
    """Distance driven at 512^2 (0.5 mm) -> 720 views x 729 bins over pi and the
    reference's distance-driven grad, against the oracle; a batch of 2 equal to
    its items."""
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    g = Geom.make(**d)
    img0 = syn.rasterize(syn.random_ellipses(2300), 512, 512, 0.5, 0.5)
    op = _dd_op(d)
    out = host(op.forward(cuda(img0)))
    assert rel_l2(out, oracle_port.fp_par_2d_dd(img0, g)) <= 1e-5
    proj = np.random.default_rng(8).standard_normal((d["na"], d["ns"])).astype(np.float32)
    gr = host(op.adjoint(cuda(proj)))
    assert rel_l2(gr, oracle_port.fp_par_2d_dd_grad(proj, g)) <= 1e-5
    stack = np.stack([img0, np.random.default_rng(9).random((512, 512)).astype(np.float32)])
    outs = host(op.forward(cuda(stack)))
    assert np.array_equal(outs[0], out)
    assert np.array_equal(outs[1], host(op.forward(cuda(stack[1]))))


def test_fp_plan_matches_per_call_path():
    """The per-geometry plan (ray tables built once) gives bit-identical
    results to the per-call entry point at config 2, for one image and a batch
    of three, and calls after a plan has grown keep doing so."""
    import ctypes
    import torch
    from ct_recon_extensions_gb300 import _lib
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    d = syn.parallel_config_2()
    op = fp_op(d)
    rng = np.random.default_rng(21)
    imgs = cuda(np.stack([syn.rasterize(syn.random_ellipses(2400), 512, 512, 0.5, 0.5),
                          rng.standard_normal((512, 512)).astype(np.float32),
                          rng.random((512, 512)).astype(np.float32)]))
    ref = torch.empty((3, d["na"], d["ns"]), dtype=torch.float32, device="cuda")
    _lib.call("ctr_fp_par_2d_f32", ctypes.byref(op.p), _ptr(imgs), _ptr(ref),
              *map(_ptr, op.tables(imgs.device)), 3, _stream())
    one = op.forward(imgs[0])           # plan for one image
    three = op.forward(imgs)            # plan grown to three
    torch.cuda.synchronize()
    assert torch.equal(one, ref[0])
    assert torch.equal(three, ref)
    assert torch.equal(op.forward(imgs[1]), ref[1])


def test_fp_adjoint_config2_batch(oracle_port):
    """The FP adjoint at 512^2 x 720 views x 729 bins: against the oracle, and a
    batch of 7 (image groups of the gather plus a remainder) equal to its items."""
    from oracle import Geom
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    g = Geom.make(**d)
    rng = np.random.default_rng(11)
    sino = fp_op(d).forward(cuda(syn.rasterize(syn.random_ellipses(2100), 512, 512, 0.5, 0.5)))
    stack = np.concatenate([host(sino)[None],
                            rng.standard_normal((6, d["na"], d["ns"])).astype(np.float32)])
    op = fp_op(d)
    out = host(op.adjoint(cuda(stack)))
    assert rel_l2(out[0], oracle_port.fp_par_2d_grad(stack[0], g)) <= 1e-5
    assert rel_l2(out[3], oracle_port.fp_par_2d_grad(stack[3], g)) <= 1e-5
    for i in range(7):
        assert np.array_equal(out[i], host(op.adjoint(cuda(stack[i]))))


def test_fp_adjoint_config2_dot():
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    assert _dot(fp_op(d), (d["ny"], d["nx"]), (d["na"], d["ns"]), np.float32) < 1e-6
    assert _dot(par_op(d), (d["na"], d["ns"]), (d["ny"], d["nx"]), np.float32) < 1e-6
    f = syn.fan_config_1()
    assert _dot(fan_op(f), (f["na"], f["ns"]), (f["ny"], f["nx"]), np.float32) < 1e-6


def test_cpu_tensor_rejected():
    import torch
    c = gc.load("par")["geom"]
    with pytest.raises(ValueError):
        par_op(c).forward(torch.zeros((c["na"], c["ns"])))
