"""The FP32 ray-driven projector's table forms and chunk paths on the GPU.

* Rays whose (begin, offset) entries are off their view's model line (a
  caller's table that is not one line per view) read their own records: the
  per-call entry point matches the oracle run on the same table, and the plan
  (one image: the projector makes its own transposed copy; a batch: a separate
  copy) matches the per-call entry point bit for bit.
* Images whose bands take the projector's 8-row and 2-row chunk kernels (nx
  above 1024 and above 2048) match the oracle, and so does a geometry with
  more ray slots than one round of one CTA per SM.
Reference: src/fp_par_2d.cc:149-280 (the table and the ray march).
"""
import ctypes
import math

import numpy as np
import pytest

from gpu_helpers import cuda, fp_op, host, rel_l2

pytestmark = pytest.mark.gpu


def _geom(n, na):
    ns = int(math.ceil(n * 1.45)) | 1
    return dict(ns=ns, na=na, ds=0.5, orbit=math.pi / na, offset_s=0.0, orbit_start=0.0,
                nx=n, ny=n, dx=0.5, dy=0.5, offset_x=0.0, offset_y=0.0, fov=-1.0)


@pytest.fixture(scope="module")
def oracle_port():
    import os
    from oracle import Oracle
    return Oracle("port", threads=os.cpu_count() or 1)


def _per_call(op, imgs, tables):
    import torch
    from ct_recon_extensions_gb300 import _lib
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    out = torch.empty((imgs.shape[0], op.na, op.ns), dtype=torch.float32, device="cuda")
    _lib.call("ctr_fp_par_2d_f32", ctypes.byref(op.p), _ptr(imgs), _ptr(out), *map(_ptr, tables),
              imgs.shape[0], _stream())
    return out


def _plan(op, imgs, tables, batches):
    """Plan made from `tables` for the largest batch, run on each batch size."""
    import torch
    from ct_recon_extensions_gb300 import _lib
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.call("ctr_fp_par_2d_plan_create", ctypes.byref(op.p), *map(_ptr, tables), max(batches),
              ctypes.byref(h), _stream())
    outs = []
    try:
        for b in batches:
            out = torch.empty((b, op.na, op.ns), dtype=torch.float32, device="cuda")
            _lib.call("ctr_fp_par_2d_plan_run", h, _ptr(imgs[:b]), _ptr(out), b, _stream())
            outs.append(out)
        torch.cuda.synchronize()
    finally:
        lib.ctr_fp_par_2d_plan_destroy(h)
    return outs


def test_fp_rays_off_the_view_model(oracle_port):
    import torch
    from oracle import Geom
    d = _geom(128, 90)
    g = Geom.make(**d)
    op = fp_op(d)
    sc, bo, ux = (host(t) for t in op.tables(torch.device("cuda")))
    rng = np.random.default_rng(31)
    bo = bo.copy()
    # 15 % of the rays start up to 2e-3 px off their view's line
    pick = rng.random(bo.shape[:2]) < 0.15
    bo[..., 0] += np.where(pick, rng.uniform(-2e-3, 2e-3, bo.shape[:2]), 0.0)
    # a few rays of view 7 step differently from the view
    bo[7, 10:14, 1] *= 1.0 + 1e-7
    # view 11's starts bend away from a line
    i = np.arange(d["ns"])
    bo[11, :, 0] += 1e-5 * (i - d["ns"] / 2) ** 2 / d["ns"]
    tables = (cuda(sc), cuda(bo), torch.as_tensor(ux, device="cuda"))
    imgs = cuda(np.stack([rng.random((128, 128)), rng.standard_normal((128, 128)),
                          rng.random((128, 128))]).astype(np.float32))
    ref = _per_call(op, imgs, tables)
    torch.cuda.synchronize()
    for k in range(3):
        want = oracle_port.fp_par_2d(host(imgs[k]), g, tables=(sc, bo, ux))
        assert rel_l2(host(ref[k]), want) <= 1e-5
    one, three = _plan(op, imgs, tables, (1, 3))
    assert torch.equal(one[0], ref[0])
    assert torch.equal(three, ref)


@pytest.mark.parametrize("n", [1100, 2100])
def test_fp_chunk_paths_vs_oracle(oracle_port, n):
    """nx = 1100 takes 8-row bands and chunks, nx = 2100 6-row bands and
    2-row chunks; the FoV-covering detector keeps every ray range exact."""
    import torch
    from oracle import Geom
    d = _geom(n, 36)
    g = Geom.make(**d)
    op = fp_op(d)
    rng = np.random.default_rng(n)
    img = rng.random((n, n)).astype(np.float32)
    out = host(op.forward(cuda(img)))  # the plan, one image
    assert rel_l2(out, oracle_port.fp_par_2d(img, g)) <= 1e-5
    ref = _per_call(op, cuda(img)[None], op.tables(torch.device("cuda")))
    torch.cuda.synchronize()
    assert np.array_equal(out, host(ref[0]))


def test_fp_many_slots_vs_oracle(oracle_port):
    """720 views x 1501 channels on a 256^2 image: more slots than one CTA per
    SM holds in a round, so the projector runs more CTAs than SMs and the plan
    keeps the separate transposed copy."""
    import torch
    from oracle import Geom
    d = dict(ns=1501, na=720, ds=0.25, orbit=math.pi / 720, offset_s=0.0, orbit_start=0.0,
             nx=256, ny=256, dx=0.5, dy=0.5, offset_x=0.0, offset_y=0.0, fov=-1.0)
    g = Geom.make(**d)
    op = fp_op(d)
    rng = np.random.default_rng(77)
    imgs = cuda(np.stack([rng.random((256, 256)), rng.standard_normal((256, 256))]).astype(np.float32))
    out = host(op.forward(imgs))
    for k in range(2):
        assert rel_l2(out[k], oracle_port.fp_par_2d(host(imgs[k]), g)) <= 1e-5
    ref = _per_call(op, imgs, op.tables(torch.device("cuda")))
    torch.cuda.synchronize()
    assert np.array_equal(out, host(ref))
    assert np.array_equal(host(op.forward(imgs[1])), out[1])
