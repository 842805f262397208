"""FP32 backprojection plans (ctr_bp_*_plan_*): the plan keeps the tables, the
stream-split scratch (its tile counters reset by the kernel) and each (tile,
view)'s constants, and must give the per-call entry points' results bit for
bit: at the parallel drop-in and fan sizes, in batches that take the stream
split and one that does not, and over repeated runs.  Reference:
src/bp_par_2d.cc:51-90, src/bp_fan_2d.cc:46-91."""
import ctypes

import numpy as np
import pytest

from gpu_helpers import cuda, fan_op, par_op

pytestmark = pytest.mark.gpu


def _per_call_par(op, proj):
    import torch
    from ct_recon_extensions_gb300 import _lib
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    img = torch.empty((proj.shape[0], op.ny, op.nx), dtype=torch.float32, device="cuda")
    xcos, ysin = op.tables(proj.device)
    _lib.call("ctr_bp_par_2d_f32", ctypes.byref(op.p), _ptr(proj), _ptr(img), _ptr(xcos), _ptr(ysin), None,
              proj.shape[0], _stream())
    return img


def _per_call_fan(op, proj):
    import torch
    from ct_recon_extensions_gb300 import _lib
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    img = torch.empty((proj.shape[0], op.ny, op.nx), dtype=torch.float32, device="cuda")
    _lib.call("ctr_bp_fan_2d_f32", ctypes.byref(op.p), _ptr(proj), _ptr(img), *map(_ptr, op.tables(proj.device)),
              proj.shape[0], _stream())
    return img


@pytest.mark.parametrize("geo", ["par", "fan"])
def test_bp_plan_matches_per_call(geo):
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2() if geo == "par" else syn.fan_config_1()
    op = par_op(d) if geo == "par" else fan_op(d)
    per_call = _per_call_par if geo == "par" else _per_call_fan
    rng = np.random.default_rng(5)
    # 16 items of 512^2: 2048 tiles, beyond the stream split (one CTA a tile)
    stack = cuda(rng.standard_normal((16, d["na"], d["ns"])).astype(np.float32))
    for b in (1, 3, 16, 1):
        got = op.forward(stack[:b])
        want = per_call(op, stack[:b])
        torch.cuda.synchronize()
        assert torch.equal(got, want), b
    again = op.forward(stack[:3])  # counters reset by the previous runs
    torch.cuda.synchronize()
    assert torch.equal(again, per_call(op, stack[:3]))


@pytest.mark.parametrize("geo", ["par", "fan"])
def test_bp_plan_adjoint_matches_per_call(geo):
    """The plan's adjoint against the per-call adjoint entry point (the same
    taps; the float atomics that add each tile's window may order the last
    bits differently)."""
    import torch
    from ct_recon_extensions_gb300 import _lib
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    from gpu_helpers import host, rel_l2
    d = syn.parallel_config_2() if geo == "par" else syn.fan_config_1()
    op = par_op(d) if geo == "par" else fan_op(d)
    rng = np.random.default_rng(8)
    imgs = cuda(rng.standard_normal((3, d["ny"], d["nx"])).astype(np.float32))
    got = op.adjoint(imgs)
    want = torch.empty_like(got)
    if geo == "par":
        xcos, ysin = op.tables(imgs.device)
        _lib.call("ctr_bp_par_2d_grad_f32", ctypes.byref(op.p), _ptr(imgs), _ptr(want), _ptr(xcos), _ptr(ysin),
                  3, _stream())
    else:
        _lib.call("ctr_bp_fan_2d_grad_f32", ctypes.byref(op.p), _ptr(imgs), _ptr(want),
                  *map(_ptr, op.tables(imgs.device)), 3, _stream())
    torch.cuda.synchronize()
    for k in range(3):
        assert rel_l2(host(got[k]), host(want[k])) <= 1e-6


@pytest.mark.parametrize("geo", ["par", "fan"])
def test_bp_stream_split_whole_tiles_vs_oracle(geo):
    """Three 512^2 images in one call: 384 tiles, still a stream-split launch
    (fewer than four waves of tiles), with more of a tile's view blocks per CTA
    than one tile holds, so CTAs finish whole tiles and go on to the next one
    (re-using their shared view records).  Each image against the oracle."""
    import os
    from oracle import Geom, Oracle
    from ct_recon_extensions_gb300 import synthetic as syn
    from gpu_helpers import host, rel_l2
    d = syn.parallel_config_2() if geo == "par" else syn.fan_config_1()
    g = Geom.make(**d)
    op = par_op(d) if geo == "par" else fan_op(d)
    port = Oracle("port", threads=os.cpu_count() or 1)
    rng = np.random.default_rng(11)
    stack = rng.standard_normal((3, d["na"], d["ns"])).astype(np.float32)
    got = host(op.forward(cuda(stack)))
    for k in range(3):
        want = port.bp_par_2d(stack[k], g) if geo == "par" else port.bp_fan_2d(stack[k], g)
        assert rel_l2(got[k], want) <= 1e-5, k
