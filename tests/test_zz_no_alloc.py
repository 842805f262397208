"""ctr_fp_par_2d_f32_noalloc: the allocation-free FP32 forward projection.

Called through the C ABI and compared with ctr_fp_par_2d_f32 (stream-ordered
scratch) on the same inputs, twice in a row on one stream, and with the
reference's golden output.  That it allocates nothing is read off the
device's default memory pool: its high watermark of memory in use does not
move during a call (and does move during an allocating ctr_fp_par_2d_f32 call,
which shows the probe sees the library's allocations).  The file sorts last
so it also runs after every other GPU test in one process.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

import golden_cases as gc
from gpu_helpers import TOL_F32, cuda, fp_op, host, rel_l2

pytestmark = pytest.mark.gpu

# noalloc vs the allocating entry point: the same kernels on the same inputs
TOL_SAME = 1e-6


def _run(name, op, img):
    import torch
    from ct_recon_extensions_gb300._lib import call
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    b = img.shape[0]
    proj = torch.full((b, op.na, op.ns), float("nan"), dtype=torch.float32, device=img.device)
    call(name, ctypes.byref(op.p), _ptr(img), _ptr(proj), *map(_ptr, op.tables(img.device)), b,
         _stream())
    return proj


def _check_pair(op, img):
    a = host(_run("ctr_fp_par_2d_f32_noalloc", op, img))
    b = host(_run("ctr_fp_par_2d_f32", op, img))
    assert np.all(np.isfinite(a))
    assert rel_l2(a, b) <= TOL_SAME
    return a


def test_noalloc_matches_allocating_twice():
    from ct_recon_extensions_gb300 import synthetic as syn
    d = syn.parallel_config_2()
    op = fp_op(d)
    rng = np.random.default_rng(7)
    for batch in (3, 2):  # two calls in a row, the second on a smaller batch
        img = cuda(rng.standard_normal((batch, d["ny"], d["nx"])).astype(np.float32))
        _check_pair(op, img)


@pytest.mark.parametrize("name", gc.names("fp"))
def test_noalloc_golden(name):
    c = gc.load(name)
    op = fp_op(c["geom"])
    img = cuda(c["img_f32"][None])
    for _ in range(2):
        a = _check_pair(op, img)
        assert rel_l2(a[0], c["fp_f32"]) <= TOL_F32


def test_noalloc_rejects_oversize():
    import torch
    from ct_recon_extensions_gb300._lib import CtrError
    from ct_recon_extensions_gb300 import synthetic as syn
    d = dict(syn.parallel_config_2())
    d["na"] = 1000  # 1000 x 729 rays exceed the fixed scratch
    op = fp_op(d)
    img = torch.zeros((1, d["ny"], d["nx"]), dtype=torch.float32, device="cuda")
    with pytest.raises(CtrError, match="16 MiB"):
        _run("ctr_fp_par_2d_f32_noalloc", op, img)


def _cudart():
    """The CUDA runtime as a shared library, only to read the device's default
    memory pool (a driver object that the library's own, statically linked,
    runtime allocates from too)."""
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so",
                 ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            return ctypes.CDLL(name)
        except OSError:
            pass
    pytest.skip("no libcudart to read the default memory pool")


def test_noalloc_allocates_nothing():
    import torch
    from ct_recon_extensions_gb300._lib import call
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.torch_ctrecon import _ptr, _stream
    used_now, used_high = 7, 8  # cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrUsedMemHigh
    rt = _cudart()
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), torch.cuda.current_device()) == 0
    d = syn.parallel_config_2()
    op = fp_op(d)
    img = cuda(np.random.default_rng(3).standard_normal((1, d["ny"], d["nx"])).astype(np.float32))
    proj = torch.empty((1, d["na"], d["ns"]), dtype=torch.float32, device="cuda")
    tables = [_ptr(t) for t in op.tables(img.device)]

    def peak_growth(name):
        torch.cuda.synchronize()
        zero, now, high = ctypes.c_uint64(0), ctypes.c_uint64(), ctypes.c_uint64()
        assert rt.cudaMemPoolSetAttribute(pool, used_high, ctypes.byref(zero)) == 0
        assert rt.cudaMemPoolGetAttribute(pool, used_now, ctypes.byref(now)) == 0
        call(name, ctypes.byref(op.p), _ptr(img), _ptr(proj), *tables, 1, _stream())
        torch.cuda.synchronize()
        assert rt.cudaMemPoolGetAttribute(pool, used_high, ctypes.byref(high)) == 0
        return high.value - now.value

    for _ in range(2):
        assert peak_growth("ctr_fp_par_2d_f32_noalloc") == 0
    # the allocating entry point's stream-ordered scratch shows up in the same probe
    assert peak_growth("ctr_fp_par_2d_f32") > 0
