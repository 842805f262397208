"""The expiry path of the kernels' bounded waits, made to run out on purpose:
a self-test kernel arms an mbarrier for a copy that is never issued (as a
producer that skipped its stage would) and waits on it with the library's own
bounded wait under a 50 us limit.  The wait gives up, the kernel sets the
timeout flag and returns, the C ABI call returns CTR_ERR_KERNEL, and the
context keeps working.  No trap, no fault, no kernel left waiting."""
import ctypes

import pytest

import golden_cases as gc
from gpu_helpers import TOL_F32, cuda, host, par_op, rel_l2

pytestmark = pytest.mark.gpu

CTR_ERR_KERNEL = 5
FLAG_WAIT_TIMEOUT = 1 << 2


def test_bounded_wait_expires_and_reports():
    import torch
    from ct_recon_extensions_gb300 import _lib
    lib = _lib.load()
    flags = ctypes.c_uint(0)
    assert lib.ctr_kernel_flags(ctypes.byref(flags), 1) == 0  # start clean
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.ctr_selftest_wait_timeout(50_000, stream)
    assert st == CTR_ERR_KERNEL, st
    assert b"bounded wait gave up" in lib.ctr_last_error()
    assert lib.ctr_kernel_flags(ctypes.byref(flags), 1) == 0
    assert flags.value & FLAG_WAIT_TIMEOUT
    # the context is usable afterwards: a backprojection against the golden output
    c = gc.load("par")
    g = c["geom"]
    assert rel_l2(host(par_op(g).forward(cuda(c["filtered_f32"]))), c["bp_f32"]) <= TOL_F32
    assert lib.ctr_kernel_flags(ctypes.byref(flags), 1) == 0
    assert flags.value == 0
