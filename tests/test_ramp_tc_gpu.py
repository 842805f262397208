"""The ramp filter on the BF16 tensor cores (ctr_ramp_filter_tc_*).

Two checks per case, both against the oracle:
  * the GEMM itself: the device output equals the sum of the term products
    (hi/lo: X0 T0 + X0 T1 + X1 T0; hi/mid/lo adds X0 T2 + X2 T0 + X1 T1)
    computed in FP64 from the same BF16 terms (the split is
    round-to-nearest-even, restated here in numpy), to FP32 accumulation
    error; this pins the tile layout, the descriptors and the epilogue;
  * the filter: against the FP64 ramp filter of the oracle (src/filter.cc:67-124)
    on the same stored input, to the split's error budget.
Inputs are stored as FP32, BF16 and FP16; fan weighting is fused in front.
A smooth fan sinogram checks the 3-term split where the filter cancels most
of its input.
"""
import numpy as np
import pytest

from gpu_helpers import cuda, host, rel_l2

pytestmark = pytest.mark.gpu

# device vs FP64 products of the same splits: the tensor core's FP32
# accumulation over up to 3 x 1536 products (2.6e-6 measured at ns=1472); a
# tile-layout or descriptor error shows as O(1)
TOL_GEMM = 6e-6
# device vs the FP64 filter on random inputs: hi/lo keeps ~16 bits of each
# operand, hi/mid/lo ~24
TOL_FILTER = {2: 3e-5, 3: 1e-5}
# a smooth sinogram (the filter cancels ~100x, which scales the FP32
# accumulation error of the GEMM check the same way): hi/mid/lo only
TOL_SMOOTH = 2e-5

DSO, DSD = 595.0, 1085.6


def bf16_rn(a):
    """Round FP64 values to BF16 (8 significant bits), ties to even."""
    a = np.asarray(a, np.float64)
    m, e = np.frexp(a)
    return np.ldexp(np.rint(m * 256.0) / 256.0, e)


def split(a, n=2):
    out, r = [], np.asarray(a, np.float64)
    for _ in range(n):
        t = bf16_rn(r)
        out.append(t)
        r = r - t
    return out


def products(xs, ts):
    """Sum of the term products the device forms (X_a T_b^T)."""
    pairs = [(0, 0), (0, 1), (1, 0)] + ([(0, 2), (2, 0), (1, 1)] if len(xs) == 3 else [])
    return sum(xs[a] @ ts[b].T for a, b in pairs)


def fan_weights(ns, ds, offset=0.0, wtype=1):
    cents = (ns - 1) / 2 + offset
    s = ds * (np.arange(ns) - cents)
    g = np.arctan2(s, DSD) if wtype == 2 else s / DSD
    return DSO * np.abs(np.cos(g)) / DSD


def toeplitz(taps, ns, ds, grad):
    i = np.arange(ns)
    d = (i[None, :] - i[:, None]) if grad else (i[:, None] - i[None, :])
    return ds * taps[ns + d]


def _case(ns, nrow, batch, ds, ftype, dtype, weighted, grad, seed, splits=3, x=None, tol_gemm=TOL_GEMM):
    import torch
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    from oracle import Oracle
    orc = Oracle("port", threads=8)
    if x is None:
        x = np.random.default_rng(seed).standard_normal((batch, nrow, ns)).astype(np.float32)
    tdt = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[dtype]
    xt = torch.from_numpy(x).to(tdt)
    stored = xt.to(torch.float32).numpy()  # the values the device reads
    dsd = DSD if ftype else -1.0
    w_op = tc.FanWeightingOp(ns, nrow, ds, 0.0, DSO, DSD, 1) if weighted else None
    op = tc.RampFilterTCOp(ns, nrow, ds, dsd, ftype, weighting=w_op, splits=splits)
    y = host(op.adjoint(xt.cuda()) if grad else op.forward(xt.cuda()))
    assert y.dtype == np.float32 and y.shape == (batch, nrow, ns)

    taps = orc.ramp_taps(ns, ds, dsd, ftype)
    w64 = fan_weights(ns, ds) if weighted else np.ones(ns)
    # GEMM: the device weights in FP32 with an FP32 weight, then splits
    xw = (stored * w64.astype(np.float32)[None, None, :]).astype(np.float32) if weighted else stored
    xs = split(xw.astype(np.float64).reshape(-1, ns), splits)
    ts = split(toeplitz(taps, ns, ds, grad), splits)
    ref = products(xs, ts).reshape(batch, nrow, ns)
    assert rel_l2(y, ref) <= tol_gemm
    # filter: FP64 weighting and FP64 filter of the stored input
    xin = stored.astype(np.float64) * w64[None, None, :]
    ora = np.stack([orc.ramp_filter(xin[b], ds, dsd, ftype, grad=grad, taps=taps) for b in range(batch)])
    return rel_l2(y, ora)


@pytest.mark.parametrize("splits", [2, 3])
@pytest.mark.parametrize("dtype", ["f32", "bf16", "f16"])
def test_small_padded(dtype, splits):
    # ns=100: one partial 128-wide tile in N and two K blocks (the second partial)
    assert _case(100, 50, 1, 1.0, 0, dtype, False, False, 1, splits) <= TOL_FILTER[splits]


@pytest.mark.parametrize("splits", [2, 3])
@pytest.mark.parametrize("ftype,weighted", [(0, False), (1, True), (2, True)])
def test_config1_sizes(ftype, weighted, splits):
    # 720 views x 736 channels (the fan drop-in), one sinogram
    assert _case(736, 720, 1, 1.2858, ftype, "f32", weighted, False, 2, splits) <= TOL_FILTER[splits]


@pytest.mark.parametrize("splits", [2, 3])
@pytest.mark.parametrize("dtype", ["bf16", "f16"])
def test_large_slice_rows_batched(dtype, splits):
    # 1472 channels at 0.6429 mm (the large fan slice), 3 sinograms of 96 rows:
    # rows of one 128-row tile span two sinograms
    assert _case(1472, 96, 3, 0.6429, 1, dtype, True, False, 3, splits) <= TOL_FILTER[splits]


@pytest.mark.parametrize("splits", [2, 3])
@pytest.mark.parametrize("ftype", [0, 1])
def test_grad(ftype, splits):
    # RampFilterGrad: the correlation (T transposed)
    assert _case(729, 40, 2, 0.5, ftype, "f32", False, True, 4, splits) <= TOL_FILTER[splits]


@pytest.mark.parametrize("dtype", ["f32", "bf16", "f16"])
def test_smooth_sinogram_three_terms(dtype):
    # analytic fan sinogram of the large slice (first 128 views): the ramp
    # filter cancels most of the weighted input, so the 3-term split is needed
    from ct_recon_extensions_gb300 import synthetic as syn
    g = syn.large_config_5()
    x = syn.fan_sinogram(syn.random_ellipses(5000), 128, g["ns"], g["ds"], g["orbit"], g["dso"], g["dsd"])
    err = _case(g["ns"], 128, 1, g["ds"], 1, dtype, True, False, 0, 3, x=x[None].astype(np.float32),
                tol_gemm=TOL_SMOOTH)
    assert err <= TOL_SMOOTH, err


def test_plan_grows_and_rejects():
    import torch
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    from ct_recon_extensions_gb300._lib import CtrError, call
    op = tc.RampFilterTCOp(64, 8, 1.0)
    x = torch.randn(1, 8, 64, device="cuda")
    a = op.forward(x)
    b = op.forward(torch.cat([x, x, x]))  # batch 3 re-plans
    assert torch.allclose(a[0], b[2])
    h = op.plan(x.device, False, 3)
    with pytest.raises(CtrError, match="batch"):
        call("ctr_ramp_filter_tc_run", h, 0, tc._ptr(x), tc._ptr(a), 4, tc._stream())
    with pytest.raises(CtrError, match="dtype"):
        call("ctr_ramp_filter_tc_run", h, 7, tc._ptr(x), tc._ptr(a), 1, tc._stream())
    with pytest.raises(TypeError):
        op.forward(x.double())


def test_no_wait_timeouts():
    from ct_recon_extensions_gb300 import torch_ctrecon  # noqa: F401
    import ctypes
    from ct_recon_extensions_gb300._lib import call
    flags = ctypes.c_uint()
    call("ctr_kernel_flags", ctypes.byref(flags), 1)
    assert flags.value & 4 == 0
