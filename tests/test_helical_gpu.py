"""Helical rebinning on the GPU (ctr_helical_interpolation_*) against the
reference's fixtures and the oracle port.

T=double runs the reference's FP64 arithmetic in its order, so against the
oracle port run on the same host (same libm cos for the channel table) it is
compared for exact equality, and against the fixtures (made on another host,
whose cos may differ in a last bit) to 1e-13 relative.

T=float runs the FP32 fast path: the reference's decisions (rows, usability,
views) with FP32 sums.  It is held to 2e-6 of the output's peak magnitude
(max abs error): a wrong row or view decision would move a value by O(0.1)."""
import numpy as np
import pytest

import golden_cases as gc
from gpu_helpers import cuda, host

pytestmark = pytest.mark.gpu

F32_TOL = 2e-6


def _close(got, want, dt):
    if np.dtype(dt) == np.float64:
        return np.array_equal(got, want)
    want = np.asarray(want, np.float64)
    return float(np.abs(np.asarray(got, np.float64) - want).max()) <= F32_TOL * float(np.abs(want).max())


SFX = [("f32", np.float32), ("f64", np.float64)]


def _op(h, method):
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    return tc.HelicalInterpolationOp(h.ns, h.nt, h.na, h.ds, h.dt, h.offset_s, h.offset_t,
                                     h.orbit_start, h.orbit, h.couch_begin, h.couch_mov,
                                     h.view_per_rot, h.nz, h.dz, h.z0, h.thickness, h.dso, h.dsd,
                                     method)


@pytest.mark.parametrize("name", gc.names("heli"))
@pytest.mark.parametrize("sfx,dt", SFX)
@pytest.mark.parametrize("method", ["360", "180"])
def test_helical_golden(port, name, sfx, dt, method):
    c = gc.load(name)
    h = gc.heli(c)
    x = c["in_f64"].astype(dt)
    want = int(c[f"status{method}"])
    if want == -1:
        with pytest.raises(RuntimeError, match="View not enough for this slice!"):
            _op(h, method).forward(cuda(x))
        return
    if want == -2:
        with pytest.raises(RuntimeError, match="No row data available!"):
            _op(h, method).forward(cuda(x))
        return
    got = host(_op(h, method).forward(cuda(x)))
    ref = c[f"out{method}_{sfx}"]
    if dt == np.float64:
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    else:
        assert _close(got, ref, dt)
    exact, _ = port.helical(x, h, method)
    assert _close(got, exact, dt)


@pytest.mark.parametrize("method", ["360", "180"])
def test_helical_clinical_size_exact(port, method):
    """736 channels x 32 rows, 720 views per rotation, pitch 0.9, offsets,
    12 slices over a rotation of couch travel: T=double equals the oracle port
    bit for bit, T=float within F32_TOL."""
    from oracle import Heli
    ns, nt, vpr, dso, dsd = 736, 32, 720, 595.0, 1085.6
    rot = 0.9 * nt * dso / dsd
    na = 3 * vpr  # slice 0 sits near view 730; the last slice needs views up to ~2110
    h = Heli.make(ns=ns, nt=nt, na=na, ds=1.2858, dt=1.0, view_per_rot=vpr, couch_mov=rot / vpr,
                  nz=12, dz=rot / 12, z0=-0.6 + 730.3 * rot / vpr, thickness=1.25, dso=dso,
                  dsd=dsd, offset_s=1.125, offset_t=-0.25, couch_begin=-0.6)
    rng = np.random.default_rng(5)
    x = (1 + 0.1 * rng.standard_normal((na, nt, ns))).astype(np.float32)
    for dt in (np.float32, np.float64):
        xd = x.astype(dt)
        got = host(_op(h, method).forward(cuda(xd)))
        exact, outside = port.helical(xd, h, method)
        assert not outside
        assert _close(got, exact, dt)


def test_helical_batch_is_items():
    c = gc.load("heli_p1")
    h = gc.heli(c)
    rng = np.random.default_rng(1)
    xs = np.stack([c["in_f64"], c["in_f64"] * 0.5 + 1, rng.standard_normal(c["in_f64"].shape)])
    for method in ("360", "180"):
        op = _op(h, method)
        both = host(op.forward(cuda(xs)))
        for i in range(3):
            assert np.array_equal(both[i], host(op.forward(cuda(xs[i]))))


def test_helical_first_view_zero_reads_zero(port):
    """A 180LI slice whose first view is 0: complementary samples before it read
    as 0 with a warning, equal to the port's defined behaviour (the reference
    reads out of bounds there)."""
    from oracle import Heli
    h = Heli.make(ns=32, nt=6, na=80, ds=1.0, dt=1.0, view_per_rot=40, couch_mov=3 * 0.5 / 40,
                  nz=1, dz=0.5, z0=20 * 3 * 0.5 / 40, thickness=0.5, dso=500.0, dsd=1000.0)
    x = np.random.default_rng(2).random((h.na, h.nt, h.ns))
    with pytest.warns(UserWarning, match="read as 0"):
        got = host(_op(h, "180").forward(cuda(x)))
    exact, outside = port.helical(x, h, "180")
    assert outside and np.array_equal(got, exact)


def test_helical_table_of_other_method_writes_nothing():
    """A table prepared for 360LI handed to the 180LI kernel: the kernel reports
    CTR_HELICAL_BAD_TABLE and leaves the output untouched."""
    import torch
    from ct_recon_extensions_gb300 import _lib
    c = gc.load("heli_p1")
    h = gc.heli(c)
    op360, op180 = _op(h, "360"), _op(h, "180")
    x = cuda(c["in_f64"][None])
    out = torch.full((1, h.nz, h.view_per_rot, h.ns), 7.0, dtype=torch.float64, device="cuda")
    status = torch.zeros(h.nz, dtype=torch.int32, device="cuda")
    op360.table(x.device)
    op180._tables = op360._tables  # the wrong method's table
    op180.launch(x, out, status)
    assert status.cpu().tolist() == [_lib.CTR_HELICAL_BAD_TABLE] + [0] * (h.nz - 1)
    assert bool((out == 7.0).all())


@pytest.mark.parametrize("method", ["360", "180"])
def test_helical_f32_edges_on_integers(port, method):
    """Slab edges exactly on detector-row boundaries (dsd/dso = 2, couch steps
    and slice positions in quarter millimetres, half-millimetre slices, an
    integer centre channel): the FP32 path's guard sends those samples to the
    exact computation, and channels near the centre land within the guard."""
    from oracle import Heli
    h = Heli.make(ns=65, nt=16, na=400, ds=0.5, dt=1.0, view_per_rot=64, couch_mov=0.0625,
                  nz=8, dz=0.25, z0=64 * 1.5 * 0.0625, thickness=0.5, dso=500.0, dsd=1000.0,
                  offset_t=0.5)
    x = np.random.default_rng(8).random((h.na, h.nt, h.ns)).astype(np.float32)
    got = host(_op(h, method).forward(cuda(x)))
    exact, _ = port.helical(x, h, method)
    assert _close(got, exact, np.float32)
