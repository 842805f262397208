"""C-ABI checks that need no GPU: the library loads, exports every entry
point declared in include/ctrecon_gb300.h, and rejects invalid arguments on
the host before touching CUDA."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from ct_recon_extensions_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(ctr_\w+)\s*\(", text, flags=re.M)
            names += re.findall(r"^\s*(?:bool|int)\s+(\w+_(?:create|run|destroy)|set_device|clear)\s*\(",
                                text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "ctr_bp_fan_2d_f32" in names and "ctr_fp_par_2d_grad_f64" in names
    assert len(names) >= 35


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_prototypes_cover_header():
    from ct_recon_extensions_gb300 import _lib
    declared = {n for n in declared_symbols() if n.startswith("ctr_")}
    assert declared <= set(_lib.exported_names()), declared - set(_lib.exported_names())


def test_status_strings(lib):
    assert lib.ctr_status_string(0) == b"ok"
    assert lib.ctr_status_string(1) == b"invalid argument"
    assert lib.ctr_version() >= 10000


def test_host_validation_without_gpu(lib):
    from ct_recon_extensions_gb300 import _lib as L
    # null parameter / null buffers are rejected before any CUDA call
    assert lib.ctr_fan_weighting_f32(None, None, None, 1, None) == 1
    assert lib.ctr_selftest_wait_timeout(0, None) == 1
    assert lib.ctr_fp_par_2d_plan_run(None, None, None, 1, None) == 1
    plan = ctypes.c_void_p(1)
    assert lib.ctr_fp_par_2d_plan_create(None, None, None, None, 1, ctypes.byref(plan), None) == 1
    assert plan.value is None
    p = L.FanWeightingParam(8, 4, 1.0, 0.0, 500.0, 1000.0, 3)
    dummy = ctypes.c_void_p(16)
    assert lib.ctr_fan_weighting_f32(ctypes.byref(p), dummy, dummy, 1, None) == 1  # bad type
    assert b"type" in lib.ctr_last_error()
    p.type = 1
    assert lib.ctr_fan_weighting_f32(ctypes.byref(p), dummy, dummy, 0, None) == 1  # batch 0
    f = L.FilterParam(8, 4, 1.0, -1.0, 0, 0)
    assert lib.ctr_ramp_filter_f32(ctypes.byref(f), dummy, dummy, dummy, 1, None) == 1  # in place
    q = L.ParParam(8, 4, 1.0, 0.1, 0.0, 0.0, 4, 6, 1.0, 1.0, 0.0, 0.0, -1.0)
    assert lib.ctr_fp_par_2d_f32(ctypes.byref(q), dummy, dummy, dummy, dummy, dummy, 1, None) == 1
    assert b"nx == ny" in lib.ctr_last_error()
    fb = L.FanBpParam(0, 4, 1.0, 0.1, 0, 0, 4, 4, 1, 1, 0, 0, 500, 1000, -1)
    assert lib.ctr_bp_fan_2d_f32(ctypes.byref(fb), dummy, dummy, dummy, dummy, dummy, 1, None) == 1


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from ct_recon_extensions_gb300 import _lib as L
    monkeypatch.setattr(L, "_lib", None)
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(L.CtrLibraryError):
        L.load()


def test_helical_host_checks_without_gpu(lib):
    """Helical prep and run: table size and argument checks resolve on the host
    before any CUDA call."""
    from ct_recon_extensions_gb300 import _lib as L
    p = L.HelicalParam(32, 6, 120, 1.0, 1.0, 0.0, 0.0, 0.0, 2 * 3.141592653589793 / 40, 0.0,
                       6 * 0.5 / 40, 40, 3, 0.5, 1.0, 0.5, 500.0, 1000.0)
    # header, FP64 channel and slice sections, FP32 channel section, one row per (slice, view)
    assert lib.ctr_helical_interpolation_table_bytes(ctypes.byref(p)) == \
        16 + 32 * 32 + 32 * 3 + 40 * 32 + 80 * 3 * 40
    assert lib.ctr_helical_interpolation_table_bytes(None) == 0
    assert lib.ctr_helical_interpolation_prep(None, 0, None, None) == 1
    assert lib.ctr_helical_interpolation_prep(ctypes.byref(p), 7, ctypes.c_void_p(16), None) == 1
    assert lib.ctr_helical_interpolation_prep(ctypes.byref(p), 0, None, None) == 1
    bad = L.HelicalParam(32, 6, 120, 1.0, 1.0, 0.0, 0.0, 0.0, 0.1, 0.0, 0.0, 40, 3, 0.5, 1.0,
                         0.5, 500.0, 1000.0)  # couch_mov == 0
    assert lib.ctr_helical_interpolation_prep(ctypes.byref(bad), 0, ctypes.c_void_p(16), None) == 1
    assert lib.ctr_helical_interpolation_360_f32(ctypes.byref(p), None, None, None, None, 1, None) == 1
