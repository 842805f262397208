"""The C++ operator mirror (include/ct_recon/*.h) as a reference C++ user would
use it: tests/cpp/mirror_fbp.cc is compiled with g++ against the headers and
libctrecon_gb300.so, runs the fan FBP chain and the BP adjoint on the golden
case's inputs, and must reproduce the reference's outputs."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_cases as gc
from gpu_helpers import rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    return None


def test_header_only_mirror_compiles(tmp_path):
    cuda = _cuda_home()
    if not cuda or not shutil.which("g++"):
        pytest.skip("g++ or CUDA headers missing")
    src = tmp_path / "all.cc"
    src.write_text("".join(f'#include "ct_recon/{h}"\n' for h in sorted(os.listdir(os.path.join(ROOT, "include", "ct_recon"))))
                   + "int main() { return 0; }\n")
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(cuda, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_mirror_fbp_matches_reference(tmp_path):
    from ct_recon_extensions_gb300 import build
    lib = build.build()
    cuda = _cuda_home()
    assert cuda, "CUDA toolkit not found"
    exe = tmp_path / "mirror_fbp"
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "mirror_fbp.cc"),
           "-o", str(exe), lib, f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"),
           "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    c = gc.load("fan_full")
    g = c["geom"]
    c["sino_f32"].tofile(tmp_path / "sino.f32")
    c["img_in_f32"].tofile(tmp_path / "img_in.f32")
    args = [str(exe), str(tmp_path)] + [repr(g[k]) for k in (
        "ns", "na", "ds", "orbit", "offset_s", "orbit_start", "nx", "ny", "dx", "dy", "offset_x",
        "offset_y", "dso", "dsd")]
    env = dict(os.environ, LD_LIBRARY_PATH=os.path.join(cuda, "lib64") + ":" + os.environ.get("LD_LIBRARY_PATH", ""))
    r = subprocess.run(args, capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    recon = np.fromfile(tmp_path / "recon.f32", np.float32).reshape(g["ny"], g["nx"])
    grad = np.fromfile(tmp_path / "grad.f32", np.float32).reshape(g["na"], g["ns"])
    assert rel_l2(recon, c["bp_f32"]) <= 1e-5
    assert rel_l2(grad, c["bp_grad_f32"]) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["heli_p1", "heli_norows", "heli_views"])
def test_mirror_helical_matches_reference(tmp_path, name):
    """HelicalInterpolation360/180<double> through the C++ mirror: the reference's
    outputs (FP64, bit-exact up to the hosts' libm cos) and its exceptions."""
    from ct_recon_extensions_gb300 import build
    lib = build.build()
    cuda = _cuda_home()
    assert cuda, "CUDA toolkit not found"
    exe = tmp_path / "mirror_helical"
    r = subprocess.run(["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "mirror_helical.cc"),
                        "-o", str(exe), lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-L",
                        os.path.join(cuda, "lib64"), "-lcudart"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    c = gc.load(name)
    h = c["heli"]
    c["in_f64"].tofile(tmp_path / "in.f64")
    env = dict(os.environ, LD_LIBRARY_PATH=os.path.join(cuda, "lib64") + ":" + os.environ.get("LD_LIBRARY_PATH", ""))
    keys = ("ns", "nt", "na", "ds", "dt", "offset_s", "offset_t", "orbit_start", "orbit", "couch_begin",
            "couch_mov", "view_per_rot", "nz", "dz", "z0", "thickness", "dso", "dsd")
    for method in ("360", "180"):
        r = subprocess.run([str(exe), str(tmp_path), method] + [repr(h[k]) for k in keys],
                           capture_output=True, text=True, env=env)
        want = int(c[f"status{method}"])
        if want == 1:
            assert r.returncode == 0, r.stdout + r.stderr
            got = np.fromfile(tmp_path / f"out{method}.f64").reshape(h["nz"], h["view_per_rot"], h["ns"])
            ref = c[f"out{method}_f64"]
            assert np.allclose(got, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
        else:
            msg = "View not enough for this slice!" if want == -1 else "No row data available!"
            assert r.returncode == 2 and msg in r.stdout, r.stdout + r.stderr
