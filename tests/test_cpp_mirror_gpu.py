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
