"""The stream-K partition of the small-launch backprojector (csrc/sk_split.h),
built for the host: unit ranges cover every (tile, view block) unit once,
the owner lookup agrees with the ranges, and segment indices fit the
partial-sum buffer that the host sizes."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_partition(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "sk_split_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "cpp", "sk_split_check.cc")],
                   check=True)
    cases, bad = map(int, subprocess.run([exe], capture_output=True, check=True).stdout.split())
    assert cases > 400 and bad == 0
