"""The FP32 forward projector's per-ray set-up (csrc/fp_setup.cuh), built for
the host and checked ray by ray against the reference's FP64 inclusion rule
(x accumulated sample by sample, src/fp_par_2d.cc:236-249) on the prep tables
of the oracle: same valid samples for every ray, and fixed-point positions
that index inside the staged row."""
import math
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from oracle import Geom, Oracle

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpp", "fp_setup_check.cc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("fpsc") / "fp_setup_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, SRC], check=True)
    return exe


def _tables(g):
    _, bo, _ = Oracle("port").fp_par_2d_tables(g)
    return struct.pack("ii", g.nx, g.na * g.ns) + np.ascontiguousarray(bo.reshape(-1, 2)).tobytes()


def _run(exe, g):
    out = subprocess.run([exe], input=_tables(g), capture_output=True, check=True).stdout.split()
    rays, fixed, split, fallback, mis_fma, mis_acc, bad = map(int, out)
    return rays, fixed, split, fallback, mis_acc, bad


def test_config2_geometry(checker):
    # 512^2 image, 720 views over pi, 729 bins at 0.5 mm (the parallel drop-in)
    g = Geom.make(729, 720, 0.5, math.pi / 720, 512, 512, 0.5, 0.5)
    rays, fixed, split, fallback, mis_acc, bad = _run(checker, g)
    assert mis_acc == 0 and bad == 0
    assert split + fallback <= 16  # ties at the image border only
    assert fallback == 0           # every tie is deferred, none takes the slow path


def test_random_geometries(checker):
    rng = np.random.default_rng(1)
    tot = np.zeros(6, np.int64)
    for _ in range(40):
        n = int(rng.choice([8, 31, 64, 100, 128, 257]))
        na, ns = int(rng.integers(4, 90)), int(rng.integers(4, 200))
        dx = float(rng.choice([0.5, 1.0, 0.8]))
        dy = dx if rng.random() < 0.7 else float(rng.choice([0.5, 1.0, 0.8]))
        orbit = float(rng.choice([math.pi / na, 2 * math.pi / na, -math.pi / na, math.pi / 4,
                                  math.pi / 2]))
        g = Geom.make(ns, na, float(rng.choice([0.5, 1.0, 0.37, 2.0])), orbit, n, n, dx, dy,
                      offset_s=float(rng.choice([0, 0.25, -1.5])),
                      orbit_start=float(rng.choice([0, math.pi / 4, 0.1])),
                      offset_x=float(rng.choice([0, 0.5, 3.0])),
                      offset_y=float(rng.choice([0, -0.5])))
        tot += _run(checker, g)
    rays, fixed, split, fallback, mis_acc, bad = tot
    assert mis_acc == 0 and bad == 0
    assert split + fallback < rays // 100


def test_dbl2flt(checker):
    # the integer double -> float conversion used on the device
    out = subprocess.run([checker, "conv"], capture_output=True, check=True).stdout
    assert int(out) == 0


@pytest.mark.parametrize("n", [64, 512])
def test_column_band_ranges(checker, n):
    # the samples of a column-marching ray that fall in each band of rows
    g = Geom.make(729 if n == 512 else 91, 720 if n == 512 else 60, 0.5 * 512 / n, math.pi / (720 if n == 512 else 60),
                  n, n, 0.5 * 512 / n, 0.5 * 512 / n)
    out = subprocess.run([checker, "col"], input=_tables(g), capture_output=True, check=True).stdout
    assert int(out) == 0


def test_accumulation_walk(checker):
    # the binade-jump walk reproduces the reference's x += step bit for bit
    cases, bad = map(int, subprocess.run([checker, "acc"], capture_output=True, check=True).stdout.split())
    assert cases > 100000 and bad == 0
