"""Exact transposition, entry by entry: on the small golden geometries the
FP32 forward of every unit input (one batch) and the FP32 adjoint of every
unit output (one batch) give the operator matrix twice; the two must agree
everywhere up to FP32 weight rounding.  A tie decided differently by the two
kernels would show as an entry of weight ~1 on one side only."""
import numpy as np
import pytest

import golden_cases as gc
from gpu_helpers import fan_op, fp_op, par_op

pytestmark = pytest.mark.gpu

# largest |A - (A^T)^T| entry relative to the largest entry of A
TOL_ENTRY = 1e-5
# the FP32 backprojector adjoints sum in fixed point: a quantum of 2^-19 of the
# tile's largest value (measured 1e-6 parallel, 2.8e-6 fan)
TOL_ENTRY_BP = 5e-6


def _matrices(op, in_shape, out_shape):
    import torch
    P, Q = int(np.prod(in_shape)), int(np.prod(out_shape))
    eye_in = torch.eye(P, dtype=torch.float32, device="cuda").reshape(P, *in_shape)
    fwd = op.forward(eye_in).reshape(P, Q)           # row p = A[:, p]
    del eye_in
    eye_out = torch.eye(Q, dtype=torch.float32, device="cuda").reshape(Q, *out_shape)
    adj = op.adjoint(eye_out).reshape(Q, P)          # row q = A^T[:, q]
    return fwd.cpu().numpy().astype(np.float64), adj.cpu().numpy().astype(np.float64).T


def _check(fwd, adjT, tol=TOL_ENTRY):
    scale = np.abs(fwd).max()
    assert scale > 0
    err = np.abs(fwd - adjT).max() / scale
    assert err <= tol, err


@pytest.mark.parametrize("name", ["fp_half", "fp_full_wrap"])
def test_fp_par_2d_transpose(name):
    g = gc.load(name)["geom"]
    _check(*_matrices(fp_op(g), (g["ny"], g["nx"]), (g["na"], g["ns"])))


def test_bp_par_2d_transpose():
    g = gc.load("par_rect_cw")["geom"]
    _check(*_matrices(par_op(g), (g["na"], g["ns"]), (g["ny"], g["nx"])), TOL_ENTRY_BP)


@pytest.mark.parametrize("name", ["fan_full", "fan_short_cw"])
def test_bp_fan_2d_transpose(name):
    g = gc.load(name)["geom"]
    _check(*_matrices(fan_op(g), (g["na"], g["ns"]), (g["ny"], g["nx"])), TOL_ENTRY_BP)
