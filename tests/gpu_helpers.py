"""Shared helpers of the GPU parity tests: operator objects built from a
golden case's geometry, and the error measures."""
import math

import numpy as np

from ct_recon_extensions_gb300 import torch_ctrecon as tc

# FP32 kernels vs the reference T=float output; FP64 kernels vs T=double.
TOL_F32 = 1e-5
TOL_F64 = 1e-11


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def tol(dtype):
    return TOL_F32 if np.dtype(dtype) == np.float32 else TOL_F64


def cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def fan_op(g):
    return tc.FanBackprojection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                    g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                    g["offset_x"], g["offset_y"], g["dso"], g["dsd"], g["fov"])


def angle_op(g, angles):
    return tc.FanBackprojection2DAngleOp(angles, g["ns"], g["ds"], g["offset_s"], g["nx"],
                                         g["ny"], g["dx"], g["dy"], g["offset_x"], g["offset_y"],
                                         g["dso"], g["dsd"], g["fov"])


def par_op(g):
    return tc.ParallelBackprojection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                         g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                         g["offset_x"], g["offset_y"], g["fov"])


def fp_op(g):
    return tc.ParallelProjection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                     g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                     g["offset_x"], g["offset_y"], g["fov"])


def weight_op(g, nrow, wt):
    return tc.FanWeightingOp(g["ns"], nrow, g["ds"], g["offset_s"], g["dso"], g["dsd"], wt)


def ramp_op(g, nrow, ftype, dsd=None):
    return tc.RampFilterOp(g["ns"], nrow, g["ds"], g["dsd"] if dsd is None else dsd, ftype)


def dot_rel(ax, y, x, aty):
    lhs = float(np.vdot(np.asarray(ax, np.float64), np.asarray(y, np.float64)))
    rhs = float(np.vdot(np.asarray(x, np.float64), np.asarray(aty, np.float64)))
    return abs(lhs - rhs) / abs(lhs)
