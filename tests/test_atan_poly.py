"""The FP32 atan2 of the shading (atan2_poly in bh_kernels.cu): its
coefficients are the ones atan_poly_fit.py fits, and an FP32 emulation of
the kernel's evaluation stays within 4e-7 rad of atan2 in every octant."""
import importlib.util
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "blackhole_8_gb300", "csrc")


def kernel_coeffs() -> np.ndarray:
    src = open(os.path.join(CSRC, "bh_kernels.cu")).read()
    body = src[src.index("__device__ __forceinline__ float atan2_poly"):]
    body = body[:body.index("\n}\n")]
    lits = re.findall(r"(-?\d\.\d+e-?\d+)f", body)
    # Horner order: c7 first, then c6 ... c0
    return np.array([float(v) for v in lits[:8]][::-1], dtype=np.float32)


def fitter():
    spec = importlib.util.spec_from_file_location("atan_poly_fit", os.path.join(CSRC, "atan_poly_fit.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def f32(v):
    return np.float32(v)


def fmaf(a, b, c):
    return (a.astype(np.float64) * b + c).astype(np.float32)


def atan2_poly(y, x, c):
    """The kernel's evaluation in FP32 (fmaf rounded once; the fast quotient
    as a correctly rounded one)."""
    y = y.astype(np.float32)
    x = x.astype(np.float32)
    ax, ay = np.abs(x), np.abs(y)
    mx, mn = np.maximum(ax, ay), np.minimum(ax, ay)
    with np.errstate(invalid="ignore", divide="ignore"):
        t = np.where(mx > 0, mn / np.where(mx > 0, mx, 1), 0).astype(np.float32)
    z = (t * t).astype(np.float32)
    p = np.full_like(z, c[7])
    for k in range(6, -1, -1):
        p = fmaf(p, z, np.float32(c[k]))
    r = (p * t).astype(np.float32)
    r = np.where(ay > ax, (f32(1.57079633) - r).astype(np.float32), r)
    r = np.where(x < 0, (f32(3.14159265) - r).astype(np.float32), r)
    return np.copysign(r, y)


def test_coefficients_are_the_fit():
    c, err = fitter().fit()
    assert err < 4e-8
    k = kernel_coeffs()
    c32 = c.astype(np.float32)
    assert np.all(np.abs(k - c32) <= np.spacing(np.abs(c32)))  # within 1 ulp of the fit


def test_fp32_evaluation_within_4e7():
    c = kernel_coeffs()
    rng = np.random.default_rng(1)
    ang = rng.uniform(-np.pi, np.pi, 400000)
    rad = np.exp(rng.uniform(-20, 20, ang.size))
    y, x = (rad * np.sin(ang)).astype(np.float32), (rad * np.cos(ang)).astype(np.float32)
    got = atan2_poly(y, x, c).astype(np.float64)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.abs(got - want).max() < 4e-7
    # axes, diagonals and zeros
    sy = np.array([0, 0, 1, -1, 1, 1, -1, -1, 0, -0.0], dtype=np.float32)
    sx = np.array([1, -1, 0, 0, 1, -1, 1, -1, 0, -1], dtype=np.float32)
    got = atan2_poly(sy, sx, c).astype(np.float64)
    want = np.arctan2(sy.astype(np.float64), sx.astype(np.float64))
    assert np.abs(got - want).max() < 4e-7
    assert got[8] == 0.0
