"""Fits the polynomial of ``atan2_poly`` in bh_kernels.cu.

atan(t) ~ t * P(t^2) on [0, 1], P of degree 7 in t^2 (8 coefficients),
minimising the largest absolute error by the Remez exchange algorithm:
solve for the coefficients and the levelled error E on n + 1 reference
points, move the points to the extrema of the new error curve, repeat until
the extrema are level. Run as a script to print the coefficients as FP32
literals and the error in exact (float64) arithmetic.
"""
from __future__ import annotations

import numpy as np

N_COEFFS = 8


def _error(c: np.ndarray, t: np.ndarray) -> np.ndarray:
    return t * np.polyval(c[::-1], t * t) - np.arctan(t)


def _extrema(err: np.ndarray) -> list[int]:
    """Index of the largest |err| on each run of one sign."""
    out, start = [], 0
    sign = np.sign(err)
    for j in range(1, len(err)):
        if sign[j] != 0 and sign[j] != sign[start]:
            out.append(start + int(np.argmax(np.abs(err[start:j]))))
            start = j
    out.append(start + int(np.argmax(np.abs(err[start:]))))
    return out


def fit(n: int = N_COEFFS, grid: int = 400001, iters: int = 60) -> tuple[np.ndarray, float]:
    m = n + 1
    t = np.linspace(0.0, 1.0, grid)
    ref = 0.5 - 0.5 * np.cos(np.pi * np.arange(m) / (m - 1))
    c = np.zeros(n)
    for _ in range(iters):
        pts = np.maximum(ref, 1e-9)  # t = 0 is a root of every basis function
        A = np.empty((m, m))
        for i, x in enumerate(pts):
            A[i, :n] = x * (x * x) ** np.arange(n)
            A[i, n] = (-1.0) ** i
        c = np.linalg.solve(A, np.arctan(pts))[:n]
        err = _error(c, t)
        ext = _extrema(err)
        if len(ext) < m:
            break
        if len(ext) > m:  # keep the m largest, in order
            ext = sorted(sorted(ext, key=lambda k: -abs(err[k]))[:m])
        new_ref = t[ext]
        if np.allclose(new_ref, ref, atol=1e-12, rtol=0):
            break
        ref = new_ref
    return c, float(np.max(np.abs(_error(c, t))))


def main() -> None:
    c, e = fit()
    print(f"max |t P(t^2) - atan t| on [0, 1] = {e:.3e}")
    for k in reversed(range(len(c))):
        print(f"  c{k} = {np.float32(c[k])!r}")


if __name__ == "__main__":
    main()
