"""The parity bar of the GPU tests, on whole images and on pixel samples.

A GPU render agrees with the FP64 oracle when:
- its hit class agrees on >= 99.9 % of pixels, and every pixel whose class
  differs lies on a boundary: within one pixel of a pixel next to another
  class (a Manhattan distance of 2 from a pixel of another class), near a
  disc edge (hit radius within `edge` M of r_in or r_out), near the critical
  impact parameter (|b - 3 sqrt(3) M| < band M), or near a texel edge
  (sampling coordinate within `tex` texels of one);
- away from boundaries its colour is within 1 LSB, the deflection of escaped
  rays within `aux_tol` rad and the hit radius of disc rays within
  `radius_tol` M.

On a pixel sample the class boundary is found lazily: only pixels that fail a
check have the oracle evaluated on their neighbourhood (the 12 pixels within
Manhattan distance 2), which decides the same as evaluating it everywhere.
"""
from __future__ import annotations

import math

import numpy as np

import helpers
from blackhole_8_gb300 import capi
from oracle import oracle

B_C = 3.0 * math.sqrt(3.0)
MIN_CLASS_AGREEMENT = 0.999


def dilate(mask, n=1):
    m = mask.copy()
    for _ in range(n):
        m2 = m.copy()
        m2[1:, :] |= m[:-1, :]
        m2[:-1, :] |= m[1:, :]
        m2[:, 1:] |= m[:, :-1]
        m2[:, :-1] |= m[:, 1:]
        m = m2
    return m


def soft_boundary(o, band=1e-4, tex=0.02, edge=2e-3):
    """Pixels whose result may flip under rounding for a reason other than a
    neighbouring class: near a disc edge, near b_c or near a texel edge."""
    m = (o["cls"] == capi.CLASS_DISC) & (o["margin_r"] < edge)
    m |= np.abs(o["b_over_m"] - B_C) < band
    m |= o["margin_tex"] < tex
    return m


def boundary_pixels(o, band=1e-4, tex=0.02, edge=2e-3):
    """Whole-image boundary mask (class boundaries dilated by one pixel, and
    the soft boundaries)."""
    return dilate(helpers.class_boundary_mask(o["cls"])) | soft_boundary(o, band, tex, edge)


def compare(out, o, boundary, aux_tol, radius_tol=1e-3, colour_lsb=1):
    """Whole-image check of a GPU frame against the oracle; returns the
    largest deflection and hit-radius errors away from boundaries."""
    cls_ok = out.hit_class == o["cls"]
    assert cls_ok.mean() >= MIN_CLASS_AGREEMENT, f"class agreement {cls_ok.mean():.5f}"
    assert not (~cls_ok & ~boundary).any(), "class mismatch away from boundaries"
    strict = cls_ok & ~boundary
    dcol = helpers.colour_lsb(out.pixels, o["bgra"])
    assert dcol[strict].max(initial=0) <= colour_lsb
    esc = strict & (o["cls"] == capi.CLASS_MISS)
    dsk = strict & (o["cls"] == capi.CLASS_DISC)
    err_esc = np.abs(out.aux[esc] - o["aux"][esc]).max(initial=0)
    err_dsk = np.abs(out.aux[dsk] - o["aux"][dsk]).max(initial=0)
    assert err_esc <= aux_tol, f"deflection error {err_esc}"
    assert err_dsk <= max(aux_tol, radius_tol), f"hit radius error {err_dsk}"
    return err_esc, err_dsk


_BALL2 = [(dx, dy) for dx in range(-2, 3) for dy in range(-2, 3) if 0 < abs(dx) + abs(dy) <= 2]


def near_class_boundary(scene, xs, ys, cls, oracle_kw):
    """For each pixel (xs[i], ys[i]) of oracle class cls[i]: whether a pixel
    within Manhattan distance 2 has another oracle class."""
    if len(xs) == 0:
        return np.zeros(0, bool)
    w, h = scene.camera.width(), scene.camera.height()
    nx = np.clip(xs[:, None] + np.array([d[0] for d in _BALL2])[None, :], 0, w - 1)
    ny = np.clip(ys[:, None] + np.array([d[1] for d in _BALL2])[None, :], 0, h - 1)
    o = oracle.render_rk4(scene, pixels=np.stack([nx.ravel(), ny.ravel()], 1), **oracle_kw)
    return (o["cls"].reshape(nx.shape) != cls[:, None]).any(1)


def sample_check(scene, xs, ys, cls, bgr, aux, o, oracle_kw, aux_tol=1e-4, radius_tol=1e-3, band=1e-4, tex=0.02,
                 edge=2e-3, colour_lsb=1, min_agreement=MIN_CLASS_AGREEMENT, aux_everywhere=False):
    """The parity bar on sampled pixels. cls, bgr, aux: the GPU's values at
    (xs, ys); o: the oracle at the same pixels; oracle_kw: the oracle's
    options (step, max_steps). min_agreement=None leaves the class-agreement
    fraction to the caller (a batch counts it over all its scenes).
    aux_everywhere: the deflection bound holds on every escaped ray whose
    class agrees, boundaries included. Returns
    the number of sample pixels, class agreements and the largest deflection
    and hit-radius errors away from boundaries."""
    cls_ok = cls == o["cls"]
    soft = soft_boundary(o, band, tex, edge)
    dcol = helpers.colour_lsb(bgr, o["bgra"])
    esc = cls_ok & (o["cls"] == capi.CLASS_MISS)
    dsk = cls_ok & (o["cls"] == capi.CLASS_DISC)
    daux = np.abs(aux - o["aux"])
    fail = ~cls_ok | (cls_ok & (dcol > colour_lsb)) | (esc & (daux > aux_tol)) | \
        (dsk & (daux > max(aux_tol, radius_tol)))
    suspect = fail & ~soft
    idx = np.nonzero(suspect)[0]
    excused = near_class_boundary(scene, xs[idx], ys[idx], o["cls"][idx], oracle_kw)
    unexplained = idx[~excused]
    if min_agreement is not None:
        assert cls_ok.mean() >= min_agreement, f"class agreement {cls_ok.mean():.5f}"
    if aux_everywhere:
        assert daux[esc].max(initial=0) <= aux_tol, f"deflection error {daux[esc].max()} on an escaped ray"
    assert len(unexplained) == 0, (
        f"{len(unexplained)} pixels fail away from boundaries, e.g. {list(zip(xs[unexplained][:5], ys[unexplained][:5]))}"
        f" cls {cls[unexplained][:5]} vs {o['cls'][unexplained][:5]}, aux err {daux[unexplained][:5]}")
    boundary = soft.copy()
    boundary[idx[excused]] = True
    strict_esc = esc & ~boundary
    strict_dsk = dsk & ~boundary
    return {"pixels": int(len(xs)), "agree": int(cls_ok.sum()), "class_agreement": float(cls_ok.mean()),
            "max_deflection_error": float(daux[strict_esc].max(initial=0)),
            "max_radius_error": float(daux[strict_dsk].max(initial=0))}
