"""The MULTI integrator's CPU restatement (oracle/bh_oracle.c multi_pixel),
pinned by physics rather than by the reference, whose multi-hole experiment
(multiple_blackhole_solution_test.cc, disabled in its CMakeLists) has no
output to compare with:

- one hole: the angle between an escaped ray's first and last direction
  against the Schwarzschild orbit integral. The swept angle phi is the same
  in Schwarzschild and isotropic coordinates; the impact parameter is the
  conserved b = n(rho) rho sin(chi), chi the angle from the inward radial
  direction, n = (1 + m/2rho)^3 / (1 - m/2rho); the bending is
  dphi - pi + chi + chi_e with chi_e the exit angle at the escape sphere.
  Bound 1e-8 rad at step 0.01 (fourth order: 3e-10 measured);
- one hole: disc hits at the radius the inverted orbit integral gives at
  the disc plane's crossing angles (isotropic radius within 1e-7 M);
- one hole: rays with b below 3 sqrt(3) m are captured, above it escape;
- an equal-mass binary seen from its mirror plane renders mirror
  symmetric (classes exactly, the bending within 1e-9 rad);
- a third hole changes the image (every hole takes part).
"""
import math

import numpy as np
import pytest

from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S
from oracle import oracle

B_C = 3.0 * math.sqrt(3.0)


def n_iso(rho, m=1.0):
    return (1 + m / (2 * rho)) ** 3 / (1 - m / (2 * rho))


def kat_bending(b, chi, rho_c, R, m=1.0):
    """Bending of a ray from isotropic radius rho_c (angle chi from the
    inward radial direction) to the escape sphere of isotropic radius R."""
    quad = pytest.importorskip("scipy.integrate").quad
    r_c = rho_c * (1 + m / (2 * rho_c)) ** 2
    r_e = R * (1 + m / (2 * R)) ** 2
    u_c, u_e = m / r_c, m / r_e
    # 2u^3 - u^2 + (m/b)^2 = 2 (u - u1)(u - up)(u - u3), u1 < 0 < up < u3
    u1, up, u3 = np.sort(np.roots([2.0, -1.0, 0.0, (m / b) ** 2]).real)

    def I(u0):  # int_{u0}^{up} du / sqrt(G), with u = up - s^2
        f = lambda s: 2.0 / math.sqrt(2.0 * ((up - s * s) - u1) * (u3 - (up - s * s)))
        return quad(f, 0.0, math.sqrt(max(up - u0, 0.0)), epsabs=1e-14, epsrel=1e-13, limit=200)[0]

    dphi = I(u_c) + I(u_e) if math.cos(chi) > 0 else I(u_e) - I(u_c)
    chi_e = math.asin(b / (n_iso(R, m) * R))
    return dphi - math.pi + chi + chi_e


def first_direction(cam, x, y):
    pv = np.asarray(cam.PixelVector(x, y, cam.focus_vector()), float)
    d = pv - np.asarray(cam.focus(), float)
    return d / np.linalg.norm(d)


@pytest.fixture(scope="module")
def single():
    sc = S.single_scene(48, 27)
    return sc, oracle.render_multi(sc, step=0.01, max_steps=20000)


def test_one_hole_bending_matches_orbit_integral(single):
    sc, o = single
    cam = sc.camera
    F = np.asarray(cam.focus(), float) - np.asarray(sc.hole.position(), float)
    rho_c = float(np.linalg.norm(F))
    errs = []
    for y in range(cam.height()):
        for x in range(cam.width()):
            T0 = first_direction(cam, x, y)
            chi = math.acos(float(np.clip(np.dot(T0, -F / rho_c), -1, 1)))
            b = n_iso(rho_c) * rho_c * math.sin(chi)
            assert abs(b - o["b_over_m"][y, x]) <= 1e-9 * b
            if o["cls"][y, x] != capi.CLASS_MISS or b < B_C + 0.05:
                continue
            k = kat_bending(b, chi, rho_c, 100.0)
            if 0 < k < math.pi:
                errs.append(abs(k - o["aux"][y, x]))
    assert len(errs) > 150
    assert max(errs) < 1e-8, max(errs)


def test_one_hole_shadow_edge(single):
    sc, _ = single
    bare = S.Scene(sc.camera, sc.hole, None, sc.background)
    o = oracle.render_multi(bare, step=0.01, max_steps=20000)
    b, cls = o["b_over_m"], o["cls"]
    inside = b < B_C - 0.02
    outside = b > B_C + 0.02
    assert inside.any() and outside.any()
    assert (cls[inside] == capi.CLASS_HORIZON).all()
    assert not (cls[outside] == capi.CLASS_HORIZON).any()


def test_binary_mirror_symmetry():
    W, H = 49, 27
    sc = S.binary_scene(W, H)
    o = oracle.render_multi(sc, step=0.02, max_steps=20000)
    cls, aux = o["cls"].astype(int), o["aux"]
    # column x sits at a = W/2 - x from the axis: its mirror is column W - x
    lo, hi = 1, W
    mirror = lambda a: a[:, lo:hi][:, ::-1]
    assert np.array_equal(cls[:, lo:hi], mirror(cls))
    miss = cls[:, lo:hi] == capi.CLASS_MISS
    assert miss.any() and (cls == capi.CLASS_DISC).any() and (cls == capi.CLASS_HORIZON).any()
    assert np.abs(aux[:, lo:hi] - mirror(aux))[miss].max() < 1e-9


def test_third_hole_changes_the_image():
    """The restatement takes every hole: a third, lighter hole above the
    binary's disc plane changes classes or bending across the image."""
    two = S.binary_scene(48, 27)
    three = S.binary_scene(48, 27)
    three.extra_holes.append(S.StaticBlackhole((-2.0, 0.0, 2.5), 0.25))
    a = oracle.render_multi(two, step=0.02, max_steps=20000)
    b = oracle.render_multi(three, step=0.02, max_steps=20000)
    changed = (a["cls"] != b["cls"]) | (np.abs(a["aux"] - b["aux"]) > 1e-3)
    assert changed.mean() > 0.05, changed.mean()
    assert (b["cls"] == capi.CLASS_HORIZON).sum() > (a["cls"] == capi.CLASS_HORIZON).sum()


def _orbit_u_at(phi_c, b, u_c, inward, m=1.0):
    """u = m / r (areal) where the one-hole orbit of impact parameter b,
    leaving u_c inward (or outward), has swept phi_c; None past the escape
    branch's start. Inverts the orbit integral with the s-substitution."""
    opt = pytest.importorskip("scipy.optimize")
    quad = pytest.importorskip("scipy.integrate").quad
    u1, up, u3 = np.sort(np.roots([2.0, -1.0, 0.0, (m / b) ** 2]).real)

    def I(u0):  # int_{u0}^{up} du / sqrt(G)
        f = lambda s: 2.0 / math.sqrt(2.0 * ((up - s * s) - u1) * (u3 - (up - s * s)))
        return quad(f, 0.0, math.sqrt(max(up - u0, 0.0)), epsabs=1e-14, epsrel=1e-13, limit=200)[0]

    i_c = I(u_c)
    if inward and phi_c <= i_c:  # before the periapsis: int_{u_c}^{u} = phi_c
        return opt.brentq(lambda u: (i_c - I(u)) - phi_c, u_c, up, xtol=1e-15)
    rest = phi_c - i_c if inward else phi_c + i_c  # past it: int_u^{up} = rest, u from up down to 0
    if rest > I(1e-12):
        return None
    return opt.brentq(lambda u: I(u) - rest, 1e-12, up, xtol=1e-15)


def test_one_hole_disc_hits_match_orbit_integral(single):
    """Where a ray first meets the equatorial disc within its radii, the
    orbit integral gives the areal radius at that crossing angle (the disc
    plane contains the hole, so the crossings lie at the line of nodes plus
    multiples of pi). Converted to the isotropic radius, it is the hit's
    distance from the disc centre; the restatement's agrees within 1e-7 M
    at step 0.01."""
    sc, o = single
    cam, d = sc.camera, sc.disc
    F = np.asarray(cam.focus(), float) - np.asarray(sc.hole.position(), float)
    rho_c = float(np.linalg.norm(F))
    Fh = F / rho_c
    r_c = rho_c * (1 + 0.5 / rho_c) ** 2
    z = np.array([0.0, 0.0, 1.0])
    errs = []
    for y in range(0, cam.height(), 2):
        for x in range(0, cam.width(), 2):
            if o["cls"][y, x] != capi.CLASS_DISC or o["margin_r"][y, x] < 1e-3:
                continue
            T0 = first_direction(cam, x, y)
            chi = math.acos(float(np.clip(np.dot(T0, -Fh), -1, 1)))
            b = n_iso(rho_c) * rho_c * math.sin(chi)
            if b < B_C + 0.05:
                continue
            e2 = T0 - np.dot(T0, Fh) * Fh
            e2 /= np.linalg.norm(e2)
            # crossings: cos(phi) (Fh . z) + sin(phi) (e2 . z) = 0
            phi_n = math.atan2(-np.dot(Fh, z), np.dot(e2, z)) % math.pi
            want = None
            for k in range(4):
                u = _orbit_u_at(phi_n + k * math.pi, b, 1.0 / r_c, math.cos(chi) > 0)
                if u is None:
                    break
                r = 1.0 / u
                rho = (r - 1 + math.sqrt(r * r - 2 * r)) / 2  # isotropic radius of areal r
                if d.r_inner() <= rho <= d.r_outer():
                    want = rho
                    break
            assert want is not None, (x, y)
            errs.append(abs(want - o["aux"][y, x]))
    assert len(errs) > 20
    assert max(errs) < 1e-7, max(errs)
