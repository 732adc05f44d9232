"""Scenes shared by the tests and tests/golden/make_golden.py.

Each builder is deterministic (hash-generated textures), so a golden fixture
stores only the builder's name and arguments plus the reference's output.
"""
from __future__ import annotations

import math

import numpy as np

from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S


def cfg0_planar(width: int, height: int) -> S.Scene:
    """The single-scene workload with the reference's planar disc mapping."""
    sc = S.single_scene(width, height)
    sc.disc.mapping = capi.DISC_MAP_REF_PLANAR
    return sc


def ref_demo(width: int, height: int) -> S.Scene:
    """The reference main()'s own scene (blackhole_solution_test.cc:61-148):
    Camera(W, H, pi/2) at (-2000, 0, 400), hole M = 10 at the origin, disc
    quad (1000,1000,0) (-1000,1000,0) (-1000,-0100,0) (1000,-1000,0) (the
    octal -0100 = -64 kept), r_out 1000, r_in 100; a 578x598 hash texture
    stands in for acc_disc.png (same size)."""
    cam = S.Camera(width, height, math.pi / 2)
    cam.MoveTo(-2000, 0, 400)
    disc = S.Annulus((1000, 1000, 0), (-1000, 1000, 0), (-1000, -64, 0), (1000, -1000, 0), 1000, 100)
    tex = S.value_noise_background(5, 578, 598, octaves=3, base_cells=16)
    bgr = tex.bgra()[..., :3].copy()
    bgr[bgr.sum(-1) == 0] = 1  # keep disc texels distinguishable from black
    disc.SetTexture(S.Texture(bgr, capi.TEXEL_BGR8))
    disc.mapping = capi.DISC_MAP_REF_PLANAR
    return S.Scene(cam, S.StaticBlackhole((0, 0, 0), 10), disc, None)


def posed(width: int, height: int) -> S.Scene:
    """Camera and disc moved with every pose operation of Object<T>."""
    sc = cfg0_planar(width, height)
    d = sc.disc
    d.RotateX(0.3)
    d.RotateZ(0.7)
    cam = sc.camera
    cam.RotateX(0.05)
    cam.MoveY(0.5)
    cam.MoveZ(-0.25)
    cam.MoveX(1.0)
    return sc


def flat_demo(width: int, height: int) -> S.Scene:
    """The reference's flat RayTracer scene (ray_tracer_test.cc:50-98)."""
    return S.flat_demo_scene(width, height)


def objects(width: int, height: int) -> S.Scene:
    """The planar-disc single scene with a chess plane and two panels."""
    return S.objects_scene(width, height)


def triangles(width: int, height: int) -> S.Scene:
    """The objects scene with two triangles added (checked against the
    restatement only: the reference's Triangle<T> does not compile when
    instantiated)."""
    sc = S.objects_scene(width, height)
    sc.objects += [S.Triangle((10, -6, -3), (10, 6, -3), (10, 0, 9)), S.Triangle((-4, 9, 5), (6, 9, 5), (0, 9, -3))]
    return sc


BUILDERS = {"cfg0_planar": cfg0_planar, "ref_demo": ref_demo, "posed": posed, "flat_demo": flat_demo,
            "objects": objects, "triangles": triangles}

GOLDEN_CASES = [
    ("cfg0_planar", 64, 36),
    ("cfg0_planar", 160, 90),
    ("ref_demo", 320, 180),
    ("posed", 80, 45),
    ("flat_demo", 160, 90),
    ("objects", 160, 90),
]

# builders rendered by the reference's flat RayTracer instead of the curved loop
FLAT_BUILDERS = {"flat_demo"}


def build(name: str, width: int, height: int) -> S.Scene:
    return BUILDERS[name](width, height)


# Colours may differ where the sampling coordinate lies within this many
# texels (or chess cells) of an edge: there FP64 rounding of the hit point
# alone decides which texel is read (a tie). The reference's own output and
# the FP64 restatement differ only at margins of ~1e-14 texels.
TEXEL_TIE_FP64 = 1e-6


def colour_lsb(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Largest per-channel difference of two BGR(A) images, in 8-bit LSB."""
    return np.abs(a[..., :3].astype(np.int16) - b[..., :3].astype(np.int16)).max(-1)


def class_boundary_mask(cls: np.ndarray) -> np.ndarray:
    """Pixels with a 4-neighbour of another class."""
    m = np.zeros(cls.shape, dtype=bool)
    m[1:, :] |= cls[1:, :] != cls[:-1, :]
    m[:-1, :] |= cls[:-1, :] != cls[1:, :]
    m[:, 1:] |= cls[:, 1:] != cls[:, :-1]
    m[:, :-1] |= cls[:, :-1] != cls[:, 1:]
    return m


# ---------------------------------------------------------------------------
# differentiable render (adjoint) cases
def adjoint_thetas(scene: S.Scene):
    """theta of the scene itself and the target theta of the adjoint workload:
    M + 5 %, disc tilt + 3 deg, r_outer + 2 M, camera yaw and pitch + 1 deg."""
    from oracle import oracle
    th0 = oracle.base_theta(scene)
    tt = th0.copy()
    tt[capi.GRAD_MASS] *= 1.05
    tt[capi.GRAD_TILT] += math.radians(3)
    tt[capi.GRAD_R_OUTER] += 2.0
    tt[capi.GRAD_YAW] += math.radians(1)
    tt[capi.GRAD_PITCH] += math.radians(1)
    return th0, tt


def adjoint_case(width: int, height: int):
    """(scene, theta0, theta_target, target image float32 (H, W, 3)) with the
    target rendered by the FP64 oracle."""
    from oracle import oracle
    sc = S.single_scene(width, height)
    th0, tt = adjoint_thetas(sc)
    target, _, _ = oracle.smooth_render(sc, tt)
    return sc, th0, tt, np.ascontiguousarray(target.astype(np.float32))


def fd_protocol(loss_at, theta: np.ndarray, i: int, h: float = 1e-5, signature_at=None):
    """Central differences of the per-pixel loss in parameter i at h, h/2 and
    h/4. Returns (Richardson estimate from h and h/2, mask of the pixels where
    the estimate is trusted): the three differences agree within 1 % of the
    estimate, or within 1e-6 of the largest estimate (the loss is resolved
    at h) and, when signature_at is given, the
    ray's structure is the same at all six points."""
    fds = []
    mask = None
    base_sig = signature_at(theta) if signature_at else None
    for hh in (h, h / 2, h / 4):
        tp = theta.copy()
        tp[i] += hh
        tm = theta.copy()
        tm[i] -= hh
        lp, lm = loss_at(tp), loss_at(tm)
        fds.append((lp - lm) / (2 * hh))
        if signature_at:
            same = (signature_at(tp) == base_sig) & (signature_at(tm) == base_sig)
            mask = same if mask is None else mask & same
    rich = (4 * fds[1] - fds[0]) / 3
    # tiny derivatives are resolved to rounding only; they weigh nothing
    atol = 1e-6 * float(np.abs(rich).max())
    ok = (np.abs(fds[0] - fds[1]) <= 1e-2 * np.abs(rich) + atol) & \
         (np.abs(fds[1] - fds[2]) <= 1e-2 * np.abs(rich) + atol)
    return rich, ok if mask is None else ok & mask
