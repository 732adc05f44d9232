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


BUILDERS = {"cfg0_planar": cfg0_planar, "ref_demo": ref_demo, "posed": posed}

GOLDEN_CASES = [
    ("cfg0_planar", 64, 36),
    ("cfg0_planar", 160, 90),
    ("ref_demo", 320, 180),
    ("posed", 80, 45),
]


def build(name: str, width: int, height: int) -> S.Scene:
    return BUILDERS[name](width, height)


def class_boundary_mask(cls: np.ndarray) -> np.ndarray:
    """Pixels with a 4-neighbour of another class."""
    m = np.zeros(cls.shape, dtype=bool)
    m[1:, :] |= cls[1:, :] != cls[:-1, :]
    m[:-1, :] |= cls[:-1, :] != cls[1:, :]
    m[:, 1:] |= cls[:, 1:] != cls[:, :-1]
    m[:, :-1] |= cls[:, :-1] != cls[:, 1:]
    return m
