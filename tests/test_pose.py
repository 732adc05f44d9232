"""Pose conventions of the scene mirror.

The first test restates, as behaviour, the assertions of the reference's
object/object_test.cc:22-55 (Move/MoveTo and the +-pi/2 RotateX/Y/Z
results), within float_equal's tolerance cbrt(DBL_EPSILON) (utility.h:17-27).
"""
import math

import numpy as np

from blackhole_8_gb300 import scene as S

EPS = np.cbrt(np.finfo(np.float64).eps)


def close(a, b):
    return np.all(np.abs(np.asarray(a) - np.asarray(b)) <= EPS)


def test_object_test_kats():
    obj = S.Object(((0, 0, 0),))
    obj.MoveTo(10, 10, 10)
    assert close(obj.position(), (10, 10, 10))
    obj.Move(11, 12, 13)
    assert close(obj.position(), (21, 22, 23))
    obj.MoveTo(0, 0, 0)
    obj.MoveX(12345)
    assert close(obj.position(), (12345, 0, 0))
    obj.MoveY(12345)
    assert close(obj.position(), (12345, 12345, 0))
    obj.MoveZ(12345)
    assert close(obj.position(), (12345, 12345, 12345))

    obj.RotateX(math.pi / 2)
    assert close(obj.vector_x(), (1, 0, 0))
    assert close(obj.vector_y(), (0, 0, 1))
    assert close(obj.vector_z(), (0, -1, 0))
    obj.RotateX(-math.pi / 2)

    obj.RotateY(math.pi / 2)
    assert close(obj.vector_x(), (0, 0, -1))
    assert close(obj.vector_y(), (0, 1, 0))
    assert close(obj.vector_z(), (1, 0, 0))
    obj.RotateY(-math.pi / 2)

    obj.RotateZ(math.pi / 2)
    assert close(obj.vector_x(), (0, 1, 0))
    assert close(obj.vector_y(), (-1, 0, 0))
    assert close(obj.vector_z(), (0, 0, 1))
    obj.RotateZ(-math.pi / 2)


def test_camera_conventions():
    cam = S.Camera(640, 360, math.radians(60))
    assert close(cam.vector_x(), (1, 0, 0)) and close(cam.vector_y(), (0, -1, 0)) and close(cam.vector_z(), (0, 0, -1))
    assert abs(cam.focus_len() - 640 / (2 * math.tan(math.radians(30)))) < 1e-12
    # PixelVector at the image centre is the focus vector (camera.h:55-63)
    assert close(cam.PixelVector(320, 180), cam.focus_vector())
    cam.fov(10.0)
    assert cam.fov() < math.pi


def test_aimed_camera_looks_at_hole():
    for inc in (0.0, 0.3, 1.4, math.pi / 2):
        for az in (0.0, 1.0, 4.0):
            cam = S.aimed_camera(64, 64, 1.0, 17.0, inc, az)
            p = cam.position()
            assert abs(np.linalg.norm(p) - 17.0) < 1e-12
            assert close(cam.vector_x(), -p / np.linalg.norm(p))
            assert abs(math.acos(p[2] / 17.0) - inc) < 1e-9


def test_annulus_keeps_default_vertex_and_fixed_normal():
    d = S.Annulus((1, 1, 0), (-1, 1, 0), (-1, -1, 0), (1, -1, 0), 1, 0.5)
    v = d.vertex()
    assert len(v) == 5 and close(v[0], (0, 0, 0))
    assert close(d.norm(), (0, 0, -1))
    d.RotateX(0.5)
    assert close(d.norm(), (0, 0, -1))  # norm_ is not updated (vector_object.h:325)
    assert not close(d.vertex()[1], (1, 1, 0))


def test_textures_are_deterministic():
    a = S.disc_ring_texture(3, 256, 16).texels
    b = S.disc_ring_texture(3, 256, 16).texels
    assert np.array_equal(a, b)
    assert (a[..., :3].sum(-1) > 0).all()
    assert len(np.unique(a.reshape(-1, 4), axis=0)) == 4
    bg = S.value_noise_background(1, 128, 64).texels
    assert bg.shape == (64, 128, 3)
    assert np.array_equal(bg, S.value_noise_background(1, 128, 64).texels)
