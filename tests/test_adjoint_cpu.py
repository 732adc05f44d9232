"""Host-only checks of the differentiable render's interface and of its oracle.

- The adjoint structs of include/bh_gb300.h match their ctypes layouts and
  the defaults are the documented ones.
- bh_scene_at_theta (host code of the library) moves a scene to theta the way
  the oracle's differentiable render applies theta: rendering the moved scene
  at its own parameters gives the same image as rendering the scene at theta.
- The oracle's FP64 dual-number gradient agrees with FP64 central finite
  differences (h = 1e-5, Richardson with h/2, pixels masked where the
  differences are not resolved or the ray's structure changes) to 1e-3.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from blackhole_8_gb300 import build, capi

from helpers import adjoint_case, fd_protocol

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def test_adjoint_struct_layouts(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stddef.h>
#include <stdio.h>
#include "bh_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(bh_adjoint_options), sizeof(bh_adjoint_frame),
         sizeof(bh_adjoint_result), offsetof(bh_adjoint_options, band),
         offsetof(bh_adjoint_options, checkpoint_every), offsetof(bh_adjoint_result, steps),
         offsetof(bh_adjoint_result, kernel_ms));
  printf("%d %d %d\n", BH_GRAD_COUNT, BH_GRAD_TILT, BH_GRAD_R_OUTER);
  return 0;
}
''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert list(map(int, out[0].split())) == [
        C.sizeof(capi.AdjointOptions), C.sizeof(capi.AdjointFrame), C.sizeof(capi.AdjointResult),
        capi.AdjointOptions.band.offset, capi.AdjointOptions.checkpoint_every.offset,
        capi.AdjointResult.steps.offset, capi.AdjointResult.kernel_ms.offset]
    assert list(map(int, out[1].split())) == [capi.GRAD_COUNT, capi.GRAD_TILT, capi.GRAD_R_OUTER]


def test_adjoint_defaults(lib):
    o = capi.adjoint_options()
    assert o.precision == capi.PRECISION_MIXED and o.max_steps == 4000 and o.step == 0.01
    assert o.r_escape == 100.0 and o.softness == 0.1 and o.checkpoint_every == 64 and o.threads_per_block == 128
    assert o.band > 0


def _rot(v, a, t):
    v, a = np.asarray(v, float), np.asarray(a, float)
    return v * math.cos(t) + np.cross(a, v) * math.sin(t) + a * np.dot(a, v) * (1 - math.cos(t))


def test_scene_at_theta_pose(lib):
    from blackhole_8_gb300 import scene as S
    sc = S.single_scene(64, 48)
    cs = sc.to_c({id(sc.disc.texture): 0, id(sc.background): 1})
    th = np.array([1.3, 0.5, -0.2, 0.7, 0.02, -0.03, 0.04, 0.05, 5.5, 21.0])
    out = capi.Scene()
    assert lib.bh_scene_at_theta(C.byref(cs), th.ctypes.data, C.byref(out)) == capi.BH_OK
    cam0, cam = cs.camera, out.camera
    ax = [np.array(cam0.axis_x[:]), np.array(cam0.axis_y[:]), np.array(cam0.axis_z[:])]
    for k, name in enumerate(("axis_x", "axis_y", "axis_z")):
        want = _rot(_rot(_rot(ax[k], ax[0], th[6]), ax[1], th[5]), ax[2], th[4])
        np.testing.assert_allclose(np.array(getattr(cam, name)[:]), want, atol=1e-14)
    np.testing.assert_allclose(np.array(cam.position[:]), np.array(cam0.position[:]) + th[1:4], atol=1e-14)
    e1 = np.array(cs.disc.edge_s1[:]) / np.linalg.norm(cs.disc.edge_s1[:])
    np.testing.assert_allclose(np.array(out.disc.normal[:]), _rot(cs.disc.normal[:], e1, th[7]), atol=1e-14)
    assert out.hole.mass == th[0] and out.disc.r_inner == th[8] and out.disc.r_outer == th[9]
    # the theta of the scene itself leaves it unchanged
    base = np.array([cs.hole.mass, 0, 0, 0, 0, 0, 0, 0, cs.disc.r_inner, cs.disc.r_outer])
    same = capi.Scene()
    assert lib.bh_scene_at_theta(C.byref(cs), base.ctypes.data, C.byref(same)) == capi.BH_OK
    assert bytes(same) == bytes(cs)
    bad = th.copy()
    bad[2] = float("nan")
    assert lib.bh_scene_at_theta(C.byref(cs), bad.ctypes.data, C.byref(out)) == capi.BH_ERR_INVALID_ARGUMENT


def test_scene_at_theta_renders_like_theta(lib):
    """Oracle render of the scene at theta == oracle render of the moved scene
    at its own parameters."""
    from oracle import oracle
    from blackhole_8_gb300 import scene as S
    sc = S.single_scene(48, 36)
    cs = oracle._scene_c(sc)
    th = oracle.base_theta(sc)
    th[0] *= 1.05
    th[2] += 0.3
    th[4] += 0.02
    th[5] -= 0.015
    th[6] += 0.03
    th[7] += math.radians(3)
    th[9] += 2
    moved = capi.Scene()
    assert lib.bh_scene_at_theta(C.byref(cs), th.ctypes.data, C.byref(moved)) == capi.BH_OK
    img_a, _, _ = oracle.smooth_render(sc, th)
    th_moved = np.array([moved.hole.mass, 0, 0, 0, 0, 0, 0, 0, moved.disc.r_inner, moved.disc.r_outer])
    img_b, _, _ = oracle.smooth_render(sc, th_moved, scene_c=moved)
    np.testing.assert_allclose(img_a, img_b, atol=1e-9)


def test_oracle_dual_gradient_matches_finite_differences():
    """Pins the oracle's gradient: FP64 dual numbers vs FP64 central
    differences of the FP64 loss (h = 1e-5)."""
    from oracle import oracle
    sc, th0, tt, target = adjoint_case(64, 48)
    g = oracle.smooth_grad(sc, target, th0)
    loss_at = lambda th: oracle.smooth_render(sc, th, target)[1]
    sig_at = lambda th: oracle.smooth_render(sc, th, target)[2]
    for i in range(capi.GRAD_COUNT):
        rich, ok = fd_protocol(loss_at, th0, i, signature_at=sig_at)
        assert ok.mean() > 0.9, (capi.GRAD_NAMES[i], ok.mean())
        fd, du = rich[ok].sum(), g[..., i][ok].sum()
        assert abs(fd - du) <= 1e-3 * abs(du), (capi.GRAD_NAMES[i], fd, du)
