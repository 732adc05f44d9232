"""include/blackhole_gb300.hpp, the C++ face of the library: compiled with g++
against the in-tree library. On the CPU: the scene built with the C++ classes
(the reference's Camera / StaticBlackhole / Annulus construction) resolves to
the same bh_scene as the Python mirror (whose poses are pinned by the
reference's object tests), and the error paths. On the GPU: blackhole::Render
gives the same frame as the Python renderer and the oracle's hit classes."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from blackhole_8_gb300 import build, capi
from blackhole_8_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "hpp_check.cc")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    lib = build.build()
    out = tmp_path_factory.mktemp("hpp") / "hpp_check"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    SRC, "-o", str(out), "-L", libdir, "-lbh_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    return str(out)


def _scene(w, h):
    disc_tex, bg = S.standard_textures(0)
    cam = S.aimed_camera(w, h, np.radians(60), 20.0, np.radians(80))
    return S.Scene(cam, S.StaticBlackhole((0.0, 0.0, 0.0), 1.0), S.equatorial_disc(6.0, 20.0, disc_tex), bg)


def _fields(struct, prefix=""):
    """Flattened (name, value) pairs of a ctypes structure."""
    out = []
    for name, typ in struct._fields_:
        v = getattr(struct, name)
        if hasattr(v, "_fields_"):
            out += _fields(v, prefix + name + ".")
        elif isinstance(v, C._Pointer):
            out.append((prefix + name, bool(v)))  # pointers compare by being set
        elif hasattr(v, "__len__"):
            for i, x in enumerate(v):
                if hasattr(x, "__len__"):
                    out += [(f"{prefix}{name}[{i}][{j}]", y) for j, y in enumerate(x)]
                else:
                    out.append((f"{prefix}{name}[{i}]", x))
        else:
            out.append((prefix + name, v))
    return out


def test_cpp_scene_matches_python_mirror(exe):
    out = subprocess.run([exe, "pod"], capture_output=True, text=True, check=True).stdout.strip()
    got = capi.Scene.from_buffer_copy(bytes.fromhex(out))
    sc = _scene(640, 360)
    want = sc.to_c({id(sc.disc.texture): 0, id(sc.background): 1})
    for (name, g), (_, w) in zip(_fields(got), _fields(want)):
        if isinstance(w, float):
            # the same operations in another order: equal to rounding
            assert abs(g - w) <= 1e-13 * max(1.0, abs(w)), (name, g, w)
        else:
            assert g == w, (name, g, w)


def test_cpp_objects_match_python_mirror(exe):
    """Rectangle, Triangle and InfinitePlane of the C++ layer (with pose
    operations) give the bh_objects of the Python mirror."""
    out = subprocess.run([exe, "objects"], capture_output=True, text=True, check=True).stdout.split()
    got = [capi.Object.from_buffer_copy(bytes.fromhex(line)) for line in out]
    plane = S.InfinitePlane((0, 0, -6), S.ChessPattern2D(2))
    back = S.Rectangle((12, 8, 8), (12, -8, 8), (12, -8, -4), (12, 8, -4))
    side = S.Rectangle((-8, -10, 6), (8, -10, 6), (8, -10, -2), (-8, -10, -2))
    side.RotateZ(0.3)
    side.MoveX(1.5)
    tri = S.Triangle((10, -6, -3), (10, 6, -3), (10, 0, 9))
    back.texture, side.texture = object(), object()
    ids = {id(back.texture): 3, id(side.texture): 4}
    want = [o.to_c(ids) for o in (plane, back, side, tri)]
    for g, w in zip(got, want):
        for (name, a), (_, b) in zip(_fields(g), _fields(w)):
            if isinstance(b, float):
                assert abs(a - b) <= 1e-13 * max(1.0, abs(b)), (name, a, b)
            else:
                assert a == b, (name, a, b)


def test_cpp_error_paths(exe):
    import torch
    args = [exe, "errors"] + ([] if torch.cuda.is_available() else ["nodevice"])
    out = subprocess.run(args, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "ok"


@pytest.mark.gpu
def test_cpp_render_matches_python(exe, tmp_path, renderer):
    from oracle import oracle
    w, h = 96, 54
    sc = _scene(w, h)
    sc.disc.texture.texels.tofile(tmp_path / "disc.raw")
    sc.background.texels.tofile(tmp_path / "bg.raw")
    out = subprocess.run([exe, "render", str(w), str(h), str(tmp_path / "disc.raw"), str(tmp_path / "bg.raw"),
                          str(tmp_path / "out.raw")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    raw = np.fromfile(tmp_path / "out.raw", dtype=np.uint8)
    px = raw[:w * h * 3].reshape(h, w, 3)
    cls = raw[w * h * 3:].reshape(h, w)
    ref = renderer.render([sc], capi.default_options(format=capi.FORMAT_BGR8), hit_class=True)[0]
    assert np.array_equal(px, ref.pixels)
    assert np.array_equal(cls, ref.hit_class)
    orc = oracle.render_rk4(sc)
    assert (cls == orc["cls"]).mean() > 0.999


@pytest.mark.gpu
def test_cpp_binary_render_matches_python(exe, tmp_path, renderer):
    """Two holes through the C++ layer's Scene::extra_holes and the MULTI
    integrator: the same frame as the Python mirror's binary scene."""
    w, h = 64, 36
    sc = S.binary_scene(w, h)
    sc.disc.texture.texels.tofile(tmp_path / "disc.raw")
    sc.background.texels.tofile(tmp_path / "bg.raw")
    out = subprocess.run([exe, "binary", str(w), str(h), str(tmp_path / "disc.raw"), str(tmp_path / "bg.raw"),
                          str(tmp_path / "out.raw")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    raw = np.fromfile(tmp_path / "out.raw", dtype=np.uint8)
    px = raw[:w * h * 3].reshape(h, w, 3)
    cls = raw[w * h * 3:].reshape(h, w)
    ref = renderer.render([sc], capi.default_options(integrator=capi.INTEGRATOR_MULTI, precision=capi.PRECISION_FP64,
                                                     step=0.02, max_steps=20000, format=capi.FORMAT_BGR8),
                          hit_class=True)[0]
    assert np.array_equal(px, ref.pixels)
    assert np.array_equal(cls, ref.hit_class)
    assert (cls == capi.CLASS_HORIZON).sum() > 0 and (cls == capi.CLASS_DISC).sum() > 0
