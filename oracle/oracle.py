"""Test infrastructure: builds and binds the FP64 CPU oracles (bh_oracle.c:
the reference's trapezoid render and the RK4 render; bh_oracle_smooth.cc:
the differentiable render, its forward-mode dual-number gradient).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker, never as the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libbh_oracle.so")
SRC = os.path.join(HERE, "bh_oracle.c")


class OrcTexture(C.Structure):
    _fields_ = [("bgra", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32)]


class OrcRk4Opts(C.Structure):
    _fields_ = [("step", C.c_double), ("max_steps", C.c_int32), ("r_escape", C.c_double)]


class OrcOutputs(C.Structure):
    _fields_ = [("bgra", C.c_void_p), ("cls", C.c_void_p), ("aux", C.c_void_p), ("margin_tex", C.c_void_p),
                ("margin_r", C.c_void_p), ("b_over_m", C.c_void_p), ("steps", C.c_void_p)]


SRC_SMOOTH = os.path.join(HERE, "bh_oracle_smooth.cc")


def build(force: bool = False) -> str:
    inc = os.path.join(ROOT, "include")
    newest = max(os.path.getmtime(SRC), os.path.getmtime(SRC_SMOOTH), os.path.getmtime(os.path.join(inc, "bh_gb300.h")))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    obj_c = os.path.join(BUILD_DIR, "bh_oracle.o")
    obj_cc = os.path.join(BUILD_DIR, "bh_oracle_smooth.o")
    subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-std=c11", "-I", inc, "-c", SRC, "-o", obj_c], check=True)
    subprocess.run(["g++", "-O2", "-fopenmp", "-fPIC", "-std=c++17", "-I", inc, "-c", SRC_SMOOTH, "-o", obj_cc],
                   check=True)
    tmp = LIB + ".tmp"
    subprocess.run(["g++", "-shared", "-fopenmp", obj_c, obj_cc, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        lib.orc_render_ref.restype = C.c_int
        lib.orc_render_ref.argtypes = [C.c_void_p, C.POINTER(OrcTexture), C.POINTER(OrcTexture), C.c_void_p,
                                       C.c_int64, C.POINTER(OrcOutputs), C.c_int]
        lib.orc_render_flat.restype = C.c_int
        lib.orc_render_flat.argtypes = [C.c_void_p, C.POINTER(OrcTexture), C.POINTER(OrcTexture), C.c_void_p,
                                        C.c_int64, C.POINTER(OrcOutputs), C.c_int]
        lib.orc_render_rk4.restype = C.c_int
        lib.orc_render_rk4.argtypes = [C.c_void_p, C.POINTER(OrcTexture), C.POINTER(OrcTexture),
                                       C.POINTER(OrcTexture), C.POINTER(OrcRk4Opts), C.c_void_p, C.c_int64,
                                       C.POINTER(OrcOutputs), C.c_int]
        lib.orc_render_multi.restype = C.c_int
        lib.orc_render_multi.argtypes = lib.orc_render_rk4.argtypes
        lib.orc_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def _tex(t):
    if t is None:
        return None, None
    arr = np.ascontiguousarray(t.bgra())
    ot = OrcTexture(arr.ctypes.data, arr.shape[1], arr.shape[0])
    return ot, arr


def _scene_c(scene):
    """bh_scene POD of a mirror Scene (texture ids are placeholders: the
    oracle receives the texels directly). The object table stays alive in
    the struct's `_keep`."""
    ids = {}
    for t in scene.textures():
        ids.setdefault(id(t), len(ids))
    s = scene.to_c(ids)
    return s


def _obj_tex(scene):
    """One OrcTexture per object (empty where it has none), and the arrays
    that keep the texels alive."""
    if not scene.objects:
        return None, []
    arr = (OrcTexture * len(scene.objects))()
    keep = []
    for i, o in enumerate(scene.objects):
        t = getattr(o, "texture", None)
        if t is not None:
            ot, a = _tex(t)
            arr[i] = ot
            keep.append(a)
    return arr, keep


def _pixels(pixels):
    if pixels is None:
        return None, 0, None
    arr = np.ascontiguousarray(np.asarray(pixels, dtype=np.int32).reshape(-1, 2))
    return arr.ctypes.data, arr.shape[0], arr


def render_ref(scene, pixels=None, threads: int = 0) -> dict:
    """Oracle A: the reference's trapezoid render, FP64. margin_tex: for disc
    and object hits, the distance (texels, or pattern cells for the chess
    plane) of the colour's sampling coordinate to the nearest edge where the
    colour can change; 1 elsewhere."""
    lib = load()
    s = _scene_c(scene)
    dt, dta = _tex(scene.disc.texture if scene.disc is not None else None)
    pp, n, keep = _pixels(pixels)
    if pp is None:
        n = scene.camera.width() * scene.camera.height()
    bgra = np.zeros((n, 4), np.uint8)
    cls = np.zeros(n, np.uint8)
    margin = np.zeros(n)
    out = OrcOutputs(bgra.ctypes.data, cls.ctypes.data, None, margin.ctypes.data, None, None, None)
    ot, otk = _obj_tex(scene)
    lib.orc_render_ref(C.byref(s), C.byref(dt) if dt else None, ot, pp, n, C.byref(out), threads)
    res = {"bgra": bgra, "cls": cls, "margin_tex": margin}
    if pixels is None:
        h, w = scene.camera.height(), scene.camera.width()
        res = {k: v.reshape((h, w) + v.shape[1:]) for k, v in res.items()}
    return res


def render_rk4(scene, step: float = 0.01, max_steps: int = 4000, r_escape: float = 100.0, pixels=None,
               threads: int = 0, multi: bool = False) -> dict:
    """Oracle B: RK4 in phi, FP64 (multi: the MULTI integrator's RK4 in arc
    length over the scene's hole and extra holes; step is its factor on the
    distance to the nearest hole, r_escape in units of the total mass)."""
    lib = load()
    s = _scene_c(scene)
    dt, dta = _tex(scene.disc.texture if scene.disc is not None else None)
    bt, bta = _tex(scene.background)
    pp, n, keep = _pixels(pixels)
    if pp is None:
        n = scene.camera.width() * scene.camera.height()
    res = {
        "bgra": np.zeros((n, 4), np.uint8), "cls": np.zeros(n, np.uint8), "aux": np.zeros(n),
        "margin_tex": np.zeros(n), "margin_r": np.zeros(n), "b_over_m": np.zeros(n),
        "steps": np.zeros(n, np.int32),
    }
    out = OrcOutputs(*(res[k].ctypes.data for k in ("bgra", "cls", "aux", "margin_tex", "margin_r", "b_over_m",
                                                    "steps")))
    opts = OrcRk4Opts(step, max_steps, r_escape)
    ot, otk = _obj_tex(scene)
    fn = lib.orc_render_multi if multi else lib.orc_render_rk4
    fn(C.byref(s), C.byref(dt) if dt else None, C.byref(bt) if bt else None, ot, C.byref(opts), pp, n, C.byref(out),
       threads)
    if pixels is None:
        h, w = scene.camera.height(), scene.camera.width()
        res = {k: v.reshape((h, w) + v.shape[1:]) for k, v in res.items()}
    return res


def render_multi(scene, step: float = 0.01, max_steps: int = 4000, r_escape: float = 100.0, pixels=None,
                 threads: int = 0) -> dict:
    """The MULTI integrator, FP64 (REF ray generation)."""
    return render_rk4(scene, step, max_steps, r_escape, pixels, threads, multi=True)


def render_flat(scene, pixels=None, threads: int = 0) -> dict:
    """The flat RayTracer (REF ray generation), FP64; aux = object index."""
    lib = load()
    s = _scene_c(scene)
    dt, dta = _tex(scene.disc.texture if scene.disc is not None else None)
    ot, otk = _obj_tex(scene)
    pp, n, keep = _pixels(pixels)
    if pp is None:
        n = scene.camera.width() * scene.camera.height()
    res = {"bgra": np.zeros((n, 4), np.uint8), "cls": np.zeros(n, np.uint8), "aux": np.zeros(n),
           "margin_tex": np.zeros(n)}
    out = OrcOutputs(res["bgra"].ctypes.data, res["cls"].ctypes.data, res["aux"].ctypes.data,
                     res["margin_tex"].ctypes.data, None, None, None)
    lib.orc_render_flat(C.byref(s), C.byref(dt) if dt else None, ot, pp, n, C.byref(out), threads)
    if pixels is None:
        h, w = scene.camera.height(), scene.camera.width()
        res = {k: v.reshape((h, w) + v.shape[1:]) for k, v in res.items()}
    return res


def max_threads() -> int:
    return load().orc_max_threads()


# ---------------------------------------------------------------------------
# differentiable render (bh_oracle_smooth.cc)
class OrcSmoothOpts(C.Structure):
    _fields_ = [("step", C.c_double), ("max_steps", C.c_int32), ("r_escape", C.c_double), ("softness", C.c_double)]


N_PARAMS = 10


def _smooth_args(scene, step, max_steps, r_escape, softness, scene_c=None):
    s = _scene_c(scene) if scene_c is None else scene_c
    dtex = np.ascontiguousarray(scene.disc.texture.bgra())
    bg = np.ascontiguousarray(scene.background.bgra()) if scene.background is not None else None
    opts = OrcSmoothOpts(step, max_steps, r_escape, softness)
    return s, dtex, bg, opts


def base_theta(scene) -> np.ndarray:
    """theta of a scene itself: M, zero pose offsets, zero tilt, its radii."""
    return np.array([scene.hole.mass(), 0, 0, 0, 0, 0, 0, 0, scene.disc.r_inner(), scene.disc.r_outer()],
                    dtype=np.float64)


def smooth_render(scene, theta=None, target=None, step=0.01, max_steps=4000, r_escape=100.0, softness=0.1,
                  threads=0, scene_c=None):
    """Differentiable render at theta (FP64): image (H, W, 3), per-pixel loss
    sum_c (C - target)^2, per-pixel ray signature. scene_c (a bh_scene)
    replaces the poses of `scene`, whose textures are used."""
    lib = load()
    lib.orc_smooth_render.restype = C.c_int
    s, dtex, bg, opts = _smooth_args(scene, step, max_steps, r_escape, softness, scene_c)
    th = np.ascontiguousarray(base_theta(scene) if theta is None else theta, dtype=np.float64)
    h, w = scene.camera.height(), scene.camera.width()
    img = np.zeros((h, w, 3))
    loss = np.zeros((h, w))
    sig = np.zeros((h, w), np.uint32)
    tg = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
    lib.orc_smooth_render(C.byref(s), th.ctypes.data_as(C.c_void_p), dtex.ctypes.data_as(C.c_void_p),
                          dtex.shape[1], dtex.shape[0], bg.ctypes.data_as(C.c_void_p) if bg is not None else None,
                          bg.shape[1] if bg is not None else 0, bg.shape[0] if bg is not None else 0, C.byref(opts),
                          tg.ctypes.data_as(C.c_void_p) if tg is not None else None, img.ctypes.data_as(C.c_void_p),
                          loss.ctypes.data_as(C.c_void_p), sig.ctypes.data_as(C.c_void_p), threads)
    return img, loss, sig


def smooth_grad(scene, target, theta=None, step=0.01, max_steps=4000, r_escape=100.0, softness=0.1, threads=0):
    """Per-pixel gradient (H, W, 10) of sum_c (C - target)^2 by FP64 forward
    mode (dual numbers)."""
    lib = load()
    lib.orc_smooth_grad.restype = C.c_int
    s, dtex, bg, opts = _smooth_args(scene, step, max_steps, r_escape, softness)
    th = np.ascontiguousarray(base_theta(scene) if theta is None else theta, dtype=np.float64)
    h, w = scene.camera.height(), scene.camera.width()
    g = np.zeros((h, w, N_PARAMS))
    tg = np.ascontiguousarray(target, dtype=np.float32)
    lib.orc_smooth_grad(C.byref(s), th.ctypes.data_as(C.c_void_p), dtex.ctypes.data_as(C.c_void_p),
                        dtex.shape[1], dtex.shape[0], bg.ctypes.data_as(C.c_void_p) if bg is not None else None,
                        bg.shape[1] if bg is not None else 0, bg.shape[0] if bg is not None else 0, C.byref(opts),
                        tg.ctypes.data_as(C.c_void_p), g.ctypes.data_as(C.c_void_p), threads)
    return g
