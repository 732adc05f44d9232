"""Test infrastructure: builds and binds the FP64 CPU oracle (bh_oracle.c).

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


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(ROOT, "include", "bh_gb300.h"))):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-I", os.path.join(ROOT, "include"),
                    SRC, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        lib.orc_render_ref.restype = C.c_int
        lib.orc_render_ref.argtypes = [C.c_void_p, C.POINTER(OrcTexture), C.c_void_p, C.c_int64,
                                       C.POINTER(OrcOutputs), C.c_int]
        lib.orc_render_rk4.restype = C.c_int
        lib.orc_render_rk4.argtypes = [C.c_void_p, C.POINTER(OrcTexture), C.POINTER(OrcTexture),
                                       C.POINTER(OrcRk4Opts), C.c_void_p, C.c_int64, C.POINTER(OrcOutputs), C.c_int]
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
    oracle receives the texels directly)."""
    from blackhole_8_gb300 import capi
    ids = {}
    if scene.disc is not None:
        ids[id(scene.disc.texture)] = 0
    if scene.background is not None:
        ids[id(scene.background)] = 1
    s = scene.to_c(ids)
    return s


def _pixels(pixels):
    if pixels is None:
        return None, 0, None
    arr = np.ascontiguousarray(np.asarray(pixels, dtype=np.int32).reshape(-1, 2))
    return arr.ctypes.data, arr.shape[0], arr


def render_ref(scene, pixels=None, threads: int = 0) -> dict:
    """Oracle A: the reference's trapezoid render, FP64."""
    lib = load()
    s = _scene_c(scene)
    dt, dta = _tex(scene.disc.texture if scene.disc is not None else None)
    pp, n, keep = _pixels(pixels)
    if pp is None:
        n = scene.camera.width() * scene.camera.height()
    bgra = np.zeros((n, 4), np.uint8)
    cls = np.zeros(n, np.uint8)
    out = OrcOutputs(bgra.ctypes.data, cls.ctypes.data, None, None, None, None, None)
    lib.orc_render_ref(C.byref(s), C.byref(dt) if dt else None, pp, n, C.byref(out), threads)
    res = {"bgra": bgra, "cls": cls}
    if pixels is None:
        h, w = scene.camera.height(), scene.camera.width()
        res = {k: v.reshape((h, w) + v.shape[1:]) for k, v in res.items()}
    return res


def render_rk4(scene, step: float = 0.01, max_steps: int = 4000, r_escape: float = 100.0, pixels=None,
               threads: int = 0) -> dict:
    """Oracle B: RK4 in phi, FP64."""
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
    lib.orc_render_rk4(C.byref(s), C.byref(dt) if dt else None, C.byref(bt) if bt else None, C.byref(opts), pp, n,
                       C.byref(out), threads)
    if pixels is None:
        h, w = scene.camera.height(), scene.camera.width()
        res = {k: v.reshape((h, w) + v.shape[1:]) for k, v in res.items()}
    return res


def max_threads() -> int:
    return load().orc_max_threads()
