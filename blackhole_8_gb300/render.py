"""Renderer: the Python face of the C ABI (the C++ face is
include/blackhole_gb300.hpp).

``Renderer.render`` is the drop-in for the reference's per-pixel render loop
(blackhole_solution_test.cc:161-298): it takes scenes built with the mirror
types of ``blackhole_8_gb300.scene`` and returns frames in host memory.
``render_device`` writes into caller-owned device buffers (torch tensors)
on a CUDA stream; ``sequence`` captures a fly-through as a CUDA graph.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .scene import Scene, Texture


def _check(lib, ctx, rc: int) -> None:
    if rc != capi.BH_OK:
        msg = lib.bh_last_error(ctx)
        raise capi.BhError(rc, msg.decode() if msg else "error")


@dataclass
class FrameBuffers:
    pixels: np.ndarray
    hit_class: np.ndarray | None = None
    aux: np.ndarray | None = None


class Renderer:
    """One CUDA device + stream (a bh_ctx). Not re-entrant across threads."""

    def __init__(self, device: int = 0):
        self.lib = capi.load()
        self.ctx = C.c_void_p()
        rc = self.lib.bh_create(C.byref(self.ctx), device)
        if rc != capi.BH_OK:
            raise capi.BhError(rc, "bh_create failed (no CUDA device?)")
        self._tex_ids: dict[int, int] = {}
        self._tex_refs: dict[int, Texture] = {}

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if self.ctx:
            self.lib.bh_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.bh_stream(self.ctx) or 0)

    # -- textures -------------------------------------------------------------
    def texture_id(self, tex: Texture) -> int:
        key = id(tex)
        if key not in self._tex_ids:
            out = C.c_int32()
            t = tex.texels
            rc = self.lib.bh_texture_create(self.ctx, t.ctypes.data_as(C.c_void_p), t.shape[1], t.shape[0],
                                            tex.layout, t.strides[0], C.byref(out))
            _check(self.lib, self.ctx, rc)
            self._tex_ids[key] = out.value
            self._tex_refs[key] = tex
        return self._tex_ids[key]

    def c_scenes(self, scenes: list[Scene]):
        for s in scenes:
            for t in s.textures():
                self.texture_id(t)
        arr = (capi.Scene * len(scenes))()
        keep = []
        for i, s in enumerate(scenes):
            c = s.to_c(self._tex_ids)
            arr[i] = c
            keep.append(c._keep)
        arr._keep = keep  # the object tables the scenes point at
        return arr

    # -- rendering ----------------------------------------------------------------
    def render(self, scenes: list[Scene], options: capi.RenderOptions | None = None,
               hit_class: bool = False, aux: bool = False) -> list[FrameBuffers]:
        """Renders into freshly allocated host arrays (synchronous)."""
        opts = options or capi.default_options()
        bpp = 3 if opts.format == capi.FORMAT_BGR8 else 4
        cs = self.c_scenes(scenes)
        out: list[FrameBuffers] = []
        frames = (capi.Frame * len(scenes))()
        for i, s in enumerate(scenes):
            h, w = s.camera.height(), s.camera.width()
            fb = FrameBuffers(np.zeros((h, w, bpp), dtype=np.uint8),
                              np.zeros((h, w), dtype=np.uint8) if hit_class else None,
                              np.zeros((h, w), dtype=np.float32) if aux else None)
            frames[i].pixels = fb.pixels.ctypes.data
            frames[i].hit_class = fb.hit_class.ctypes.data if hit_class else None
            frames[i].aux = fb.aux.ctypes.data if aux else None
            out.append(fb)
        rc = self.lib.bh_render(self.ctx, cs, len(scenes), frames, C.byref(opts))
        _check(self.lib, self.ctx, rc)
        return out

    def render_into(self, c_scenes, frames, options: capi.RenderOptions) -> None:
        """bh_render on prepared C arrays (host frames)."""
        rc = self.lib.bh_render(self.ctx, c_scenes, len(c_scenes), frames, C.byref(options))
        _check(self.lib, self.ctx, rc)

    def render_device(self, c_scenes, frames, options: capi.RenderOptions, stream: int | None = None) -> None:
        """bh_render_device: frames hold device pointers; asynchronous."""
        rc = self.lib.bh_render_device(self.ctx, c_scenes, len(c_scenes), frames, C.byref(options),
                                       C.c_void_p(stream) if stream else None)
        _check(self.lib, self.ctx, rc)

    def stats(self) -> capi.RenderStats:
        st = capi.RenderStats()
        _check(self.lib, self.ctx, self.lib.bh_get_stats(self.ctx, C.byref(st)))
        return st

    # -- sequences (CUDA graphs) ------------------------------------------------------
    def sequence(self, c_scenes, frames, options: capi.RenderOptions) -> "Sequence":
        h = C.c_void_p()
        rc = self.lib.bh_sequence_create(self.ctx, c_scenes, len(c_scenes), frames, C.byref(options), C.byref(h))
        _check(self.lib, self.ctx, rc)
        return Sequence(self, h, len(c_scenes))

    # -- autotuner ---------------------------------------------------------------------------
    def autotune(self, c_scenes, options: capi.RenderOptions | None = None, max_error: float = 1e-4,
                 cache_path: str | None = None) -> tuple[capi.RenderOptions, capi.TuneReport]:
        """bh_autotune: the mixed batched tracer's step and schedule for a batch."""
        opts = options or capi.default_options()
        out = capi.RenderOptions()
        C.memmove(C.byref(out), C.byref(opts), C.sizeof(out))
        rep = capi.TuneReport()
        rc = self.lib.bh_autotune(self.ctx, c_scenes, len(c_scenes), C.byref(out), max_error,
                                  cache_path.encode() if cache_path else None, C.byref(rep))
        _check(self.lib, self.ctx, rc)
        return out, rep

    # -- differentiable render -----------------------------------------------------------
    def render_adjoint(self, c_scenes, frames, theta=None,
                       options: capi.AdjointOptions | None = None) -> list[capi.AdjointResult]:
        """bh_render_adjoint: ``frames`` is a ctypes array of AdjointFrame with
        device pointers; ``theta`` an (n, 10) float64 array or None (each
        scene's own parameters). Returns loss and gradient per scene."""
        n = len(c_scenes)
        res = (capi.AdjointResult * n)()
        th = None
        if theta is not None:
            th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(n, capi.GRAD_COUNT))
        opts = options or capi.adjoint_options()
        rc = self.lib.bh_render_adjoint(self.ctx, c_scenes, n, th.ctypes.data if th is not None else None, frames,
                                        C.byref(opts), res)
        _check(self.lib, self.ctx, rc)
        return list(res)

    def scene_at_theta(self, c_scene: capi.Scene, theta) -> capi.Scene:
        """The scene moved to theta (bh_scene_at_theta)."""
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(capi.GRAD_COUNT))
        out = capi.Scene()
        _check(self.lib, self.ctx, self.lib.bh_scene_at_theta(C.byref(c_scene), th.ctypes.data, C.byref(out)))
        return out

    # -- probes ---------------------------------------------------------------------------
    def fp32_peak(self) -> tuple[float, int]:
        t = C.c_double()
        sms = C.c_int32()
        _check(self.lib, self.ctx, self.lib.bh_probe_fp32_peak(self.ctx, C.byref(t), C.byref(sms)))
        return t.value, sms.value

    def fp64_peak(self) -> float:
        t = C.c_double()
        _check(self.lib, self.ctx, self.lib.bh_probe_fp64_peak(self.ctx, C.byref(t)))
        return t.value


class Sequence:
    """A captured CUDA graph of one multi-frame render."""

    def __init__(self, renderer: Renderer, handle: C.c_void_p, n: int):
        self.r = renderer
        self.h = handle
        self.n = n

    def update(self, c_scenes) -> None:
        _check(self.r.lib, self.r.ctx, self.r.lib.bh_sequence_update(self.h, c_scenes, len(c_scenes)))

    def launch(self, stream: int | None = None) -> None:
        rc = self.r.lib.bh_sequence_launch(self.h, C.c_void_p(stream) if stream else None)
        _check(self.r.lib, self.r.ctx, rc)

    def stats(self) -> capi.RenderStats:
        st = capi.RenderStats()
        _check(self.r.lib, self.r.ctx, self.r.lib.bh_sequence_stats(self.h, C.byref(st)))
        return st

    def close(self) -> None:
        if self.h:
            self.r.lib.bh_sequence_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
