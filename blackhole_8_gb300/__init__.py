"""GB300-native (sm_103a) Schwarzschild geodesic ray tracer.

A drop-in for the per-pixel geodesic render of lackhole/blackhole_8: the
reference's scene types (Camera, StaticBlackhole, Annulus, textures) on the
host, hand-written CUDA kernels behind the C ABI of include/bh_gb300.h.
"""
from . import capi, scene
from .scene import (Annulus, Camera, Object, Scene, StaticBlackhole, Texture, aimed_camera, batched_scenes,
                    equatorial_disc, flythrough, photon_ring_scene, single_scene)

__all__ = [
    "capi", "scene", "Annulus", "Camera", "Object", "Scene", "StaticBlackhole", "Texture", "aimed_camera",
    "batched_scenes", "equatorial_disc", "flythrough", "photon_ring_scene", "single_scene", "Renderer",
]


def __getattr__(name):
    if name in ("Renderer", "render"):
        from . import render
        return render.Renderer if name == "Renderer" else render
    raise AttributeError(name)
