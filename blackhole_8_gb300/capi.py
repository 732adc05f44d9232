"""ctypes binding of the C ABI in include/bh_gb300.h.

The library is the in-tree ``_lib/libbh_gb300.so`` built by
``blackhole_8_gb300.build``. Loading fails loudly when it is missing: there is
no CPU fallback for the render.
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libbh_gb300.so")

BH_OK = 0
BH_ERR_INVALID_ARGUMENT = -1
BH_ERR_EMPTY_TEXTURE = -2
BH_ERR_BAD_TEXTURE = -3
BH_ERR_CUDA = -4
BH_ERR_OUT_OF_MEMORY = -5
BH_ERR_UNSUPPORTED = -6
BH_ERR_TIMEOUT = -7
BH_ERR_NO_DEVICE = -8
BH_ERR_DEVICE_FAULT = -9

INTEGRATOR_REF_TRAPEZOID, INTEGRATOR_RK4, INTEGRATOR_FLAT, INTEGRATOR_MULTI = 0, 1, 2, 3
PRECISION_FP32, PRECISION_FP64, PRECISION_MIXED = 0, 1, 2
RAYGEN_REF, RAYGEN_PINHOLE = 0, 1
DISC_MAP_REF_PLANAR, DISC_MAP_POLAR = 0, 1
FORMAT_BGRA8, FORMAT_BGR8, FORMAT_RGBA8 = 0, 1, 2
TEXEL_BGR8, TEXEL_RGB8, TEXEL_BGRA8, TEXEL_RGBA8 = 0, 1, 2, 3
SCHEDULE_GRID, SCHEDULE_PERSISTENT, SCHEDULE_HYBRID = 0, 1, 2
CLASS_MISS, CLASS_HORIZON, CLASS_DISC, CLASS_MAXSTEPS, CLASS_OBJECT = 0, 1, 2, 3, 4
OBJECT_RECTANGLE, OBJECT_TRIANGLE, OBJECT_PLANE = 1, 2, 3
MAX_OBJECTS = 64
MAX_HOLES = 8
ABI_VERSION = 3
RK4_ALGO_FLOPS_PER_STEP = 50  # BH_RK4_ALGO_FLOPS_PER_STEP: the roofline unit
RK4_FLOPS_PER_STEP = 26
RK4_INSTRUCTIONS_PER_STEP = 15

D3 = C.c_double * 3


class Camera(C.Structure):
    _fields_ = [("position", D3), ("axis_x", D3), ("axis_y", D3), ("axis_z", D3),
                ("focus_len", C.c_double), ("width", C.c_int32), ("height", C.c_int32)]


class Hole(C.Structure):
    _fields_ = [("position", D3), ("mass", C.c_double)]


class Disc(C.Structure):
    _fields_ = [("center", D3), ("normal", D3), ("corner", D3), ("edge_s1", D3), ("edge_s2", D3),
                ("r_inner", C.c_double), ("r_outer", C.c_double), ("texture", C.c_int32),
                ("mapping", C.c_int32), ("enabled", C.c_int32), ("reserved", C.c_int32)]


class Object(C.Structure):
    _fields_ = [("type", C.c_int32), ("texture", C.c_int32), ("v", D3 * 4), ("axis_x", D3), ("axis_y", D3),
                ("axis_z", D3), ("pattern_size", C.c_double)]


class Scene(C.Structure):
    _fields_ = [("camera", Camera), ("hole", Hole), ("disc", Disc), ("background", C.c_int32),
                ("n_objects", C.c_int32), ("objects", C.POINTER(Object)), ("n_extra_holes", C.c_int32),
                ("reserved_holes", C.c_int32), ("extra_holes", C.POINTER(Hole))]


class Frame(C.Structure):
    _fields_ = [("pixels", C.c_void_p), ("hit_class", C.c_void_p), ("aux", C.c_void_p)]


class RenderOptions(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("precision", C.c_int32), ("raygen", C.c_int32),
                ("format", C.c_int32), ("schedule", C.c_int32), ("max_steps", C.c_int32),
                ("step", C.c_double), ("r_escape", C.c_double), ("band", C.c_double),
                ("block_x", C.c_int32), ("block_y", C.c_int32), ("threads_per_block", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("refill_threshold", C.c_int32),
                ("band_step", C.c_double), ("setup_band", C.c_double), ("slice_steps", C.c_int32),
                ("band_lanes", C.c_int32), ("band_serial", C.c_int32), ("rays_per_thread", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class RenderStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("steps", C.c_uint64), ("band_rays", C.c_uint64),
                ("band_steps", C.c_uint64), ("band_overflow", C.c_uint64), ("flags", C.c_uint64),
                ("kernel_ms", C.c_double), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64)]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "bh_abi_version": (C.c_int, []),
    "bh_default_options": (None, [C.POINTER(RenderOptions)]),
    "bh_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "bh_destroy": (None, [C.c_void_p]),
    "bh_last_error": (C.c_char_p, [C.c_void_p]),
    "bh_stream": (C.c_void_p, [C.c_void_p]),
    "bh_texture_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                    C.POINTER(C.c_int32)]),
    "bh_texture_destroy": (C.c_int, [C.c_void_p, C.c_int32]),
    "bh_render": (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int32, C.POINTER(Frame),
                            C.POINTER(RenderOptions)]),
    "bh_render_device": (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int32, C.POINTER(Frame),
                                   C.POINTER(RenderOptions), C.c_void_p]),
    "bh_get_stats": (C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    "bh_sequence_create": (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int32, C.POINTER(Frame),
                                     C.POINTER(RenderOptions), C.POINTER(C.c_void_p)]),
    "bh_sequence_update": (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int32]),
    "bh_sequence_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "bh_sequence_destroy": (None, [C.c_void_p]),
    "bh_sequence_stats": (C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    "bh_probe_fp32_peak": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "bh_probe_fp64_peak": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with blackhole_8_gb300.build.build() "
                           "(there is no CPU fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class BhError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def default_options(**overrides) -> RenderOptions:
    o = RenderOptions()
    load().bh_default_options(C.byref(o))
    for k, v in overrides.items():
        if not hasattr(o, k):
            raise AttributeError(f"no render option {k!r}")
        setattr(o, k, v)
    return o


class DeviceTexture(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32)]


SIGNATURES["bh_render_noalloc"] = (C.c_int, [C.c_int, C.POINTER(Scene), C.c_int32, C.POINTER(DeviceTexture),
                                             C.c_int32, C.POINTER(Frame), C.POINTER(RenderOptions), C.c_void_p,
                                             C.c_char_p, C.c_int32])
NOALLOC_MAX_SCENES = 64
STATS_DIRECT_HOST = 256  # BH_STATS_DIRECT_HOST: bh_render's kernels wrote the frames into host memory
NOALLOC_MAX_RAYS = 4000000


class TuneReport(C.Structure):
    _fields_ = [("step", C.c_double), ("max_deflection", C.c_double), ("max_radius_error", C.c_double),
                ("class_mismatch", C.c_double), ("kernel_ms", C.c_double), ("candidates", C.c_int32),
                ("from_cache", C.c_int32)]


SIGNATURES["bh_autotune"] = (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int32, C.POINTER(RenderOptions),
                                       C.c_double, C.c_char_p, C.POINTER(TuneReport)])

# differentiable render and its adjoint
GRAD_MASS, GRAD_CAM_X, GRAD_CAM_Y, GRAD_CAM_Z, GRAD_YAW, GRAD_PITCH, GRAD_ROLL, GRAD_TILT, GRAD_R_INNER, \
    GRAD_R_OUTER = range(10)
GRAD_COUNT = 10
GRAD_NAMES = ("mass", "cam_x", "cam_y", "cam_z", "yaw", "pitch", "roll", "tilt", "r_inner", "r_outer")


class AdjointOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_steps", C.c_int32), ("step", C.c_double),
                ("r_escape", C.c_double), ("softness", C.c_double), ("band", C.c_double),
                ("checkpoint_every", C.c_int32), ("threads_per_block", C.c_int32), ("reserved", C.c_int32 * 8)]


class AdjointFrame(C.Structure):
    _fields_ = [("target", C.c_void_p), ("image", C.c_void_p), ("pixel_grad", C.c_void_p)]


class AdjointResult(C.Structure):
    _fields_ = [("loss", C.c_double), ("grad", C.c_double * GRAD_COUNT), ("steps", C.c_uint64),
                ("band_rays", C.c_uint64), ("kernel_ms", C.c_double)]


SIGNATURES["bh_adjoint_default_options"] = (None, [C.POINTER(AdjointOptions)])
SIGNATURES["bh_render_adjoint"] = (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int32, C.c_void_p,
                                             C.POINTER(AdjointFrame), C.POINTER(AdjointOptions),
                                             C.POINTER(AdjointResult)])
SIGNATURES["bh_scene_at_theta"] = (C.c_int, [C.POINTER(Scene), C.c_void_p, C.POINTER(Scene)])


def adjoint_options(**overrides) -> AdjointOptions:
    o = AdjointOptions()
    load().bh_adjoint_default_options(C.byref(o))
    for k, v in overrides.items():
        if not hasattr(o, k):
            raise AttributeError(f"no adjoint option {k!r}")
        setattr(o, k, v)
    return o
