"""bh_render_noalloc against the context entry point.

bh_render_noalloc is for callers that may not allocate device memory at
render time (a real-time frame loop with a fixed budget, a host that lends
the library only pre-allocated buffers). It keeps its scratch in a fixed
device array shared by all calls. Here two calls in a row, on scenes of
different sizes so the second finds the first's scratch contents left
behind, must each reproduce what bh_render gives for the same scenes and
options, for every schedule, precision and integrator the entry point
offers: the same kernels run on the same inputs, so the frames and classes
must be identical and the deflections equal to 1e-6 rad. Oversized calls
and the integrators it does not offer are refused before any device work,
which the CPU tests check.
"""
import ctypes as C

import numpy as np
import pytest

from blackhole_8_gb300 import build, capi
from blackhole_8_gb300 import scene as S


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def _device_textures(torch, textures):
    bufs = [torch.from_numpy(np.ascontiguousarray(t.bgra())).cuda() for t in textures]
    arr = (capi.DeviceTexture * len(bufs))()
    for i, b in enumerate(bufs):
        arr[i] = capi.DeviceTexture(b.data_ptr(), b.shape[1], b.shape[0])
    return bufs, arr


def _device_frames(torch, scenes, channels, with_aux):
    bufs, frames = [], (capi.Frame * len(scenes))()
    for i, s in enumerate(scenes):
        h, w = s.camera.height(), s.camera.width()
        px = torch.zeros((h, w, channels), dtype=torch.uint8, device="cuda")
        cl = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
        ax = torch.zeros((h, w), dtype=torch.float32, device="cuda") if with_aux else None
        bufs.append((px, cl, ax))
        frames[i] = capi.Frame(px.data_ptr(), cl.data_ptr(), ax.data_ptr() if with_aux else None)
    return bufs, frames


# (schedule, precision, integrator, raygen, format): every combination the
# entry point accepts, the pinhole camera and the drop-in BGR8 layout once each
CASES = [
    ("persistent-mixed", capi.SCHEDULE_PERSISTENT, capi.PRECISION_MIXED, capi.INTEGRATOR_RK4, capi.RAYGEN_REF,
     capi.FORMAT_BGRA8),
    ("persistent-fp32", capi.SCHEDULE_PERSISTENT, capi.PRECISION_FP32, capi.INTEGRATOR_RK4, capi.RAYGEN_REF,
     capi.FORMAT_BGRA8),
    ("hybrid-mixed-bgr8", capi.SCHEDULE_HYBRID, capi.PRECISION_MIXED, capi.INTEGRATOR_RK4, capi.RAYGEN_REF,
     capi.FORMAT_BGR8),
    ("grid-mixed", capi.SCHEDULE_GRID, capi.PRECISION_MIXED, capi.INTEGRATOR_RK4, capi.RAYGEN_REF,
     capi.FORMAT_BGRA8),
    ("grid-fp32", capi.SCHEDULE_GRID, capi.PRECISION_FP32, capi.INTEGRATOR_RK4, capi.RAYGEN_REF, capi.FORMAT_BGRA8),
    ("grid-fp64", capi.SCHEDULE_GRID, capi.PRECISION_FP64, capi.INTEGRATOR_RK4, capi.RAYGEN_REF, capi.FORMAT_BGRA8),
    ("grid-trapezoid-fp64-bgr8", capi.SCHEDULE_GRID, capi.PRECISION_FP64, capi.INTEGRATOR_REF_TRAPEZOID,
     capi.RAYGEN_REF, capi.FORMAT_BGR8),
    ("grid-trapezoid-fp32", capi.SCHEDULE_GRID, capi.PRECISION_FP32, capi.INTEGRATOR_REF_TRAPEZOID,
     capi.RAYGEN_REF, capi.FORMAT_BGRA8),
    ("grid-fp32-pinhole", capi.SCHEDULE_GRID, capi.PRECISION_FP32, capi.INTEGRATOR_RK4, capi.RAYGEN_PINHOLE,
     capi.FORMAT_BGRA8),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_context_entry_point(renderer, case):
    torch = pytest.importorskip("torch")
    _, schedule, precision, integrator, raygen, fmt = case
    lib = capi.load()
    disc_tex, sky = S.standard_textures(0)
    tex_bufs, textures = _device_textures(torch, [disc_tex, sky])
    ids = {id(disc_tex): 0, id(sky): 1}
    opts = capi.default_options(precision=precision, schedule=schedule, integrator=integrator, raygen=raygen,
                                format=fmt)
    rk4 = integrator == capi.INTEGRATOR_RK4
    channels = 3 if fmt == capi.FORMAT_BGR8 else 4
    calls = [S.flythrough(3, 320, 180), [S.single_scene(200, 120)]]
    err = C.create_string_buffer(512)
    for scenes in calls:  # two calls in a row
        if not rk4:
            for s in scenes:
                s.disc.mapping = capi.DISC_MAP_REF_PLANAR
        cs = (capi.Scene * len(scenes))(*[s.to_c(ids) for s in scenes])
        bufs, frames = _device_frames(torch, scenes, channels, with_aux=rk4)
        rc = lib.bh_render_noalloc(0, cs, len(scenes), textures, len(tex_bufs), frames, C.byref(opts), None,
                                   err, len(err))
        assert rc == capi.BH_OK, err.value.decode()
        torch.cuda.synchronize()
        ref = renderer.render(scenes, opts, hit_class=True, aux=rk4)
        for (px, cl, ax), r in zip(bufs, ref):
            assert np.array_equal(px.cpu().numpy(), r.pixels)
            assert np.array_equal(cl.cpu().numpy(), r.hit_class)
            if rk4:
                assert np.abs(ax.cpu().numpy() - r.aux).max() <= 1e-6


@pytest.mark.gpu
def test_noalloc_refuses_a_capturing_stream():
    """A call made while its stream captures a CUDA graph is refused before
    any device work: the copy it would record reads the entry point's static
    host array of scene records, which later calls rewrite before a replay."""
    torch = pytest.importorskip("torch")
    lib = capi.load()
    disc_tex, sky = S.standard_textures(0)
    tex_bufs, textures = _device_textures(torch, [disc_tex, sky])
    scenes = [S.single_scene(64, 36)]
    ids = {id(disc_tex): 0, id(sky): 1}
    cs = (capi.Scene * 1)(*[s.to_c(ids) for s in scenes])
    bufs, frames = _device_frames(torch, scenes, 4, with_aux=False)
    torch.cuda.synchronize()
    err = C.create_string_buffer(512)
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        graph.capture_begin()
        try:
            rc = lib.bh_render_noalloc(0, cs, 1, textures, len(tex_bufs), frames, None, side.cuda_stream, err,
                                       len(err))
        finally:
            graph.capture_end()
    assert rc == capi.BH_ERR_UNSUPPORTED, err.value
    assert b"capturing" in err.value
    # the refusal left the stream and the entry point usable
    rc = lib.bh_render_noalloc(0, cs, 1, textures, len(tex_bufs), frames, None, None, err, len(err))
    assert rc == capi.BH_OK, err.value.decode()
    torch.cuda.synchronize()
    assert int(bufs[0][1].max().item()) > 0  # classes were written


def _textures_and_frames(n):
    # placeholders: these calls are refused before any pointer is used
    textures = (capi.DeviceTexture * 2)(capi.DeviceTexture(1, 1024, 64), capi.DeviceTexture(1, 2048, 1024))
    frames = (capi.Frame * n)(*[capi.Frame(1, None, None) for _ in range(n)])
    return textures, frames


def test_noalloc_refuses_oversized_calls(lib):
    err = C.create_string_buffer(512)
    big = S.flythrough(3, 1920, 1080)  # 3 x 2.07 M rays > BH_NOALLOC_MAX_RAYS
    ids = {id(big[0].disc.texture): 0, id(big[0].background): 1}
    cs = (capi.Scene * 3)(*[s.to_c(ids) for s in big])
    textures, frames = _textures_and_frames(3)
    rc = lib.bh_render_noalloc(0, cs, 3, textures, 2, frames, None, None, err, len(err))
    assert rc == capi.BH_ERR_INVALID_ARGUMENT
    assert b"no-alloc maximum" in err.value
    many = (capi.Scene * (capi.NOALLOC_MAX_SCENES + 1))()
    mframes = (capi.Frame * (capi.NOALLOC_MAX_SCENES + 1))()
    rc = lib.bh_render_noalloc(0, many, capi.NOALLOC_MAX_SCENES + 1, textures, 2, mframes, None, None, err,
                               len(err))
    assert rc == capi.BH_ERR_INVALID_ARGUMENT


def test_noalloc_refuses_several_holes(lib):
    """The no-alloc entry traces one hole: the MULTI integrator and extra
    holes are refused before any device work."""
    err = C.create_string_buffer(512)
    sc = S.binary_scene(32, 18)
    ids = {id(sc.disc.texture): 0, id(sc.background): 1}
    textures, frames = _textures_and_frames(1)
    cs = (capi.Scene * 1)(sc.to_c(ids))
    rc = lib.bh_render_noalloc(0, cs, 1, textures, 2, frames, None, None, err, len(err))
    assert rc == capi.BH_ERR_UNSUPPORTED and b"one hole" in err.value
    sc.extra_holes = []
    cs = (capi.Scene * 1)(sc.to_c(ids))
    opts = capi.default_options(integrator=capi.INTEGRATOR_MULTI)
    rc = lib.bh_render_noalloc(0, cs, 1, textures, 2, frames, C.byref(opts), None, err, len(err))
    assert rc == capi.BH_ERR_UNSUPPORTED and b"MULTI" in err.value


@pytest.mark.parametrize("bad", [{"band": float("inf")}, {"setup_band": float("inf")}, {"band": float("nan")},
                                 {"step": 0.0 - 1}, {"slice_steps": 2}, {"block_x": 7, "block_y": 1},
                                 {"rays_per_thread": 129}, {"rays_per_thread": -1}, {"schedule": 3},
                                 {"threads_per_block": 512}, {"threads_per_block": 544, "schedule": capi.SCHEDULE_HYBRID,
                                                              "precision": capi.PRECISION_MIXED}])
def test_noalloc_refuses_the_options_bh_render_refuses(lib, bad):
    """The option checks are the context entry points' own: non-finite bands
    and out-of-range values are refused with the same status."""
    err = C.create_string_buffer(512)
    sc = S.single_scene(32, 18)
    ids = {id(sc.disc.texture): 0, id(sc.background): 1}
    textures, frames = _textures_and_frames(1)
    cs = (capi.Scene * 1)(sc.to_c(ids))
    opts = capi.default_options(**bad)
    rc = lib.bh_render_noalloc(0, cs, 1, textures, 2, frames, C.byref(opts), None, err, len(err))
    assert rc == capi.BH_ERR_INVALID_ARGUMENT, err.value


@pytest.mark.parametrize("bad", [{"schedule": capi.SCHEDULE_HYBRID, "precision": capi.PRECISION_FP64},
                                 {"schedule": capi.SCHEDULE_HYBRID, "integrator": capi.INTEGRATOR_REF_TRAPEZOID}])
def test_noalloc_refuses_unsupported_schedules(lib, bad):
    """The hybrid schedule runs the RK4 tracer in FP32 or MIXED: other
    combinations are refused as unsupported before any device work."""
    err = C.create_string_buffer(512)
    sc = S.single_scene(32, 18)
    ids = {id(sc.disc.texture): 0, id(sc.background): 1}
    textures, frames = _textures_and_frames(1)
    cs = (capi.Scene * 1)(sc.to_c(ids))
    opts = capi.default_options(**bad)
    rc = lib.bh_render_noalloc(0, cs, 1, textures, 2, frames, C.byref(opts), None, err, len(err))
    assert rc == capi.BH_ERR_UNSUPPORTED, err.value
