"""bh_render_noalloc against the context entry point.

bh_render_noalloc is for callers that may not allocate device memory at
render time (a real-time frame loop with a fixed budget, a host that lends
the library only pre-allocated buffers). It keeps its scratch in a fixed
device array shared by all calls. Here two calls in a row, on scenes of
different sizes so the second finds the first's scratch contents left
behind, must each reproduce what bh_render gives for the same scenes and
options: the same kernels run on the same inputs, so the frames, classes
and deflections must be identical. Oversized calls must be refused.
"""
import ctypes as C

import numpy as np
import pytest

from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _device_textures(torch, textures):
    bufs = [torch.from_numpy(np.ascontiguousarray(t.bgra())).cuda() for t in textures]
    arr = (capi.DeviceTexture * len(bufs))()
    for i, b in enumerate(bufs):
        arr[i] = capi.DeviceTexture(b.data_ptr(), b.shape[1], b.shape[0])
    return bufs, arr


def _device_frames(torch, scenes):
    bufs, frames = [], (capi.Frame * len(scenes))()
    for i, s in enumerate(scenes):
        h, w = s.camera.height(), s.camera.width()
        px = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
        cl = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
        ax = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        bufs.append((px, cl, ax))
        frames[i] = capi.Frame(px.data_ptr(), cl.data_ptr(), ax.data_ptr())
    return bufs, frames


def test_noalloc_matches_context_entry_point(renderer):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    disc_tex, sky = S.standard_textures(0)
    tex_bufs, textures = _device_textures(torch, [disc_tex, sky])
    ids = {id(disc_tex): 0, id(sky): 1}
    opts = capi.default_options(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_PERSISTENT)
    calls = [S.flythrough(3, 320, 180), [S.single_scene(200, 120)]]
    err = C.create_string_buffer(512)
    for scenes in calls:  # two calls in a row
        cs = (capi.Scene * len(scenes))(*[s.to_c(ids) for s in scenes])
        bufs, frames = _device_frames(torch, scenes)
        rc = lib.bh_render_noalloc(0, cs, len(scenes), textures, len(tex_bufs), frames, C.byref(opts), None,
                                   err, len(err))
        assert rc == capi.BH_OK, err.value.decode()
        torch.cuda.synchronize()
        ref = renderer.render(scenes, opts, hit_class=True, aux=True)
        for (px, cl, ax), r in zip(bufs, ref):
            assert np.array_equal(px.cpu().numpy(), r.pixels)
            assert np.array_equal(cl.cpu().numpy(), r.hit_class)
            assert np.abs(ax.cpu().numpy() - r.aux).max() <= 1e-6


def test_noalloc_refuses_oversized_calls():
    lib = capi.load()
    err = C.create_string_buffer(512)
    big = S.flythrough(3, 1920, 1080)  # 3 x 2.07 M rays > BH_NOALLOC_MAX_RAYS
    ids = {id(big[0].disc.texture): 0, id(big[0].background): 1}
    cs = (capi.Scene * 3)(*[s.to_c(ids) for s in big])
    textures = (capi.DeviceTexture * 2)(capi.DeviceTexture(1, 1024, 64), capi.DeviceTexture(1, 2048, 1024))
    frames = (capi.Frame * 3)(*[capi.Frame(1, None, None) for _ in range(3)])
    rc = lib.bh_render_noalloc(0, cs, 3, textures, 2, frames, None, None, err, len(err))
    assert rc == capi.BH_ERR_INVALID_ARGUMENT
    assert b"no-alloc maximum" in err.value
    many = (capi.Scene * (capi.NOALLOC_MAX_SCENES + 1))()
    mframes = (capi.Frame * (capi.NOALLOC_MAX_SCENES + 1))()
    rc = lib.bh_render_noalloc(0, many, capi.NOALLOC_MAX_SCENES + 1, textures, 2, mframes, None, None, err,
                               len(err))
    assert rc == capi.BH_ERR_INVALID_ARGUMENT


def test_noalloc_refuses_several_holes():
    """The no-alloc entry traces one hole: the MULTI integrator and extra
    holes are refused before any device work (no GPU needed)."""
    lib = capi.load()
    err = C.create_string_buffer(512)
    sc = S.binary_scene(32, 18)
    ids = {id(sc.disc.texture): 0, id(sc.background): 1}
    textures = (capi.DeviceTexture * 2)(capi.DeviceTexture(1, 1024, 64), capi.DeviceTexture(1, 2048, 1024))
    frames = (capi.Frame * 1)(capi.Frame(1, None, None))
    cs = (capi.Scene * 1)(sc.to_c(ids))
    rc = lib.bh_render_noalloc(0, cs, 1, textures, 2, frames, None, None, err, len(err))
    assert rc == capi.BH_ERR_UNSUPPORTED and b"one hole" in err.value
    sc.extra_holes = []
    cs = (capi.Scene * 1)(sc.to_c(ids))
    opts = capi.default_options(integrator=capi.INTEGRATOR_MULTI)
    rc = lib.bh_render_noalloc(0, cs, 1, textures, 2, frames, C.byref(opts), None, err, len(err))
    assert rc == capi.BH_ERR_UNSUPPORTED and b"MULTI" in err.value
