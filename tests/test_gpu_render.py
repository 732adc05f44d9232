"""GPU parity: the sm_103a tracer through the C ABI against the FP64 oracle
and against the reference's own render (golden fixtures).

Bars (the tolerances are written in each test):
- trapezoid (reference scheme), FP64: hit classes equal to the reference's
  except on class boundaries; colours equal except where a texel-edge tie
  rounds the other way.
- RK4 FP64: classes and deflections equal to the FP64 oracle to rounding.
- RK4 FP32 / MIXED: hit class agrees on >= 99.9 % of pixels and the rest lie
  on class boundaries; colour within 1 LSB away from texel and disc edges;
  deflection within 1e-4 rad of the FP64 oracle (MIXED: every escaped ray;
  FP32: rays outside the band around 3 sqrt(3) M).
"""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

import helpers
from parity import boundary_pixels, compare, dilate, sample_check
from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S
from oracle import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(GOLDEN, "index.json")))["cases"]
B_C = 3.0 * math.sqrt(3.0)


def opts(**kw):
    return capi.default_options(**kw)


# ---------------------------------------------------------------------------
# the reference's trapezoid scheme
@pytest.mark.parametrize("case", CASES, ids=lambda c: c["file"])
def test_trapezoid_fp64_matches_reference(renderer, case):
    """The reference's curved loop (or, for flat cases, its RayTracer) in
    FP64 on the GPU against the reference's own output: hit classes agree on
    >= 99.9 % of pixels and differ only on class boundaries; where the
    classes agree, colours are within 1 LSB except where the oracle's
    sampling coordinate lies within 1e-6 texels of a texel edge (a tie that
    FP64 rounding of the hit point decides)."""
    sc = helpers.build(case["builder"], case["width"], case["height"])
    g = np.load(os.path.join(GOLDEN, case["file"]))
    flat = case.get("mode") == "flat"
    integ = capi.INTEGRATOR_FLAT if flat else capi.INTEGRATOR_REF_TRAPEZOID
    o = opts(integrator=integ, precision=capi.PRECISION_FP64, format=capi.FORMAT_BGR8)
    out = renderer.render([sc], o, hit_class=True, aux=flat)[0]
    margin = (oracle.render_flat(sc) if flat else oracle.render_ref(sc))["margin_tex"]
    boundary = dilate(helpers.class_boundary_mask(g["cls"]))
    if flat:
        idx = np.where(out.hit_class == capi.CLASS_OBJECT, out.aux, -1).astype(np.int32)
        assert (idx != g["obj"]).mean() <= 1e-3 and not ((idx != g["obj"]) & ~boundary).any()
    bad = out.hit_class != g["cls"]
    assert bad.mean() <= 1e-3 and not (bad & ~boundary).any()
    tie = margin < helpers.TEXEL_TIE_FP64
    dl = helpers.colour_lsb(out.pixels, g["bgr"])
    strict = ~bad & ~tie
    assert dl[strict].max(initial=0) <= 1, f"{(dl[strict] > 1).sum()} pixels differ away from texel edges"


def test_trapezoid_fp32_matches_oracle(renderer):
    """The reference's scheme in FP32 against the FP64 oracle: classes agree
    on >= 99.5 % of pixels, the rest within two pixels of a class boundary;
    colours within 1 LSB where the classes agree and the sampling coordinate
    lies 1e-3 texels or more from a texel edge (FP32 rounding of the hit
    point is ~1e-4 texels)."""
    sc = helpers.cfg0_planar(160, 90)
    ref = oracle.render_ref(sc)
    o = opts(integrator=capi.INTEGRATOR_REF_TRAPEZOID, precision=capi.PRECISION_FP32)
    out = renderer.render([sc], o, hit_class=True)[0]
    bad = out.hit_class != ref["cls"]
    assert bad.mean() <= 5e-3
    assert not (bad & ~dilate(helpers.class_boundary_mask(ref["cls"]), 2)).any()
    strict = ~bad & (ref["margin_tex"] >= 1e-3) & ~dilate(helpers.class_boundary_mask(ref["cls"]), 2)
    assert helpers.colour_lsb(out.pixels, ref["bgra"])[strict].max(initial=0) <= 1


# ---------------------------------------------------------------------------
# RK4
@pytest.fixture(scope="module")
def single():
    sc = S.single_scene(320, 180)
    return sc, oracle.render_rk4(sc)


def test_rk4_fp64_matches_oracle(renderer, single):
    sc, o = single
    out = renderer.render([sc], opts(precision=capi.PRECISION_FP64), hit_class=True, aux=True)[0]
    boundary = boundary_pixels(o, band=1e-6, tex=1e-6, edge=1e-9)
    e1, e2 = compare(out, o, boundary, aux_tol=1e-6)
    assert (out.hit_class == o["cls"]).mean() >= 0.9999


def test_rk4_fp32_matches_oracle(renderer, single):
    sc, o = single
    out = renderer.render([sc], opts(precision=capi.PRECISION_FP32), hit_class=True, aux=True)[0]
    # plain FP32 meets 1e-4 rad outside |b - b_c| < 0.1 M (no FP64, no projection)
    compare(out, o, boundary_pixels(o, band=0.1), aux_tol=1e-4)


@pytest.mark.parametrize("schedule", [capi.SCHEDULE_GRID, capi.SCHEDULE_PERSISTENT, capi.SCHEDULE_HYBRID])
def test_rk4_mixed_meets_bound_on_every_escaped_ray(renderer, single, schedule):
    sc, o = single
    out = renderer.render([sc], opts(precision=capi.PRECISION_MIXED, schedule=schedule, rays_per_thread=4),
                          hit_class=True, aux=True)[0]
    st = renderer.stats()
    assert st.rays == 320 * 180
    assert st.band_overflow == 0
    # near the critical impact parameter only the class itself may flip
    compare(out, o, boundary_pixels(o, band=1e-4), aux_tol=1e-4)


def test_hybrid_matches_persistent(renderer, single):
    """The hybrid schedule traces every ray with the persistent schedule's
    per-ray code (FP32 pass on a grid, the same FP64 band pass): the same
    rays go to the band, and the images agree up to the compiler's
    multiply-add contraction in the two FP32 kernels."""
    sc, _ = single
    a = renderer.render([sc], opts(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_PERSISTENT),
                        hit_class=True, aux=True)[0]
    sa = renderer.stats()
    b = renderer.render([sc], opts(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_HYBRID, rays_per_thread=4),
                        hit_class=True, aux=True)[0]
    sb = renderer.stats()
    assert (sa.rays, sa.band_rays, sa.band_steps) == (sb.rays, sb.band_rays, sb.band_steps)
    assert (a.hit_class == b.hit_class).mean() >= 0.9999
    assert (a.pixels != b.pixels).any(-1).mean() <= 1e-3
    assert np.quantile(np.abs(a.aux - b.aux), 0.999) <= 1e-5
    assert abs(int(sa.steps) - int(sb.steps)) <= 1e-4 * sa.steps


def test_persistent_matches_grid(renderer, single):
    sc, _ = single
    a = renderer.render([sc], opts(schedule=capi.SCHEDULE_GRID), hit_class=True, aux=True)[0]
    sa = renderer.stats()
    b = renderer.render([sc], opts(schedule=capi.SCHEDULE_PERSISTENT), hit_class=True, aux=True)[0]
    sb = renderer.stats()
    # same per-ray arithmetic; the compiler may contract a multiply-add
    # differently in the two kernels, which only shows near b_c
    assert (a.hit_class == b.hit_class).mean() >= 0.9999
    assert (a.pixels != b.pixels).any(-1).mean() <= 1e-3
    assert np.quantile(np.abs(a.aux - b.aux), 0.999) <= 1e-5
    assert sa.rays == sb.rays and abs(int(sa.steps) - int(sb.steps)) <= 1e-4 * sa.steps


@pytest.mark.parametrize("precision,integrator", [(capi.PRECISION_MIXED, capi.INTEGRATOR_RK4),
                                                  (capi.PRECISION_FP32, capi.INTEGRATOR_RK4),
                                                  (capi.PRECISION_FP64, capi.INTEGRATOR_REF_TRAPEZOID)],
                         ids=["mixed", "fp32", "trapezoid-fp64"])
def test_grid_shape_and_rays_per_thread_change_nothing(renderer, precision, integrator):
    """The GRID schedule's block shape and rays per thread only change which
    thread traces a pixel: frames, classes and counters are identical (two
    frames of different sizes, so that block tiles overhang the images)."""
    scenes = [S.single_scene(200, 117), S.flythrough(3, 150, 83)[1]]
    ref, ref_st = None, None
    for bx, by, rpt in [(8, 16, 1), (8, 16, 2), (16, 8, 4), (32, 4, 3), (8, 8, 8), (16, 16, 1), (8, 16, 64),
                        (32, 4, 128)]:
        o = opts(precision=precision, integrator=integrator, block_x=bx, block_y=by, rays_per_thread=rpt)
        out = renderer.render(scenes, o, hit_class=True)
        st = renderer.stats()
        if ref is None:
            ref, ref_st = out, st
            continue
        for a, b in zip(ref, out):
            assert np.array_equal(a.pixels, b.pixels) and np.array_equal(a.hit_class, b.hit_class), (bx, by, rpt)
        assert (st.rays, st.steps, st.band_rays, st.band_steps) == \
            (ref_st.rays, ref_st.steps, ref_st.band_rays, ref_st.band_steps), (bx, by, rpt)
    assert ref_st.rays == 200 * 117 + 150 * 83


def test_step_counts_match_oracle(renderer):
    sc = S.single_scene(96, 54)
    o = oracle.render_rk4(sc)
    renderer.render([sc], opts(precision=capi.PRECISION_FP64))
    st = renderer.stats()
    assert st.rays == 96 * 54
    assert abs(int(st.steps) - int(o["steps"].sum())) <= 2


@pytest.mark.parametrize("schedule,precision,bx,by", [
    (capi.SCHEDULE_PERSISTENT, capi.PRECISION_MIXED, 8, 16), (capi.SCHEDULE_PERSISTENT, capi.PRECISION_FP32, 8, 16),
    (capi.SCHEDULE_GRID, capi.PRECISION_FP32, 8, 16), (capi.SCHEDULE_GRID, capi.PRECISION_FP32, 16, 8),
    (capi.SCHEDULE_GRID, capi.PRECISION_MIXED, 32, 4), (capi.SCHEDULE_GRID, capi.PRECISION_FP32, 4, 8),
    (capi.SCHEDULE_GRID, capi.PRECISION_FP32, 64, 2), (capi.SCHEDULE_GRID, capi.PRECISION_FP32, 12, 8)],
    ids=["persistent-mixed", "persistent-fp32", "grid-8x16", "grid-16x8", "grid-mixed-32x4", "grid-4x8",
         "grid-64x2", "grid-12x8"])
def test_bgr8_frames_equal_bgra8(renderer, schedule, precision, bx, by):
    """BGR8 (CV_8UC3) frames, which whole warps write as packed 32-bit words
    where the frame width allows it and byte by byte elsewhere, hold exactly
    the BGRA8 frame's first three channels: widths that are multiples of 4
    (packed) and not (bytes), image edges, several block shapes (12-wide
    blocks do not map warps to rows and always take the byte path)."""
    scenes = [S.single_scene(200, 117), S.flythrough(3, 150, 83)[1], S.single_scene(64, 36)]
    o = opts(schedule=schedule, precision=precision, block_x=bx, block_y=by, format=capi.FORMAT_BGRA8)
    a = renderer.render(scenes, o, hit_class=True)
    o.format = capi.FORMAT_BGR8
    b = renderer.render(scenes, o, hit_class=True)
    for fa, fb in zip(a, b):
        assert np.array_equal(fa.pixels[..., :3], fb.pixels)
        assert np.array_equal(fa.hit_class, fb.hit_class)


def test_pixel_formats_agree(renderer):
    sc = S.single_scene(64, 36)
    a = renderer.render([sc], opts(format=capi.FORMAT_BGRA8))[0].pixels
    b = renderer.render([sc], opts(format=capi.FORMAT_BGR8))[0].pixels
    c = renderer.render([sc], opts(format=capi.FORMAT_RGBA8))[0].pixels
    assert np.array_equal(a[..., :3], b)
    assert np.array_equal(a[..., 2::-1], c[..., :3])
    assert (a[..., 3] == 255).all()


def test_pinhole_raygen_differs_from_ref(renderer):
    sc = S.single_scene(64, 36)
    a = renderer.render([sc], opts(raygen=capi.RAYGEN_REF), hit_class=True)[0].hit_class
    b = renderer.render([sc], opts(raygen=capi.RAYGEN_PINHOLE), hit_class=True)[0].hit_class
    assert (a != b).any()


@pytest.mark.parametrize("precision,schedule", [(capi.PRECISION_FP64, capi.SCHEDULE_GRID),
                                                (capi.PRECISION_FP32, capi.SCHEDULE_GRID),
                                                (capi.PRECISION_MIXED, capi.SCHEDULE_GRID),
                                                (capi.PRECISION_MIXED, capi.SCHEDULE_PERSISTENT),
                                                (capi.PRECISION_MIXED, capi.SCHEDULE_HYBRID)],
                         ids=["fp64", "fp32", "mixed-grid", "mixed-persistent", "mixed-hybrid"])
def test_cfg0_full_size(renderer, precision, schedule):
    """The single-scene workload at its own 640x360 against the FP64 oracle,
    every pixel: FP64 to rounding, MIXED within 1e-4 rad on every escaped
    ray, plain FP32 within 1e-4 rad outside |b - b_c| < 0.1 M."""
    sc = S.single_scene(640, 360)
    o = oracle.render_rk4(sc)
    out = renderer.render([sc], opts(precision=precision, schedule=schedule, rays_per_thread=4), hit_class=True,
                          aux=True)[0]
    if precision == capi.PRECISION_FP64:
        compare(out, o, boundary_pixels(o, band=1e-6, tex=1e-6, edge=1e-9), aux_tol=1e-6)
    elif precision == capi.PRECISION_FP32:
        compare(out, o, boundary_pixels(o, band=0.1), aux_tol=1e-4)
    else:
        compare(out, o, boundary_pixels(o, band=1e-4), aux_tol=1e-4)


@pytest.mark.parametrize("step", [0.01, 0.1])
def test_full_hd_frames_sampled_against_oracle(renderer, step):
    """Full-size 1920x1080 fly-through frames through the mixed tracer on the
    persistent schedule, at the oracle's step and at the step the autotuner
    picks for the fly-through; 4000 seeded pixels of each frame against the
    FP64 oracle (step 0.01) with the full parity bar (hit radius within
    2e-3 M at step 0.1)."""
    scenes = S.flythrough(120)
    picks = [scenes[0], scenes[39], scenes[79], scenes[119]]
    out = renderer.render(picks, opts(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_PERSISTENT, step=step),
                          hit_class=True, aux=True)
    rng = np.random.default_rng(11)
    for sc, fb in zip(picks, out):
        xs = rng.integers(0, 1920, 4000)
        ys = rng.integers(0, 1080, 4000)
        o = oracle.render_rk4(sc, pixels=np.stack([xs, ys], 1))
        sample_check(sc, xs, ys, fb.hit_class[ys, xs], fb.pixels[ys, xs], fb.aux[ys, xs], o, {},
                     radius_tol=1e-3 if step <= 0.01 else 2e-3)


def test_batched_uneven_scenes(renderer):
    """Uneven scenes (sides 32-160, each its own M, camera, disc and sky) in
    one persistent mixed-precision launch: every scene against the FP64
    oracle, every pixel, with the full parity bar over the batch (class
    agreement counted over all its pixels)."""
    scenes = S.batched_scenes(24, seed=3, min_side=32, max_side=160, bg_size=(256, 128))
    out = renderer.render(scenes, opts(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_PERSISTENT),
                          hit_class=True, aux=True)
    st = renderer.stats()
    assert st.rays == sum(s.camera.width() * s.camera.height() for s in scenes)
    agree = total = 0
    for sc, fb in zip(scenes, out):
        o = oracle.render_rk4(sc)
        cls_ok = fb.hit_class == o["cls"]
        agree += int(cls_ok.sum())
        total += cls_ok.size
        bnd = boundary_pixels(o, band=1e-4)
        assert not (~cls_ok & ~bnd).any(), sc.meta
        strict = cls_ok & ~bnd
        assert helpers.colour_lsb(fb.pixels, o["bgra"])[strict].max(initial=0) <= 1, sc.meta
        esc = strict & (o["cls"] == capi.CLASS_MISS)
        dsk = strict & (o["cls"] == capi.CLASS_DISC)
        assert np.abs(fb.aux[esc] - o["aux"][esc]).max(initial=0) <= 1e-4, sc.meta
        # the hit radius, in units of the scene's M
        assert np.abs(fb.aux[dsk] - o["aux"][dsk]).max(initial=0) <= 1e-3, sc.meta
    assert agree / total >= 0.999


@pytest.mark.parametrize("schedule", [capi.SCHEDULE_PERSISTENT, capi.SCHEDULE_HYBRID])
@pytest.mark.parametrize("band", [2e-5, 5e-4, 0.05, 0.2])
def test_mixed_band_order_is_bit_exact(renderer, band, schedule):
    """The FP64 band pass beside the FP32 pass (it launches the FP32 pass
    from the device) and the serial orders (both passes launched by the host:
    the FP32 pass first, or the FP64 pass first with the FP32 pass as the
    host's one-wave launch looping over the frame blocks, the path that runs
    when a device-side launch fails) trace every ray with the same code:
    frames, classes, deflections and counters equal, and no device-side
    launch failed. Every pixel is traced exactly once: the classification
    (32-pixel row segments, skipped by a bound on b along the row) lists
    exactly the rays the FP32 pass leaves out, also when the band is wider
    than setup_band (0.1 M)."""
    scenes = S.flythrough(4, 160, 90) + S.flythrough(120, 320, 180)[60:64]
    pixels = sum(s.camera.width() * s.camera.height() for s in scenes)
    res = []
    for serial in (0, 1, 2):
        o = opts(precision=capi.PRECISION_MIXED, schedule=schedule, band=band, band_serial=serial, rays_per_thread=3)
        res.append((renderer.render(scenes, o, hit_class=True, aux=True), renderer.stats()))
    a, sa = res[0]
    for b, sb in res[1:]:
        for fa, fb in zip(a, b):
            assert np.array_equal(fa.pixels, fb.pixels)
            assert np.array_equal(fa.hit_class, fb.hit_class)
            assert np.array_equal(fa.aux.view(np.uint32), fb.aux.view(np.uint32))
        assert (sa.rays, sa.steps, sa.band_rays, sa.band_steps) == (sb.rays, sb.steps, sb.band_rays, sb.band_steps)
        assert sb.flags == 0
    assert sa.rays == pixels
    if band >= 0.05:
        assert sa.band_rays > 0
    assert sa.flags == 0
    # the same frames through the grid schedule, which tests the band inline
    g = renderer.render(scenes, opts(precision=capi.PRECISION_MIXED, band=band), hit_class=True)
    for fa, fg in zip(a, g):
        assert (fa.hit_class == fg.hit_class).mean() >= 0.999


# ---------------------------------------------------------------------------
# device buffers and captured sequences
def _device_frames(torch, scenes, with_cls=True):
    bufs, frames = [], (capi.Frame * len(scenes))()
    for i, s in enumerate(scenes):
        px = torch.zeros((s.camera.height(), s.camera.width(), 4), dtype=torch.uint8, device="cuda")
        cl = torch.zeros((s.camera.height(), s.camera.width()), dtype=torch.uint8, device="cuda")
        bufs.append((px, cl))
        frames[i].pixels = px.data_ptr()
        frames[i].hit_class = cl.data_ptr() if with_cls else None
        frames[i].aux = None
    return bufs, frames


@pytest.mark.parametrize("schedule", [capi.SCHEDULE_PERSISTENT, capi.SCHEDULE_HYBRID])
def test_sequence_graph_matches_direct_render(renderer, schedule):
    torch = pytest.importorskip("torch")
    scenes = S.flythrough(6, 96, 54)
    o = opts(precision=capi.PRECISION_MIXED, schedule=schedule, rays_per_thread=2)
    bufs, frames = _device_frames(torch, scenes)
    seq = renderer.sequence(renderer.c_scenes(scenes), frames, o)
    seq.launch()
    torch.cuda.synchronize()
    renderer.stats()
    direct = renderer.render(scenes, o, hit_class=True)
    for (px, cl), d in zip(bufs, direct):
        assert np.array_equal(px.cpu().numpy(), d.pixels)
        assert np.array_equal(cl.cpu().numpy(), d.hit_class)
    # new poses, same sizes: update and replay
    later = S.flythrough(12, 96, 54)[6:]
    seq.update(renderer.c_scenes(later))
    seq.launch()
    torch.cuda.synchronize()
    direct = renderer.render(later, o, hit_class=True)
    for (px, cl), d in zip(bufs, direct):
        assert np.array_equal(px.cpu().numpy(), d.pixels)
    seq.close()


def test_host_render_in_chunks_matches_device_render(renderer):
    """bh_render of more than 64 M pixels over >= 8 scenes renders in chunks
    whose copy-back overlaps the next chunk: frames equal the device render
    and the statistics cover every chunk."""
    torch = pytest.importorskip("torch")
    scenes = S.flythrough(8, 2900, 2900)
    o = opts(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_PERSISTENT, step=0.1)
    host = renderer.render(scenes, o)
    st = renderer.stats()
    assert st.rays == 8 * 2900 * 2900 and st.flags == 0
    assert st.d2h_bytes == 8 * 2900 * 2900 * 4
    bufs, frames = _device_frames(torch, scenes, with_cls=False)
    renderer.render_device(renderer.c_scenes(scenes), frames, o)
    torch.cuda.synchronize()
    sd = renderer.stats()
    assert (sd.rays, sd.steps, sd.band_rays) == (st.rays, st.steps, st.band_rays)
    for (px, _), h in zip(bufs, host):
        assert np.array_equal(px.cpu().numpy(), h.pixels)


@pytest.mark.parametrize("schedule,fmt,rpt,band,precision", [
    (capi.SCHEDULE_HYBRID, capi.FORMAT_BGR8, 4, 5e-4, capi.PRECISION_MIXED),
    (capi.SCHEDULE_HYBRID, capi.FORMAT_BGR8, 8, 0.05, capi.PRECISION_MIXED),
    (capi.SCHEDULE_HYBRID, capi.FORMAT_BGR8, 2, 5e-4, capi.PRECISION_MIXED),
    (capi.SCHEDULE_HYBRID, capi.FORMAT_BGRA8, 4, 5e-4, capi.PRECISION_MIXED),
    (capi.SCHEDULE_GRID, capi.FORMAT_BGR8, 4, 5e-4, capi.PRECISION_MIXED),
    (capi.SCHEDULE_GRID, capi.FORMAT_BGR8, 4, 5e-4, capi.PRECISION_FP32),
    (capi.SCHEDULE_PERSISTENT, capi.FORMAT_BGR8, 1, 5e-4, capi.PRECISION_MIXED)],
    ids=["hybrid-bgr8", "hybrid-bgr8-r8-band0.05", "hybrid-bgr8-r2", "hybrid-bgra8", "grid-bgr8", "grid-fp32-bgr8",
         "persistent-bgr8"])
def test_bh_render_writes_pinned_host_frames_directly(renderer, schedule, fmt, rpt, band, precision):
    """bh_render into page-locked host frames: on the GRID and HYBRID
    schedules the kernels write them directly (stats flag, no device copy;
    BGR8 rows go out as packed 32-bit words, one 32-pixel row segment per
    warp), on the persistent schedule the frames are copied back as for
    pageable memory; either way the frames, classes and deflections equal those of
    the render into pageable host memory, and d2h_bytes counts every byte of
    every buffer. Frame widths: multiples of 32, of 4 only (block rows partly
    outside the frame) and of neither (rows not 4-byte aligned: pixel
    stores); a wide band leaves many tiles with pixels the FP64 pass writes."""
    torch = pytest.importorskip("torch")
    scenes = S.flythrough(3, 320, 180) + [S.single_scene(200, 117), S.flythrough(3, 150, 83)[1]]
    o = opts(precision=precision, schedule=schedule, format=fmt, rays_per_thread=rpt, band=band)
    ref = renderer.render(scenes, o, hit_class=True, aux=True)
    assert not renderer.stats().flags & capi.STATS_DIRECT_HOST
    bpp = 3 if fmt == capi.FORMAT_BGR8 else 4
    bufs, frames = [], (capi.Frame * len(scenes))()
    for i, s in enumerate(scenes):
        h, w = s.camera.height(), s.camera.width()
        px = torch.zeros((h, w, bpp), dtype=torch.uint8).pin_memory()
        cl = torch.zeros((h, w), dtype=torch.uint8).pin_memory()
        ax = torch.zeros((h, w), dtype=torch.float32).pin_memory()
        bufs.append((px, cl, ax))
        frames[i] = capi.Frame(px.data_ptr(), cl.data_ptr(), ax.data_ptr())
    renderer.render_into(renderer.c_scenes(scenes), frames, o)
    st = renderer.stats()
    direct = bool(st.flags & capi.STATS_DIRECT_HOST)
    assert direct == (schedule != capi.SCHEDULE_PERSISTENT)
    assert st.d2h_bytes == sum(s.camera.width() * s.camera.height() * (bpp + 1 + 4) for s in scenes)
    for (px, cl, ax), r in zip(bufs, ref):
        assert np.array_equal(px.numpy(), r.pixels)
        assert np.array_equal(cl.numpy(), r.hit_class)
        assert np.array_equal(ax.numpy().view(np.uint32), r.aux.view(np.uint32))


@pytest.mark.parametrize("band_serial", [0, 1, 2])
def test_bgr8_32_wide_blocks_match_8_wide(renderer, band_serial):
    """BGR8 frames in 32 x 4 blocks (each warp stores one 96-byte row
    segment as packed words) against 8 x 16 blocks (packed rows of 8 pixels):
    the same pixels and classes, for the FP32 pass launched by the band pass,
    by the host before it (band_serial 1) and by the host after it
    (band_serial 2); frames whose blocks cross the right or bottom edge and a
    band wide enough to leave many warps with pixels the band pass writes."""
    torch = pytest.importorskip("torch")
    scenes = S.flythrough(2, 320, 180) + [S.single_scene(200, 117), S.flythrough(3, 150, 83)[1]]
    base = dict(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_HYBRID, format=capi.FORMAT_BGR8,
                band=0.02, step=0.15, band_serial=band_serial)
    ref = renderer.render(scenes, opts(**base, block_x=8, block_y=16, rays_per_thread=4), hit_class=True)
    bufs, frames = [], (capi.Frame * len(scenes))()
    for i, s in enumerate(scenes):
        h, w = s.camera.height(), s.camera.width()
        px = torch.zeros((h, w, 3), dtype=torch.uint8, device="cuda")
        cl = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
        bufs.append((px, cl))
        frames[i] = capi.Frame(px.data_ptr(), cl.data_ptr(), None)
    renderer.render_device(renderer.c_scenes(scenes), frames, opts(**base, block_x=32, block_y=4, rays_per_thread=8))
    torch.cuda.synchronize()
    assert renderer.stats().band_rays > 0
    for (px, cl), r in zip(bufs, ref):
        assert np.array_equal(px.cpu().numpy(), r.pixels)
        assert np.array_equal(cl.cpu().numpy(), r.hit_class)


def test_fp32_step_is_fourth_order(renderer):
    """The FP32 tracers' step (Nystrom's three-stage method) is fourth order:
    against FP64 RK4 at step 0.01, halving the step from 0.2 to 0.1 divides
    the largest deflection error of the escaped rays away from b_c
    (|b - b_c| > 0.5 M, where FP32 rounding stays far below the truncation)
    by about 2^4 = 16; at least 6 here, and at step 0.2 that error is below
    the 1e-4 rad bound."""
    sc = S.flythrough(3, 320, 180)[1]
    h, w = sc.camera.height(), sc.camera.width()
    ys, xs = np.mgrid[0:h, 0:w]
    far = (np.abs(S.ref_impact_parameter(sc, xs.ravel(), ys.ravel()) - 3.0 * 3.0 ** 0.5) > 0.5).reshape(h, w)
    ref = renderer.render([sc], opts(precision=capi.PRECISION_FP64, step=0.01), hit_class=True, aux=True)[0]
    errs = []
    for step in (0.2, 0.1):
        out = renderer.render([sc], opts(precision=capi.PRECISION_FP32, step=step), hit_class=True, aux=True)[0]
        m = far & (out.hit_class == capi.CLASS_MISS) & (ref.hit_class == capi.CLASS_MISS)
        assert m.sum() > 1000
        errs.append(float(np.abs(out.aux[m].astype(np.float64) - ref.aux[m]).max()))
    assert errs[0] < 1e-4
    assert errs[0] / errs[1] > 6.0, errs


def test_hybrid_band_pass_block_sizes_agree(renderer):
    """The HYBRID band pass in blocks of 128, 256 and 512 threads (the
    tuner's candidates): every band ray is traced by the same code whatever
    lane takes it, so frames, classes and deflections are identical."""
    scenes = S.flythrough(2, 320, 180) + [S.photon_ring_scene(256)]
    out = []
    for threads in (128, 256, 512):
        o = opts(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_HYBRID, band=0.02, step=0.175,
                 threads_per_block=threads, rays_per_thread=8, max_steps=20000)
        out.append(renderer.render(scenes, o, hit_class=True, aux=True))
        assert renderer.stats().band_rays > 0
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a.pixels, b.pixels)
            assert np.array_equal(a.hit_class, b.hit_class)
            assert np.array_equal(a.aux.view(np.uint32), b.aux.view(np.uint32))


def test_render_device_on_torch_stream(renderer):
    torch = pytest.importorskip("torch")
    scenes = [S.single_scene(64, 36)]
    bufs, frames = _device_frames(torch, scenes)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        renderer.render_device(renderer.c_scenes(scenes), frames, opts(), stream=st.cuda_stream)
    st.synchronize()
    ref = renderer.render(scenes, opts())[0]
    assert np.array_equal(bufs[0][0].cpu().numpy(), ref.pixels)


# ---------------------------------------------------------------------------
# error paths (no GPU fault involved)
def test_error_paths(renderer):
    lib, ctx = renderer.lib, renderer.ctx
    out = C.c_int32()
    empty = np.zeros((0, 0, 3), np.uint8)
    assert lib.bh_texture_create(ctx, None, 0, 0, capi.TEXEL_BGR8, 0, C.byref(out)) == capi.BH_ERR_EMPTY_TEXTURE
    assert b"empty" in lib.bh_last_error(ctx)
    sc = S.single_scene(32, 18)
    cs = renderer.c_scenes([sc])
    frames = (capi.Frame * 1)()
    buf = np.zeros((18, 32, 4), np.uint8)
    frames[0].pixels = buf.ctypes.data
    # bad texture id
    bad = renderer.c_scenes([sc])
    bad[0].disc.texture = 999
    assert lib.bh_render(ctx, bad, 1, frames, C.byref(opts())) == capi.BH_ERR_BAD_TEXTURE
    # disc plane not through the hole: the RK4 events need it
    off = renderer.c_scenes([sc])
    off[0].disc.center[2] = 0.5
    assert lib.bh_render(ctx, off, 1, frames, C.byref(opts())) == capi.BH_ERR_UNSUPPORTED
    # ... while the reference scheme handles any disc placement
    o = opts(integrator=capi.INTEGRATOR_REF_TRAPEZOID)
    assert lib.bh_render(ctx, off, 1, frames, C.byref(o)) == capi.BH_OK
    # camera outside the escape radius
    far = renderer.c_scenes([sc])
    far[0].camera.position[0] = -150.0
    assert lib.bh_render(ctx, far, 1, frames, C.byref(opts())) == capi.BH_ERR_UNSUPPORTED
    # invalid options
    for kw in ({"step": 0.0 - 1}, {"max_steps": -1}, {"block_x": 7, "block_y": 1}, {"precision": 9},
               {"integrator": capi.INTEGRATOR_REF_TRAPEZOID, "precision": capi.PRECISION_MIXED}):
        assert lib.bh_render(ctx, cs, 1, frames, C.byref(opts(**kw))) in (capi.BH_ERR_INVALID_ARGUMENT,
                                                                          capi.BH_ERR_UNSUPPORTED)
    # non-finite camera
    nan = renderer.c_scenes([sc])
    nan[0].camera.axis_x[0] = float("nan")
    assert lib.bh_render(ctx, nan, 1, frames, C.byref(opts())) == capi.BH_ERR_INVALID_ARGUMENT
    # the context still renders after the errors
    assert lib.bh_render(ctx, cs, 1, frames, C.byref(opts())) == capi.BH_OK
