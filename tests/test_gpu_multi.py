"""GPU parity of the MULTI integrator (several holes) through the C ABI,
against its FP64 CPU restatement (oracle/bh_oracle.c multi_pixel, itself
pinned by the Schwarzschild orbit integral and by symmetry in
tests/test_oracle_multi.py).

Bars (tolerances written in each test):
- FP64: classes equal away from class boundaries (dilated 1 pixel); the
  bending of escaped rays and the radius of disc hits within 1e-7 (rad /
  units of M); colours equal away from texel edges.
- FP32: classes agree on >= 99 % and differ only near class boundaries
  (dilated 2 pixels); the bending within 2e-3 rad away from boundaries.
- an equal-mass binary renders mirror symmetric on the GPU too (FP64).
- objects take part on the step chords: object indices as the oracle's.
- invalid requests fail with status codes (no launch).
"""
import ctypes as C

import numpy as np
import pytest

import helpers
from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S
from oracle import oracle

pytestmark = pytest.mark.gpu

STEP = 0.02
MAX_STEPS = 20000


def opts(**kw):
    kw.setdefault("step", STEP)
    kw.setdefault("max_steps", MAX_STEPS)
    return capi.default_options(integrator=capi.INTEGRATOR_MULTI, **kw)


def dilate(m, n=1):
    for _ in range(n):
        m2 = m.copy()
        m2[1:, :] |= m[:-1, :]
        m2[:-1, :] |= m[1:, :]
        m2[:, 1:] |= m[:, :-1]
        m2[:, :-1] |= m[:, 1:]
        m = m2
    return m


def scenes():
    binary = S.binary_scene(96, 54)
    unequal = S.binary_scene(96, 54, separation=8.0, mass_ratio=0.3, inclination_deg=65.0)
    with_objects = S.binary_scene(96, 54, radius=40.0)
    with_objects.objects = [S.InfinitePlane((0.0, 0.0, -8.0), S.ChessPattern2D(2)),
                            S.Rectangle((25, 10, 10), (25, -10, 10), (25, -10, -6), (25, 10, -6))]
    with_objects.objects[1].SetTexture(S.panel_texture(5))
    return {"binary": binary, "unequal": unequal, "objects": with_objects, "single": S.single_scene(96, 54)}


SCENES = scenes()


@pytest.fixture(scope="module")
def oracle_out():
    return {k: oracle.render_multi(v, step=STEP, max_steps=MAX_STEPS) for k, v in SCENES.items()}


@pytest.mark.parametrize("name", list(SCENES))
def test_fp64_matches_oracle(renderer, oracle_out, name):
    sc, o = SCENES[name], oracle_out[name]
    out = renderer.render([sc], opts(precision=capi.PRECISION_FP64), hit_class=True, aux=True)[0]
    edge = dilate(helpers.class_boundary_mask(o["cls"]))
    edge |= (o["cls"] == capi.CLASS_DISC) & (o["margin_r"] < 1e-6)
    same = out.hit_class == o["cls"]
    assert not (~same & ~edge).any(), "class mismatch away from boundaries"
    strict = same & ~edge
    for cls in (capi.CLASS_MISS, capi.CLASS_DISC):
        m = strict & (o["cls"] == cls)
        if m.any():
            err = np.abs(out.aux[m] - o["aux"][m]).max()
            assert err <= 1e-7 * max(1.0, np.abs(o["aux"][m]).max()), (cls, err)
    obj = strict & (o["cls"] == capi.CLASS_OBJECT)
    assert np.array_equal(np.rint(out.aux[obj]), o["aux"][obj])
    # texel-edge margins exist for the sky and the disc; an object's colour
    # (texture or chess cell) may flip on its own edges
    colour = strict & (o["margin_tex"] > 1e-6) & (o["cls"] != capi.CLASS_OBJECT)
    assert np.array_equal(out.pixels[..., :3][colour], o["bgra"][..., :3][colour])
    if obj.any():
        same_obj = (out.pixels[..., :3][obj] == o["bgra"][..., :3][obj]).all(-1)
        assert same_obj.mean() >= 0.98, same_obj.mean()
    assert (o["cls"] == capi.CLASS_HORIZON).any() and (o["cls"] == capi.CLASS_MISS).any()
    if name == "objects":
        assert (o["cls"] == capi.CLASS_OBJECT).any()


@pytest.mark.parametrize("name", ["binary", "unequal", "single"])
def test_fp32_matches_oracle(renderer, oracle_out, name):
    sc, o = SCENES[name], oracle_out[name]
    out = renderer.render([sc], opts(precision=capi.PRECISION_FP32), hit_class=True, aux=True)[0]
    same = out.hit_class == o["cls"]
    assert same.mean() >= 0.99, same.mean()
    edge = dilate(helpers.class_boundary_mask(o["cls"]), 2)
    edge |= (o["cls"] == capi.CLASS_DISC) & (o["margin_r"] < 1e-3)
    assert not (~same & ~edge).any(), "class mismatch away from boundaries"
    esc = same & ~edge & (o["cls"] == capi.CLASS_MISS)
    err = np.abs(out.aux[esc] - o["aux"][esc]).max(initial=0)
    assert err <= 2e-3, err


def test_binary_mirror_symmetric_on_gpu(renderer):
    W, H = 97, 55
    sc = S.binary_scene(W, H)
    out = renderer.render([sc], opts(precision=capi.PRECISION_FP64), hit_class=True, aux=True)[0]
    cls, aux = out.hit_class.astype(int), out.aux
    lo, hi = 1, W
    mirror = lambda a: a[:, lo:hi][:, ::-1]
    assert np.array_equal(cls[:, lo:hi], mirror(cls))
    miss = cls[:, lo:hi] == capi.CLASS_MISS
    assert np.abs(aux[:, lo:hi] - mirror(aux))[miss].max() < 1e-6


def test_sequence_matches_direct_render(renderer):
    import torch
    scs = [S.binary_scene(64, 36, separation=s) for s in (5.0, 6.0, 7.0)]
    o = opts(precision=capi.PRECISION_FP32)
    direct = renderer.render(scs, o)
    bufs = [torch.zeros((36, 64, 4), dtype=torch.uint8, device="cuda") for _ in scs]
    frames = (capi.Frame * len(scs))()
    for i, b in enumerate(bufs):
        frames[i].pixels = b.data_ptr()
    cs = renderer.c_scenes(scs)
    seq = renderer.sequence(cs, frames, o)
    try:
        seq.launch()
        torch.cuda.synchronize()
        for d, b in zip(direct, bufs):
            assert np.array_equal(d.pixels, b.cpu().numpy())
    finally:
        seq.close()


def test_invalid_requests(renderer):
    sc = S.binary_scene(32, 18)
    with pytest.raises(capi.BhError) as e:  # extra holes need MULTI
        renderer.render([sc], capi.default_options(integrator=capi.INTEGRATOR_RK4))
    assert e.value.code == capi.BH_ERR_UNSUPPORTED
    for bad in (dict(precision=capi.PRECISION_MIXED), dict(schedule=capi.SCHEDULE_PERSISTENT)):
        with pytest.raises(capi.BhError) as e:
            renderer.render([sc], opts(**bad))
        assert e.value.code == capi.BH_ERR_UNSUPPORTED
    many = S.binary_scene(32, 18)
    many.extra_holes = [S.StaticBlackhole((0.0, 3.0 + i, 0.0), 0.1) for i in range(capi.MAX_HOLES)]
    with pytest.raises(capi.BhError) as e:
        renderer.render([many], opts())
    assert e.value.code == capi.BH_ERR_INVALID_ARGUMENT
    far = S.binary_scene(32, 18, radius=150.0)  # camera outside r_escape * total mass
    with pytest.raises(capi.BhError) as e:
        renderer.render([far], opts())
    assert e.value.code == capi.BH_ERR_UNSUPPORTED
    neg = S.binary_scene(32, 18)
    neg.extra_holes = [S.StaticBlackhole((0.0, 3.0, 0.0), -1.0)]
    with pytest.raises(capi.BhError) as e:
        renderer.render([neg], opts())
    assert e.value.code == capi.BH_ERR_INVALID_ARGUMENT


def triple_scene(w=96, h=54):
    """The binary with a third, lighter hole above the disc plane: three
    holes take the kernel's general (runtime-count) path."""
    sc = S.binary_scene(w, h)
    sc.extra_holes.append(S.StaticBlackhole((-2.0, 0.0, 2.5), 0.25))
    return sc


def test_three_holes_match_oracle(renderer):
    """FP64 through the general hole loop against the restatement. Three
    holes scatter some rays chaotically, so the bars are robust ones:
    classes equal on >= 99.5 % and only near boundaries; the bending of
    escaped rays (the library returns it in FP32) equal to the
    restatement's rounded to FP32 at the median and within one FP32 ulp
    of pi at the 99th percentile. (Moving the camera by 1e-13 moves the
    restatement's bending by at most 5e-13 rad on this scene.)"""
    sc = triple_scene()
    o = oracle.render_multi(sc, step=STEP, max_steps=MAX_STEPS)
    out = renderer.render([sc], opts(precision=capi.PRECISION_FP64), hit_class=True, aux=True)[0]
    same = out.hit_class == o["cls"]
    assert same.mean() >= 0.995, same.mean()
    edge = dilate(helpers.class_boundary_mask(o["cls"]), 2)
    assert not (~same & ~edge).any(), "class mismatch away from boundaries"
    esc = same & ~edge & (o["cls"] == capi.CLASS_MISS)
    err = np.abs(out.aux[esc].astype(np.float64) - o["aux"][esc].astype(np.float32).astype(np.float64))
    assert np.median(err) == 0.0 and np.percentile(err, 99) <= 2.4e-7, (np.median(err), np.percentile(err, 99))
