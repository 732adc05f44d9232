"""GPU parity of the ordinary objects (Rectangle, Triangle, InfinitePlane with
ChessPattern2D) and of the flat RayTracer, through the C ABI.

Bars (tolerances written in each test):
- FLAT and REF_TRAPEZOID with objects, FP64: against the reference's own
  output (tests/test_gpu_render.py::test_trapezoid_fp64_matches_reference on
  the flat_demo and objects fixtures) and here against the FP64 oracle with
  triangles added (the reference's Triangle<T> does not compile when
  instantiated): classes and object indices equal except on class
  boundaries, colours equal except texel-edge ties.
- RK4 with objects (FP64 and FP32) against oracle B with the same chord rule:
  classes agree on >= 99.9 % (FP64) / 99.5 % (FP32) away from boundaries,
  object indices agree where both hit an object, deflection of escaped rays
  within 1e-4 rad (FP64).
"""
import numpy as np
import pytest

import helpers
from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S
from oracle import oracle

pytestmark = pytest.mark.gpu


def opts(**kw):
    return capi.default_options(**kw)


def _away(cls, n=1):
    m = helpers.class_boundary_mask(cls)
    for _ in range(n):
        m2 = m.copy()
        m2[1:, :] |= m[:-1, :]
        m2[:-1, :] |= m[1:, :]
        m2[:, 1:] |= m[:, :-1]
        m2[:, :-1] |= m[:, 1:]
        m = m2
    return ~m


def _obj_index(cls, aux):
    return np.where(cls == capi.CLASS_OBJECT, np.rint(aux), -1).astype(np.int32)


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_FP32])
def test_flat_matches_oracle(renderer, precision):
    sc = helpers.flat_demo(160, 90)
    sc.objects.append(S.Triangle((0, -60, 40), (0, 60, 40), (0, 0, 140)))
    ref = oracle.render_flat(sc)
    out = renderer.render([sc], opts(integrator=capi.INTEGRATOR_FLAT, precision=precision), hit_class=True,
                          aux=True)[0]
    away = _away(ref["cls"])
    assert np.array_equal(out.hit_class[away], ref["cls"][away])
    gi, oi = _obj_index(out.hit_class, out.aux), _obj_index(ref["cls"], ref["aux"])
    tol = 1e-3 if precision == capi.PRECISION_FP64 else 2e-2
    assert (gi != oi).mean() <= tol
    assert (gi == 4).any(), "the triangle is visible"
    diff = (out.pixels[..., :3] != ref["bgra"][..., :3]).any(-1)
    assert diff.mean() <= (2e-3 if precision == capi.PRECISION_FP64 else 3e-2)


def test_trapezoid_with_triangles_matches_oracle(renderer):
    sc = helpers.triangles(160, 90)
    ref = oracle.render_ref(sc)
    out = renderer.render([sc], opts(integrator=capi.INTEGRATOR_REF_TRAPEZOID, precision=capi.PRECISION_FP64),
                          hit_class=True)[0]
    bad = out.hit_class != ref["cls"]
    assert bad.mean() <= 1e-3 and not (bad & _away(ref["cls"])).any()
    assert (ref["cls"] == capi.CLASS_OBJECT).sum() > 100
    diff = (out.pixels[..., :3] != ref["bgra"][..., :3]).any(-1)
    assert diff.mean() <= 3e-3


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_FP32])
def test_rk4_with_objects_matches_oracle(renderer, precision):
    sc = helpers.triangles(160, 90)
    ref = oracle.render_rk4(sc)
    out = renderer.render([sc], opts(precision=precision), hit_class=True, aux=True)[0]
    away = _away(ref["cls"], 2)
    agree = out.hit_class == ref["cls"]
    need = 0.999 if precision == capi.PRECISION_FP64 else 0.995
    assert agree[away].mean() >= need, agree[away].mean()
    assert (ref["cls"] == capi.CLASS_OBJECT).sum() > 100
    both = agree & (ref["cls"] == capi.CLASS_OBJECT)
    assert (_obj_index(out.hit_class, out.aux)[both] == ref["aux"][both]).mean() >= 0.999
    if precision == capi.PRECISION_FP64:
        esc = agree & (ref["cls"] == capi.CLASS_MISS) & away
        d = np.abs(out.aux[esc] - ref["aux"][esc])
        d = np.minimum(d, 2 * np.pi - d)
        assert d.max(initial=0) <= 1e-4


def test_sequence_with_objects_matches_direct_render(renderer):
    torch = pytest.importorskip("torch")
    scenes = [helpers.objects(96, 54), helpers.triangles(96, 54)]
    o = opts(precision=capi.PRECISION_FP32)
    bufs, frames = [], (capi.Frame * len(scenes))()
    for i, s in enumerate(scenes):
        px = torch.zeros((54, 96, 4), dtype=torch.uint8, device="cuda")
        bufs.append(px)
        frames[i].pixels = px.data_ptr()
    seq = renderer.sequence(renderer.c_scenes(scenes), frames, o)
    seq.launch()
    torch.cuda.synchronize()
    direct = renderer.render(scenes, o)
    for px, d in zip(bufs, direct):
        assert np.array_equal(px.cpu().numpy(), d.pixels)
    seq.close()


def test_object_options_rejected(renderer):
    sc = helpers.objects(32, 18)
    for bad in (opts(schedule=capi.SCHEDULE_PERSISTENT), opts(precision=capi.PRECISION_MIXED)):
        with pytest.raises(capi.BhError):
            renderer.render([sc], bad)
    with pytest.raises(capi.BhError):
        renderer.render([helpers.flat_demo(32, 18)], opts(integrator=capi.INTEGRATOR_FLAT,
                                                          schedule=capi.SCHEDULE_PERSISTENT))
    sc.objects[0].pattern = S.ChessPattern2D(0.25)  # (int)(2 * size) == 0: division by zero in the reference
    with pytest.raises(capi.BhError):
        renderer.render([sc], opts())
