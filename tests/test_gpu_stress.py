"""The near-critical stress configurations and the uneven batch at their
specified sizes, through the C ABI against the FP64 oracle.

- Photon ring: a 4096x4096 image with a 0.5 deg field of view aimed at the
  photon ring (b within ~0.085 M of 3 sqrt(3) M), at most 20000 steps, mixed
  precision on the persistent schedule. Every ray of the FP64 band and 4000
  seeded others against the oracle: full parity bar, deflection within
  1e-4 rad on every escaped ray (no exclusion near b_c).
- Impact-parameter grid: b uniform over 3 sqrt(3) M +- 1e-4 M (a 1024x1024
  grid here): with the default band every ray is traced in FP64 and matches
  the oracle's deflection to 1e-6 rad.
- Uneven batch: 256 scenes, sides 64-1024, in one persistent launch; 300
  seeded pixels of every scene against the oracle, class agreement counted
  over the batch.
"""
import math

import numpy as np
import pytest

from parity import B_C, sample_check
from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S
from oracle import oracle

pytestmark = pytest.mark.gpu


def _band_pixels(scene, band):
    """Pixels whose impact parameter lies within `band` M of b_c (FP64)."""
    w, h = scene.camera.width(), scene.camera.height()
    out = []
    for y0 in range(0, h, 256):
        ys, xs = np.mgrid[y0:min(h, y0 + 256), 0:w]
        b = S.ref_impact_parameter(scene, xs, ys)
        sel = np.abs(b - B_C) < band
        out.append(np.stack([xs[sel], ys[sel]], 1))
    return np.concatenate(out)


@pytest.mark.parametrize("schedule", [capi.SCHEDULE_PERSISTENT, capi.SCHEDULE_HYBRID])
def test_photon_ring_4096(renderer, schedule):
    sc = S.photon_ring_scene(4096)
    o = capi.default_options(precision=capi.PRECISION_MIXED, schedule=schedule, max_steps=20000, rays_per_thread=4)
    fb = renderer.render([sc], o, hit_class=True, aux=True)[0]
    st = renderer.stats()
    assert st.rays == 4096 * 4096 and st.flags == 0 and st.band_overflow == 0
    band = _band_pixels(sc, o.band)
    # the GPU's band decision is the FP64 first integral's: the same rays up
    # to ties at the band's edge
    assert abs(int(st.band_rays) - len(band)) <= 2, (st.band_rays, len(band))
    rng = np.random.default_rng(4)
    rand = np.stack([rng.integers(0, 4096, 4000), rng.integers(0, 4096, 4000)], 1)
    pts = np.concatenate([band, rand])
    xs, ys = pts[:, 0], pts[:, 1]
    kw = {"max_steps": 20000}
    orc = oracle.render_rk4(sc, pixels=pts, **kw)
    sample_check(sc, xs, ys, fb.hit_class[ys, xs], fb.pixels[ys, xs], fb.aux[ys, xs], orc, kw, band=0.0,
                 aux_everywhere=True)


def test_impact_grid_all_rays_in_band(renderer):
    sc = S.impact_grid_scene(1024)
    o = capi.default_options(precision=capi.PRECISION_MIXED, schedule=capi.SCHEDULE_PERSISTENT, max_steps=20000)
    fb = renderer.render([sc], o, hit_class=True, aux=True)[0]
    st = renderer.stats()
    assert st.rays == 1024 * 1024 and st.band_rays == 1024 * 1024 and st.flags == 0
    rng = np.random.default_rng(5)
    xs, ys = rng.integers(0, 1024, 3000), rng.integers(0, 1024, 3000)
    kw = {"max_steps": 20000}
    orc = oracle.render_rk4(sc, pixels=np.stack([xs, ys], 1), **kw)
    assert np.abs(orc["b_over_m"] - B_C).max() <= 1.001e-4
    sample_check(sc, xs, ys, fb.hit_class[ys, xs], fb.pixels[ys, xs], fb.aux[ys, xs], orc, kw, band=0.0,
                 aux_tol=1e-6, aux_everywhere=True)


@pytest.fixture(scope="module")
def batch():
    return S.batched_scenes(256)


@pytest.mark.parametrize("step,schedule,band", [(0.01, capi.SCHEDULE_PERSISTENT, 5e-4),
                                               (0.1, capi.SCHEDULE_PERSISTENT, 5e-4),
                                               (0.1, capi.SCHEDULE_HYBRID, 2e-5)],
                         ids=["persistent-0.01", "persistent-0.1", "hybrid-0.1-band2e-5"])
def test_uneven_batch_256(renderer, batch, step, schedule, band):
    o = capi.default_options(precision=capi.PRECISION_MIXED, schedule=schedule, step=step, band=band,
                             rays_per_thread=4)
    out = renderer.render(batch, o, hit_class=True, aux=True)
    st = renderer.stats()
    assert st.rays == sum(s.camera.width() * s.camera.height() for s in batch) and st.flags == 0
    rng = np.random.default_rng(6)
    agree = total = 0
    worst = 0.0
    for sc, fb in zip(batch, out):
        w, h = sc.camera.width(), sc.camera.height()
        xs, ys = rng.integers(0, w, 300), rng.integers(0, h, 300)
        orc = oracle.render_rk4(sc, pixels=np.stack([xs, ys], 1))
        res = sample_check(sc, xs, ys, fb.hit_class[ys, xs], fb.pixels[ys, xs], fb.aux[ys, xs], orc, {},
                           radius_tol=1e-3 if step <= 0.01 else 2e-3, min_agreement=None)
        agree += res["agree"]
        total += res["pixels"]
        worst = max(worst, res["max_deflection_error"])
    assert agree / total >= 0.999, agree / total
    assert worst <= 1e-4
