"""The autotuner (bh_autotune): its choice must keep the mixed tracer within
the deflection bound against the FP64 oracle, and the cache must return the
same choice."""
import os

import numpy as np
import pytest

from blackhole_8_gb300 import capi
from blackhole_8_gb300 import scene as S
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_autotune_choice_meets_bound(renderer, tmp_path):
    scenes = S.flythrough(6, 320, 180)
    cs = renderer.c_scenes(scenes)
    cache = str(tmp_path / "tune.txt")
    opts, rep = renderer.autotune(cs, max_error=1e-4, cache_path=cache)
    assert rep.from_cache == 0 and rep.candidates > 2
    assert opts.precision == capi.PRECISION_MIXED
    assert opts.schedule in (capi.SCHEDULE_PERSISTENT, capi.SCHEDULE_GRID, capi.SCHEDULE_HYBRID)
    assert opts.band in (2e-5, 1e-4, 5e-4)
    # 12 persistent, 12 hybrid and 2 grid schedule candidates after the step
    # (and band) candidates
    assert rep.candidates >= 1 + 12 + 12 + 2
    assert 0.01 <= opts.step <= 0.2
    assert rep.max_deflection <= 5e-5 and rep.class_mismatch <= 1e-4
    # the choice against the FP64 oracle on a seeded pixel sample of two frames
    out = renderer.render([scenes[1], scenes[4]], opts, hit_class=True, aux=True)
    rng = np.random.default_rng(5)
    for sc, fb in zip([scenes[1], scenes[4]], out):
        xs, ys = rng.integers(0, 320, 2000), rng.integers(0, 180, 2000)
        o = oracle.render_rk4(sc, pixels=np.stack([xs, ys], 1))
        agree = fb.hit_class[ys, xs] == o["cls"]
        assert agree.mean() >= 0.998
        esc = agree & (o["cls"] == capi.CLASS_MISS)
        assert np.abs(fb.aux[ys, xs][esc] - o["aux"][esc]).max(initial=0) <= 1e-4
    # cached: same choice, no tuning
    opts2, rep2 = renderer.autotune(cs, max_error=1e-4, cache_path=cache)
    assert rep2.from_cache == 1
    fields = ("step", "band", "threads_per_block", "refill_threshold", "slice_steps", "schedule", "block_x", "block_y",
              "rays_per_thread")
    assert [getattr(opts2, f) for f in fields] == [getattr(opts, f) for f in fields]
    assert os.path.getsize(cache) > 0
