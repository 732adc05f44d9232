"""Generates the golden fixtures of the reference's own render.

Runs the reference's render loop (blackhole_solution_test.cc:161-308, built
into oracle/_ref by oracle/build_ref.py against the OpenCV stand-in), or its
flat RayTracer (ray_tracer.h:52-96) for the flat cases, on the scenes of
tests/helpers.py and stores, per case, the BGR frame, the hit class of every
pixel and the index of the object hit (-1: none), the last two from the
runner's tag pass. Needs the reference checkout; the fixtures then pin the
oracle and the GPU on hosts without it.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import refbridge  # noqa: E402
import helpers  # noqa: E402


def main() -> None:
    index = []
    for name, w, h in helpers.GOLDEN_CASES:
        sc = helpers.build(name, w, h)
        flat = name in helpers.FLAT_BUILDERS
        img, cls, obj = refbridge.render_with_classes(sc, flat=flat, with_objects=True)
        fn = f"ref_{name}_{w}x{h}.npz"
        np.savez_compressed(os.path.join(HERE, fn), bgr=img, cls=cls, obj=obj)
        index.append({"file": fn, "builder": name, "width": w, "height": h, "mode": "flat" if flat else "curved",
                      "classes": np.bincount(cls.ravel(), minlength=5).tolist()})
        print(fn, index[-1]["classes"])
    with open(os.path.join(HERE, "index.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "source": "reference render loop blackhole_solution_test.cc:161-308 (flat: RayTracer, "
                             "ray_tracer.h:52-96) via oracle/_ref/ref_runner",
                   "cases": index}, fh, indent=1)


if __name__ == "__main__":
    main()
