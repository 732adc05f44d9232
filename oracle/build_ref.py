"""Test infrastructure (oracle only): builds the reference's own CPU render.

Recipe for ``oracle/_ref/`` (git-ignored; it travels with the working tree
but is never committed):

1. Stage (only where the reference checkout exists, at ``REFERENCE_ROOT``):
   - the render loop of ``include/blackhole/blackhole_solution_test.cc``,
     lines 161-308 (the body of its frame loop: ray generation, orbital-plane
     reduction, the 20+20-step trapezoid integration, collisions and shading),
     is extracted unmodified into ``_ref/src/ref_render_loop.inc``. One line
     is inserted between 161 and 162: an OpenMP ``parallel for`` over the
     column loop, so the same code can also be timed on all host cores
     (pixels are independent; ``ObjectManager::FindCollision`` is const);
   - the scene/physics headers the loop needs are staged next to it under
     ``_ref/src/include/blackhole``.
   The extraction checks that the marker lines are where they are expected
   and refuses otherwise.
2. Compile (anywhere the staged sources exist, e.g. also on an Arm GPU host):
   ``oracle/ref_runner.cc`` + the staged sources + the OpenCV stand-in in
   ``oracle/cvshim`` -> ``_ref/ref_runner`` with plain ``g++`` (no cmake).

The reference needs OpenCV, which is not installed; its physics headers only
touch the small API surface that ``oracle/cvshim/opencv2/opencv.hpp``
provides.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(REF_DIR, "src")
RUNNER = os.path.join(REF_DIR, "ref_runner")
# The reference checkout: $BH_REFERENCE_ROOT, else a sibling directory
# named "reference" next to this repository.
REFERENCE_ROOT = os.environ.get("BH_REFERENCE_ROOT",
                                os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference")))

LOOP_FILE = "include/blackhole/blackhole_solution_test.cc"
LOOP_FIRST, LOOP_SPLIT, LOOP_LAST = 161, 162, 308
HEADERS = [
    "camera.h", "constants.h", "math.h", "matrix.h", "object.h", "utility.h",
    "blackhole_solution.h", "object/material.h", "object/object.h",
    "object/object_manager.h", "object/pattern.h", "object/polygon_object.h",
    "object/vector_object.h", "ray_tracer.h",
]
# (line number, text that must appear on it) -- guards against a moved loop.
MARKERS = [
    (161, "const auto fv = camera.focus_vector();"),
    (162, "for (int x = 0; x < kScreenWidth; ++x) {"),
    (163, "for (int y = 0; y < kScreenHeight; ++y) {"),
    (217, "for (int i = 0; i < nstep_safe; ++i) {"),
    (298, "kGOTO_PIXEL_LOOP_END:;"),
]


def reference_present() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_ROOT, LOOP_FILE))


def stage() -> None:
    """Extracts the loop and stages the headers (needs the reference)."""
    path = os.path.join(REFERENCE_ROOT, LOOP_FILE)
    with open(path, encoding="utf-8") as fh:
        lines = fh.read().split("\n")
    for ln, text in MARKERS:
        if text not in lines[ln - 1]:
            raise RuntimeError(f"{LOOP_FILE}:{ln} does not hold {text!r}")
    if lines[LOOP_LAST - 1].strip() != "}" or lines[LOOP_LAST - 2].strip() != "}":
        raise RuntimeError(f"{LOOP_FILE}:{LOOP_LAST - 1}-{LOOP_LAST} are not the loop's closing braces")
    os.makedirs(os.path.join(SRC_DIR, "include", "blackhole", "object"), exist_ok=True)
    src_name = "blackhole_solution_test.cc"
    body = [f'#line {LOOP_FIRST} "{src_name}"', lines[LOOP_FIRST - 1],
            "#pragma omp parallel for schedule(dynamic, 2)",
            f'#line {LOOP_SPLIT} "{src_name}"']
    body += lines[LOOP_SPLIT - 1:LOOP_LAST]
    with open(os.path.join(SRC_DIR, "ref_render_loop.inc"), "w", encoding="utf-8") as fh:
        fh.write("\n".join(body) + "\n")
    for h in HEADERS:
        shutil.copyfile(os.path.join(REFERENCE_ROOT, "include", "blackhole", h),
                        os.path.join(SRC_DIR, "include", "blackhole", h))


def staged() -> bool:
    return os.path.isfile(os.path.join(SRC_DIR, "ref_render_loop.inc"))


def compile_runner() -> str:
    cmd = [
        os.environ.get("CXX", "g++"), "-std=c++17", "-O3", "-DNDEBUG", "-fopenmp", "-w",
        "-I", SRC_DIR, "-I", os.path.join(SRC_DIR, "include"),
        "-I", os.path.join(HERE, "cvshim"),
        os.path.join(HERE, "ref_runner.cc"), "-o", RUNNER,
    ]
    subprocess.run(cmd, check=True)
    return RUNNER


def build(force: bool = False) -> str | None:
    """Stages (when the reference is present) and compiles; returns the
    runner path, or None when neither the reference nor staged sources exist."""
    if reference_present():
        stage()
    if not staged():
        return None
    src = os.path.join(HERE, "ref_runner.cc")
    newest = max(os.path.getmtime(os.path.join(SRC_DIR, "ref_render_loop.inc")),
                 os.path.getmtime(src))
    if force or not os.path.exists(RUNNER) or os.path.getmtime(RUNNER) < newest:
        compile_runner()
    return RUNNER


if __name__ == "__main__":
    out = build(force="--force" in sys.argv)
    print(out if out else "reference sources unavailable: nothing built")
