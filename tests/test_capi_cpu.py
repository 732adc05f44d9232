"""Host-only checks of the C ABI: the library loads, exports every function
declared in include/bh_gb300.h, and the ctypes layouts match the C structs
(sizes and offsets printed by a C program compiled against the header)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from blackhole_8_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bh_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bh_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_abi_version_and_defaults(lib):
    assert lib.bh_abi_version() == capi.ABI_VERSION == 3
    o = capi.default_options()
    assert o.integrator == capi.INTEGRATOR_RK4 and o.step == 0.01 and o.max_steps == 4000
    assert o.r_escape == 100.0 and o.block_x * o.block_y % 32 == 0


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stddef.h>
#include <stdio.h>
#include "bh_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(bh_camera), sizeof(bh_hole), sizeof(bh_disc),
         sizeof(bh_scene), sizeof(bh_frame), sizeof(bh_render_options), sizeof(bh_render_stats),
         offsetof(bh_scene, background));
  printf("%zu %zu %zu %zu %zu\n", offsetof(bh_render_options, step), offsetof(bh_render_options, band),
         offsetof(bh_render_options, refill_threshold), offsetof(bh_render_options, band_lanes),
         offsetof(bh_render_options, band_serial));
  printf("%zu %zu %zu %d %d\n", offsetof(bh_scene, objects), offsetof(bh_scene, n_extra_holes),
         offsetof(bh_scene, extra_holes), BH_MAX_HOLES, BH_INTEGRATOR_MULTI);
  printf("%d %d %d\n", BH_RK4_ALGO_FLOPS_PER_STEP, BH_RK4_FLOPS_PER_STEP, BH_RK4_INSTRUCTIONS_PER_STEP);
  return 0;
}
''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = list(map(int, out[0].split()))
    assert sizes == [C.sizeof(capi.Camera), C.sizeof(capi.Hole), C.sizeof(capi.Disc), C.sizeof(capi.Scene),
                     C.sizeof(capi.Frame), C.sizeof(capi.RenderOptions), C.sizeof(capi.RenderStats),
                     capi.Scene.background.offset]
    offs = list(map(int, out[1].split()))
    assert offs == [capi.RenderOptions.step.offset, capi.RenderOptions.band.offset,
                    capi.RenderOptions.refill_threshold.offset, capi.RenderOptions.band_lanes.offset,
                    capi.RenderOptions.band_serial.offset]
    assert list(map(int, out[2].split())) == [capi.Scene.objects.offset, capi.Scene.n_extra_holes.offset,
                                              capi.Scene.extra_holes.offset, capi.MAX_HOLES, capi.INTEGRATOR_MULTI]
    # the roofline's per-step constants the bench reports
    assert list(map(int, out[3].split())) == [capi.RK4_ALGO_FLOPS_PER_STEP, capi.RK4_FLOPS_PER_STEP,
                                              capi.RK4_INSTRUCTIONS_PER_STEP]


def test_create_without_device_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.bh_create(C.byref(h), 0) == capi.BH_ERR_NO_DEVICE
    assert lib.bh_last_error(None) == b"null context"
