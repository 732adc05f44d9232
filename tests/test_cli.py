"""The headless frame pipeline (blackhole_8_gb300/cli.py), which stands in
for the reference's interactive frame loop (blackhole_solution_test.cc:
117-158, 327-407): on the CPU the PPM writer and the workload builders; on
the GPU each workload renders, prints its JSON line, and writes frames equal
to the renderer's own."""
import json

import numpy as np
import pytest

from blackhole_8_gb300 import capi, cli


def read_ppm(path):
    data = open(path, "rb").read()
    magic, dims, maxval, rest = data.split(b"\n", 3)
    w, h = map(int, dims.split())
    assert magic == b"P6" and maxval == b"255"
    return np.frombuffer(rest, np.uint8).reshape(h, w, 3)


def test_ppm_holds_rgb_of_bgra(tmp_path):
    bgra = np.zeros((3, 4, 4), np.uint8)
    bgra[..., 0], bgra[..., 1], bgra[..., 2], bgra[..., 3] = 10, 20, 30, 255
    bgra[1, 2] = (1, 2, 3, 255)
    cli.write_ppm(str(tmp_path / "f.ppm"), bgra)
    rgb = read_ppm(tmp_path / "f.ppm")
    assert rgb.shape == (3, 4, 3)
    assert tuple(rgb[0, 0]) == (30, 20, 10) and tuple(rgb[1, 2]) == (3, 2, 1)


def test_ppm_of_bgr_and_rgba_frames(tmp_path):
    bgr = np.zeros((2, 3, 3), np.uint8)
    bgr[0, 1] = (1, 2, 3)
    cli.write_ppm(str(tmp_path / "a.ppm"), bgr)
    assert tuple(read_ppm(tmp_path / "a.ppm")[0, 1]) == (3, 2, 1)
    rgba = np.zeros((2, 3, 4), np.uint8)
    rgba[1, 2] = (7, 8, 9, 255)
    cli.write_ppm(str(tmp_path / "b.ppm"), rgba, rgb_first=True)
    assert tuple(read_ppm(tmp_path / "b.ppm")[1, 2]) == (7, 8, 9)


@pytest.mark.parametrize("workload,n", [("flythrough", 3), ("objects", 2), ("flat", 2), ("binary", 2),
                                        ("single", 1), ("batched", 3)])
def test_workloads_build(workload, n):
    args = cli.argparse.Namespace(workload=workload, frames=n, width=48, height=27)
    scenes = cli.build_scenes(args)
    assert len(scenes) == n
    if workload == "binary":
        assert all(len(s.extra_holes) == 1 for s in scenes)
    if workload in ("objects", "flat"):
        assert all(s.objects for s in scenes)


@pytest.mark.gpu
@pytest.mark.parametrize("argv", [
    ["--workload", "flythrough", "--frames", "3", "--precision", "mixed", "--schedule", "persistent", "--step", "0.1"],
    ["--workload", "objects", "--frames", "2"],
    ["--workload", "flat", "--frames", "2", "--integrator", "flat"],
    ["--workload", "binary", "--frames", "2", "--integrator", "multi", "--step", "0.05", "--max-steps", "20000"],
    ["--workload", "binary", "--frames", "1", "--step", "0.05", "--max-steps", "20000"],  # MULTI by default
    ["--workload", "flythrough", "--frames", "2", "--precision", "mixed", "--schedule", "hybrid", "--step", "0.15",
     "--format", "bgr8", "--block", "32x4"],
    ["--workload", "flythrough", "--frames", "2", "--format", "rgba8"],
])
def test_cli_renders_and_writes_frames(tmp_path, capsys, renderer, argv):
    w, h = 96, 54
    rc = cli.main(argv + ["--width", str(w), "--height", str(h), "--repeat", "2", "--ppm", str(tmp_path)])
    assert rc == 0
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    frames = int(argv[argv.index("--frames") + 1])
    assert out["frames"] == frames and out["rays"] == frames * w * h and out["mrays_per_s"] > 0
    # the first frame equals the renderer's own render of the same scene and options
    args = cli.argparse.Namespace(workload=argv[1], frames=frames, width=w, height=h)
    scenes = cli.build_scenes(args)
    kw = {"--integrator": ("integrator", cli.INTEGRATORS), "--precision": ("precision", cli.PRECISIONS),
          "--schedule": ("schedule", cli.SCHEDULES), "--format": ("format", cli.FORMATS)}
    opts = {"integrator": cli.INTEGRATORS[{"binary": "multi", "flat": "flat"}.get(argv[1], "rk4")]}
    for flag, (name, table) in kw.items():
        if flag in argv:
            opts[name] = table[argv[argv.index(flag) + 1]]
    if "--block" in argv:
        opts["block_x"], opts["block_y"] = (int(v) for v in argv[argv.index("--block") + 1].split("x"))
    for flag, name in (("--step", "step"), ("--max-steps", "max_steps")):
        if flag in argv:
            opts[name] = type(getattr(capi.default_options(), name))(argv[argv.index(flag) + 1])
    ref = renderer.render(scenes[:1], capi.default_options(**opts))[0]
    rgb = read_ppm(tmp_path / "frame_0000.ppm")
    rgba = "--format" in argv and argv[argv.index("--format") + 1] == "rgba8"
    assert np.array_equal(rgb, ref.pixels[..., :3] if rgba else ref.pixels[..., 2::-1])
