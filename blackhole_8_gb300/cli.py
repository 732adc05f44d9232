"""Headless renderer: the reference's interactive frame loop
(blackhole_solution_test.cc:153-407: render, HUD, VideoWriter, imshow)
without a window. Renders one of the synthetic workloads on the GPU, keeps
frames on the device, optionally copies them out as binary PPM files, and
prints one JSON line of timings.

    python -m blackhole_8_gb300.cli --workload flythrough --frames 8 \
        --precision fp32 --schedule grid --repeat 3 [--ppm DIR]

``--workload adjoint`` runs the differentiable render instead: a target is
rendered (FP64) at M + 5 %, disc tilt + 3 deg, r_outer + 2 M, yaw and pitch
+ 1 deg, then bh_render_adjoint gives the loss and its gradient at the
scene's own parameters (--precision fp32|fp64|mixed), --repeat times.
"""
from __future__ import annotations

import argparse
import json
import os
import time

PRECISIONS = {"fp32": 0, "fp64": 1, "mixed": 2}
SCHEDULES = {"grid": 0, "persistent": 1, "hybrid": 2}
FORMATS = {"bgra8": 0, "bgr8": 1, "rgba8": 2}
INTEGRATORS = {"ref": 0, "rk4": 1, "flat": 2, "multi": 3}


def build_scenes(args):
    from . import scene as S
    if args.workload == "single":
        return [S.single_scene(args.width or 640, args.height or 360)]
    if args.workload == "flythrough":
        sc = S.flythrough(120, args.width or 1920, args.height or 1080)
        idx = [round(i * (len(sc) - 1) / max(1, args.frames - 1)) for i in range(args.frames)]
        return [sc[i] for i in idx]
    if args.workload == "batched":
        return S.batched_scenes(args.frames)
    if args.workload == "photon-ring":
        return [S.photon_ring_scene(args.width or 4096)]
    if args.workload == "impact-grid":
        return [S.impact_grid_scene(args.width or 4096)]
    if args.workload == "objects":
        return [S.objects_scene(args.width or 640, args.height or 360) for _ in range(args.frames)]
    if args.workload == "flat":
        return [S.flat_demo_scene(args.width or 800, args.height or 450) for _ in range(args.frames)]
    if args.workload == "binary":
        return S.binary_orbit(args.frames, args.width or 1920, args.height or 1080)
    raise SystemExit(f"unknown workload {args.workload}")


def write_ppm(path: str, px, rgb_first: bool = False) -> None:
    """px: BGRA8 / BGR8 (or, rgb_first, RGBA8) frame, height x width x channels."""
    h, w = px.shape[:2]
    with open(path, "wb") as fh:
        fh.write(f"P6\n{w} {h}\n255\n".encode())
        fh.write((px[..., :3] if rgb_first else px[..., 2::-1]).tobytes())


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", default="flythrough",
                    choices=["single", "flythrough", "batched", "photon-ring", "impact-grid", "adjoint", "objects",
                             "flat", "binary"])
    ap.add_argument("--frames", type=int, default=8)
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--integrator", default=None, choices=list(INTEGRATORS),
                    help="default: multi for the binary workload, flat for the flat one, rk4 otherwise")
    ap.add_argument("--precision", default="fp32", choices=list(PRECISIONS))
    ap.add_argument("--schedule", default="grid", choices=list(SCHEDULES))
    ap.add_argument("--step", type=float, default=0.01)
    ap.add_argument("--max-steps", type=int, default=4000)
    ap.add_argument("--band", type=float, default=-1)
    ap.add_argument("--setup-band", type=float, default=-1)
    ap.add_argument("--slice", type=int, default=0)
    ap.add_argument("--refill", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--band-serial", action="store_true",
                    help="MIXED + persistent or hybrid: FP32 pass, then FP64 band pass, both host-launched")
    ap.add_argument("--block", default="", help="GRID / HYBRID block shape WxH (default 8x16)")
    ap.add_argument("--rays-per-thread", type=int, default=0, help="GRID / HYBRID block tiles per block")
    ap.add_argument("--format", default="bgra8", choices=list(FORMATS),
                    help="frame layout (bgr8: the reference's CV_8UC3 frames)")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--ppm", default="")
    args = ap.parse_args(argv)
    if args.integrator is None:
        args.integrator = {"binary": "multi", "flat": "flat"}.get(args.workload, "rk4")

    import ctypes as C

    import numpy as np

    from . import build, capi
    from .render import Renderer
    build.build()
    if args.workload == "adjoint":
        return run_adjoint(args)
    scenes = build_scenes(args)
    opts = capi.default_options(integrator=INTEGRATORS[args.integrator], precision=PRECISIONS[args.precision],
                                schedule=SCHEDULES[args.schedule], step=args.step, max_steps=args.max_steps,
                                band=args.band, setup_band=args.setup_band, slice_steps=args.slice,
                                refill_threshold=args.refill, threads_per_block=args.threads,
                                band_serial=int(args.band_serial), rays_per_thread=args.rays_per_thread,
                                format=FORMATS[args.format])
    if args.block:
        opts.block_x, opts.block_y = (int(v) for v in args.block.lower().split("x"))
    with Renderer(0) as r:
        cs = r.c_scenes(scenes)
        import torch
        channels = 3 if args.format == "bgr8" else 4
        bufs = [torch.empty((s.camera.height(), s.camera.width(), channels), dtype=torch.uint8, device="cuda")
                for s in scenes]
        frames = (capi.Frame * len(scenes))()
        for i, b in enumerate(bufs):
            frames[i].pixels = b.data_ptr()
        times = []
        for _ in range(args.repeat):
            r.render_device(cs, frames, opts)
            st = r.stats()
            times.append(st.kernel_ms)
        rays = sum(s.camera.width() * s.camera.height() for s in scenes)
        best = min(times)
        out = {"workload": args.workload, "frames": len(scenes), "rays": rays, "kernel_ms": times,
               "mrays_per_s": rays / (best * 1e-3) / 1e6, "steps": int(st.steps), "band_rays": int(st.band_rays),
               "band_steps": int(st.band_steps),
               "fp32_tflops": st.steps * capi.RK4_FLOPS_PER_STEP / (best * 1e-3) / 1e12}
        if args.ppm:
            os.makedirs(args.ppm, exist_ok=True)
            for i, b in enumerate(bufs):
                write_ppm(os.path.join(args.ppm, f"frame_{i:04d}.ppm"), b.cpu().numpy(),
                          rgb_first=args.format == "rgba8")
        print(json.dumps(out))
    return 0


def run_adjoint(args) -> int:
    import math

    import numpy as np
    import torch

    from . import capi
    from . import scene as S
    from .render import Renderer
    sc = S.single_scene(args.width or 512, args.height or 512)
    th0 = np.array([sc.hole.mass(), 0, 0, 0, 0, 0, 0, 0, sc.disc.r_inner(), sc.disc.r_outer()], dtype=np.float64)
    tt = th0.copy()
    tt[capi.GRAD_MASS] *= 1.05
    tt[capi.GRAD_TILT] += math.radians(3)
    tt[capi.GRAD_R_OUTER] += 2.0
    tt[capi.GRAD_YAW] += math.radians(1)
    tt[capi.GRAD_PITCH] += math.radians(1)
    h, w = sc.camera.height(), sc.camera.width()
    with Renderer(0) as r:
        cs = r.c_scenes([sc])
        target = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
        fr = (capi.AdjointFrame * 1)()
        fr[0].image = target.data_ptr()
        r.render_adjoint(cs, fr, tt[None], capi.adjoint_options(precision=capi.PRECISION_FP64, max_steps=args.max_steps,
                                                                step=args.step))
        fr = (capi.AdjointFrame * 1)()
        fr[0].target = target.data_ptr()
        opts = capi.adjoint_options(precision=PRECISIONS[args.precision], max_steps=args.max_steps, step=args.step)
        if args.band >= 0:
            opts.band = args.band
        times = []
        for _ in range(args.repeat):
            res = r.render_adjoint(cs, fr, th0[None], opts)[0]
            times.append(res.kernel_ms)
        out = {"workload": "adjoint", "width": w, "height": h, "precision": args.precision, "kernel_ms": times,
               "mrays_per_s": w * h / (min(times) * 1e-3) / 1e6, "loss": res.loss,
               "grad": dict(zip(capi.GRAD_NAMES, list(res.grad))), "steps": int(res.steps),
               "band_rays": int(res.band_rays)}
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
