"""Test infrastructure: replays a mirror Scene on the reference's own code.

Writes the scene in ``ref_runner``'s text format (the pose operations logged
by the mirror objects are replayed on the reference's Camera and Annulus) and
runs ``oracle/_ref/ref_runner`` (built by ``oracle/build_ref.py``) in a
fresh process per call: the reference's ObjectManager is a process-wide
singleton with no removal, so one process holds one scene.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

from . import build_ref


def available() -> bool:
    return os.path.exists(build_ref.RUNNER) or build_ref.build() is not None


def runner() -> str:
    path = build_ref.build()
    if path is None:
        raise RuntimeError("the reference runner is not built and the reference sources are absent")
    return path


def _op_line(op) -> str:
    return " ".join([op[0]] + [repr(float(a)) for a in op[1:]])


def _floats(ps) -> str:
    return " ".join(repr(float(x)) for p in ps for x in p)


def write_scene(path: str, scenes, tex_path: str, flat: bool = False) -> None:
    from blackhole_8_gb300 import scene as S
    s0 = scenes[0]
    d = s0.disc
    lines = [f"mode {'flat' if flat else 'curved'}",
             f"image {s0.camera.width()} {s0.camera.height()}",
             f"fov {s0.camera.fov()!r}",
             "bh " + " ".join(repr(float(x)) for x in s0.hole.position()) + f" {s0.hole.mass()!r}"]
    if d is not None:
        tex = d.texture.bgra()[..., :3]
        tex.tofile(tex_path)
        lines.append("disc " + _floats(d.construction) + f" {d.r_outer()!r} {d.r_inner()!r}")
        for op in d.ops:
            lines.append("disc_op " + _op_line(op))
        lines.append(f"texture {tex_path} {tex.shape[1]} {tex.shape[0]}")
    for k, o in enumerate(s0.objects):
        if isinstance(o, S.Rectangle):
            if o.texture is not None:
                t = o.texture.bgra()[..., :3]
                tp = f"{tex_path}.obj{k}"
                t.tofile(tp)
                tex_spec = f"{tp} {t.shape[1]} {t.shape[0]}"
            else:
                tex_spec = "- 0 0"
            lines.append("rect " + _floats(o.construction) + " " + tex_spec)
        elif isinstance(o, S.InfinitePlane):
            size = o.pattern.pattern_size if o.pattern is not None else 0
            if size != int(size):
                raise ValueError("the reference's ChessPattern2D takes an integer size")
            lines.append("plane " + _floats(o.construction) + f" {int(size)}")
        else:
            raise ValueError(f"the reference cannot build {type(o).__name__}")
        for op in o.ops:
            lines.append("obj_op " + _op_line(op))
    lines.append(f"frames {len(scenes)}")
    for s in scenes:
        if (s.camera.width(), s.camera.height()) != (s0.camera.width(), s0.camera.height()):
            raise ValueError("one runner call renders frames of one size")
        ops = [op for op in s.camera.ops if op[0] != "Fov"]
        fov_ops = [("Fov", s.camera.fov())] if s.camera.fov() != s0.camera.fov() else []
        all_ops = fov_ops + ops
        lines.append(f"frame {len(all_ops)} " + " ".join(_op_line(op) for op in all_ops))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def render(scenes, tag: bool = False, threads: int = 0, timed: bool = False, flat: bool = False):
    """Runs the reference loop (flat: its RayTracer); returns (frames uint8
    [F,H,W,3] BGR, timing). Objects and the disc are taken from the first
    scene; frames differ by their camera."""
    if not isinstance(scenes, (list, tuple)):
        scenes = [scenes]
    with tempfile.TemporaryDirectory() as td:
        sp, tp, op = (os.path.join(td, n) for n in ("scene.txt", "tex.bin", "out.bin"))
        write_scene(sp, scenes, tp, flat=flat)
        cmd = [runner(), sp, op]
        if tag:
            cmd.append("--tag")
        if threads:
            cmd += ["--threads", str(threads)]
        if timed:
            cmd.append("--time")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_runner failed: {r.stderr}")
        h, w = scenes[0].camera.height(), scenes[0].camera.width()
        frames = np.fromfile(op, dtype=np.uint8).reshape(len(scenes), h, w, 3)
        timing = json.loads(r.stdout) if timed else None
    return frames, timing


def render_with_classes(scene, threads: int = 0, flat: bool = False, with_objects: bool = False):
    """(BGR image, class per pixel) of one scene from two runner passes;
    with_objects adds the object index per pixel (-1 elsewhere)."""
    img, _ = render([scene], threads=threads, flat=flat)
    tag, _ = render([scene], tag=True, threads=threads, flat=flat)
    cls = tag[0][..., 0].copy()
    if not with_objects:
        return img[0], cls
    idx = np.where(cls == 4, tag[0][..., 1].astype(np.int32), -1)
    return img[0], cls, idx
