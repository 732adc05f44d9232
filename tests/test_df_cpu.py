"""The double-float arithmetic of blackhole_8_gb300/csrc/bh_df.cuh, compiled
for the CPU from the same source (tests/cpp/df_check.cc). The mixed tracer's
FP32 passes take the first integral of near-critical rays and refine crossings
near the disc edges in it, and the band pass integrates in it, so it must
carry ~48 significant bits:
- df_add / df_mul / df_div within a few 1e-14 relative (2^-46 .. 2^-45);
- the first integral eps = (M/b)^2 - 1/27 from the per-scene quadratic forms
  of |e|^2 and |F x e|^2 (resolve_derived) within 1e-14 of FP64 wherever the
  tracer takes it (|b - b_c| < 0.5 M): the FP64 band's edges in eps are
  ~1e-7 apart, and a decision must not depend on rounding;
- RK4 in double-float (the tracer's Nystrom operations) within 5e-7 rad of FP64
  RK4 in the escape angle down to |b - b_c| = 1e-6 M and within 1e-6 rad down
  to 1e-7 M, where the band pass hands its rays to FP64."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "df_check.cc")
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = tmp_path_factory.mktemp("df") / "df_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "blackhole_8_gb300", "csrc"), "-I", CUDA_INC, SRC, "-o", str(out)],
                   check=True)
    return str(out)


def _run(exe, mode):
    line = subprocess.run([exe, mode], capture_output=True, text=True, check=True).stdout.split()
    return {line[i]: float(line[i + 1]) for i in range(0, len(line), 2)}


def test_df_arithmetic(exe):
    r = _run(exe, "arith")
    assert r["add"] <= 2e-14 and r["mul"] <= 2e-14 and r["div"] <= 5e-14, r


def test_df_first_integral(exe):
    r = _run(exe, "eps")
    assert r["near"] > 1000
    assert r["eps_abs"] <= 1e-14, r
    assert r["eps_rel"] <= 1e-12, r


def test_df_rk4_against_fp64(exe):
    r = _run(exe, "rk4")
    assert r["rk4_phi"] <= 5e-7, r
    assert r["rk4_phi_near"] <= 1e-6, r
