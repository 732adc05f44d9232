"""bench.py with several ranks (one replica of the fly-through per GPU, no
collective on the data path): the step time is the slowest rank's, the
whole-job throughput counts every rank's rays, and the reference arm runs on
rank 0 alone. Checked with two gloo ranks on the CPU (127.0.0.1)."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r reports a step of (r + 1) ms: the job takes the slowest
        t = bench.max_over_ranks((rank + 1) * 1e-3, world, device="cpu")
        q.put((rank, t, bench.job_throughput(1000, world, t)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in procs)
    assert [g[1] for g in got] == [2e-3, 2e-3]
    assert all(abs(g[2] - 1000 * 2 / 2e-3 / 1e6) < 1e-9 for g in got)  # 1 Mrays/s


def test_single_rank_is_identity():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(2_000_000, 1, 0.5) == 4.0


def test_reference_arm_runs_on_rank_0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_line_has_the_contract_keys():
    """The reference arm (the reference's own loop on the host cores) prints
    one JSON line with the benchmark's keys, its cpu_baseline and an e2e
    with no device copies."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    if "unavailable" in line:
        pytest.skip(line["unavailable"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Mrays/s"
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
