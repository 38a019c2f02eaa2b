"""bench.py host logic without a GPU: replica runs (one process per GPU, no data-path collective) with the
timing reduction across ranks exercised by two CPU ranks over gloo; the reference arm's rank rule (rank 0
alone measures and prints; the other ranks exit 0 without work) and its JSON line."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench

    # each rank's mean step time; the job is as slow as its slowest replica
    ms = bench.barrier_max(1.5 + rank, world, None)
    q.put((rank, ms, world * 1000 / (ms / 1e3)))
    dist.destroy_process_group()


def test_step_time_is_the_maximum_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [2.5, 2.5]
    # value = the events of all replicas over the slowest replica's time
    assert got[0][2] == pytest.approx(2 * 1000 / 2.5e-3)


def test_reference_arm_prints_only_on_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference"], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_json_line_contract():
    """The reference arm (FP64 restatement of the reference's CPU path on the host cores) prints one JSON
    line with the engine arm's metric and unit, its own cpu_baseline and an e2e entry without copies."""
    import json

    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "3", "--warmup", "3",
                        "--ref-sample", "3000"], env=env, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    sys.path.insert(0, str(ROOT))
    import bench

    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "event-NLL evals/s"
    assert d["steps"] == 3 and d["warmup"] == 3 and d["higher_is_better"] is True and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["cpu_baseline"]["cores"] >= 1 and "3000 events" in d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == bench.WORKLOAD
