"""The bench's multi-rank path on the CPU: two gloo ranks.

Independent sweeps shard across GPUs with no exchange (replicas), so the only
cross-rank step is the bench's own aggregation: the timed region's maximum
over ranks and the sum of the frames every rank processed. These run here as
two processes over gloo, and the reference arm is checked to leave every rank
but rank 0 without work.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        elapsed = bench.max_over_ranks(10.0 + 5.0 * rank, w)
        frames = bench.sum_over_ranks(16.0 * (rank + 1), w)
        dist.barrier()
        out.put((r, w, local, elapsed, frames))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_bench():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert [g[0] for g in got] == [0, 1]
    for r, w, local, elapsed, frames in got:
        assert w == 2 and local == r
        assert elapsed == 15.0          # the slowest rank sets the time
        assert frames == 16.0 + 32.0    # every rank's frames count


def test_reference_arm_runs_on_rank_0_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.main(["--impl", "reference", "--gpus", "2", "--steps", "1",
                       "--warmup", "0"]) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_line_on_rank_0(monkeypatch, capsys):
    """At N=1 the reference arm prints one line in the bench's contract: the
    CPU port's frames/s as the value, described by its cpu_baseline, and an
    e2e with no device copies."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    assert bench.main(["--impl", "reference", "--steps", "1", "--warmup", "0"]) == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "frames/s" and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "frames/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("eiger_16m")


def test_our_arm_fails_loudly_without_a_device(monkeypatch):
    """No CPU stand-in: without a usable GPU the bench's own arm stops with the
    reason instead of printing a line."""
    sys.path.insert(0, ROOT)
    import bench
    from sfgb import api
    if api.available():
        pytest.skip("a device is present")
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    with pytest.raises(SystemExit, match="no usable GB300"):
        bench.main(["--steps", "1", "--warmup", "0"])
