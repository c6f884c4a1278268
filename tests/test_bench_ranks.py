"""Replica bench on several ranks: the host-side reduction, on CPU with gloo.

The GB300 path runs one replica per rank (the path does not shard); the bench
line reports every rank's discs over the slowest rank's time. Two gloo ranks
check that reduction and the aggregate formula without a GPU.
"""

import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    try:
        w, r, _ = bench._dist()
        assert (w, r) == (world, rank)
        slowest = bench.max_over_ranks(1.0 + rank, "cpu")  # rank 1 is the slow one
        rate = bench.aggregate_rate(w, 1000, 10, slowest)
        out.put((rank, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_aggregate_over_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [2.0, 2.0]
    assert all(abs(g[2] - 2 * 1000 * 10 / 2.0) < 1e-9 for g in got)


def test_single_process_reduction_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.aggregate_rate(1, 100, 10, 2.0) == 500.0


def test_cpu_baseline_runs_the_oracle_on_every_requested_core():
    """The reference arm's sample: slabs of equal disc count, one spawned
    process per core, all discs counted once."""
    import bench
    r = bench.cpu_oracle_rate(2, n_side=32, workers=2)
    assert r["cores"] == 2 and r["kind"] == "port" and r["value"] > 0
    assert "1,024-disc case" in r["sample"] and "2 vertical slabs" in r["sample"]
    assert bench.host_cores() >= 1


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the bench's reference arm) prints one
    JSON line with the GPU arm's metric and unit, a cpu_baseline object
    describing its own run and an e2e object with no host-device copies."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                         cwd=root, capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "particle-steps/s @1M discs" and d["unit"] == "particle-steps/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1 and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
