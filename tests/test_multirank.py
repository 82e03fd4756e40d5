"""The replicas path of bench.py on CPU: two gloo ranks (no GPU).

`bench.py --gpus N` under torchrun runs one independent mesh build per rank
(no collective on the data path, `scaling: weak`); the only exchange is the
whole-job reduction: the MAX of the timed milliseconds and the SUM of the
vertices over the ranks.  The reference arm runs on rank 0 alone.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        assert (ws, r, local) == (world, rank, rank)
        ms, units = bench.aggregate_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
        out.put((rank, ms, units))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replicas_reduce_max_time_and_sum_units(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, ms, units in res:
        assert ms == 10.0 + 5.0 * (world - 1)
        assert units == 1000 * world * (world + 1) // 2


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"])
    bench.main()
    assert capsys.readouterr().out == ""


def test_reference_arm_json_line(monkeypatch, capsys):
    """Rank 0 of the reference arm times the CPU restatement on the host cores and
    prints one JSON line with the contract's keys; no GPU is involved."""
    import json
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"])
    bench.main()
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "Voronoi vertices/s" and d["unit"] == "vertices/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["config"]["workload"] == "4d_uniform_20000_vertex_search"
