"""Replica aggregation of bench.py across ranks (gloo, world size 2, CPU):
each rank runs its own system; the job time is the slowest rank's."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    # rank r took (r + 1) s for its timed steps and (r + 1) * 0.5 s end to end
    value, e2e, total_s, t_e2e = bench.replica_rates(ws, 10, 3, 1024, float(rank + 1),
                                                     0.5 * (rank + 1), torch.device("cpu"))
    out[rank] = (value, e2e, total_s, t_e2e)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rates_take_the_slowest_rank():
    ws = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    pairs = 1024.0 ** 2
    for r in range(ws):
        value, e2e, total_s, t_e2e = res[r]
        assert total_s == 2.0 and t_e2e == 1.0
        assert value == pytest.approx(ws * 10 * pairs / 2.0 / 1e9)
        assert e2e == pytest.approx(ws * 3 * pairs / 1.0 / 1e9)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench

    value, e2e, total_s, t_e2e = bench.replica_rates(1, 4, 2, 2048, 2.0, 1.0, None)
    assert (total_s, t_e2e) == (2.0, 1.0)
    assert value == pytest.approx(4 * 2048.0 ** 2 / 2.0 / 1e9)


def test_bench_gpus_2_relaunches_replicas_and_takes_the_max():
    """`bench.py --gpus 2` started as one process re-launches itself as two
    replica ranks (torch.distributed.run, gloo in the host-only dry run) and
    reports n_gpus = 2 with the slower rank's time (rank 1 takes 100 ms)."""
    import json
    import subprocess

    env = {k: v for k, v in os.environ.items()
           if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--steps", "4",
                        "--warmup", "3", "--dry-run"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(s) for s in r.stdout.splitlines() if s.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["n_gpus"] == 2 and line["dry_run"]
    job_s = line["ms_per_step"] * line["steps"] / 1e3
    assert 0.1 <= job_s < 1.0  # the slower rank's 100 ms, not rank 0's 50 ms


def test_bench_rejects_a_world_size_that_differs_from_gpus():
    import subprocess

    env = dict(os.environ, WORLD_SIZE="3", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--dry-run"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 2 and "WORLD_SIZE" in r.stderr
