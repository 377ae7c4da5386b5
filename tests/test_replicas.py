"""Replicas over several ranks (CPU, gloo, world size 2): every rank works on
its own slice with no data-path exchange; the timed duration is the max over
ranks and the throughput counts every rank's units."""
import multiprocessing as mp
import os
import socket

import pytest

from relxill_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = replicas.rank_info()
    seeds = replicas.rank_seeds(r)
    lo, hi = replicas.set_range(r, w, 10)
    t = replicas.max_over_ranks(1.0 + r, dist)  # rank 1 is the slow one
    v = replicas.job_throughput(hi - lo, 3, w, t)
    q.put((r, w, local, seeds, (lo, hi), t, v))
    dist.destroy_process_group()


def test_two_rank_replicas_on_gloo():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    (r0, w0, l0, s0, sl0, t0, v0), (r1, w1, l1, s1, sl1, t1, v1) = out
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert s0 != s1                        # different slices of the workload
    assert sl0 == (0, 5) and sl1 == (5, 10)
    assert t0 == t1 == 2.0                 # the slowest rank's time on every rank
    assert v0 == v1 == 2 * 5 * 3 / 2.0     # all ranks' units over that time


def test_set_ranges_cover_the_batch():
    for world in (1, 2, 3, 8):
        for n in (0, 1, 7, 4096):
            spans = [replicas.set_range(r, world, n) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1


def test_single_process_max_is_identity():
    assert replicas.max_over_ranks(3.5) == 3.5


def test_bench_gpus_two_spawns_two_ranks():
    """bench.py --gpus 2 without a launcher starts two ranks through torch.distributed.run (here with
    the GPU work replaced by the dry run): the line reports both ranks."""
    pytest.importorskip("torch")
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--steps", "3", "--warmup", "1",
                        "--sets", "16", "--dry-run"], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    assert lines[0]["n_gpus"] == 2 and lines[0]["ranks"] == 2
    assert abs(lines[0]["value"] - 2 * 16 * 3 / (3 * 0.01)) / lines[0]["value"] < 0.5
