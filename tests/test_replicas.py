"""bench.py --gpus N runs N independent replicas (no data-path collective): every rank builds its own
world, the job's step time is the slowest rank's (all-reduce MAX) and the whole-job value is
N x units / that time. Checked here with two gloo ranks on CPU (127.0.0.1), each reporting a
different step time."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, rank, world)
    ms = bench.max_over_ranks(1.5 + rank, world)
    out.put((rank, ms, bench.replica_throughput(4096, world, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[0][2] == pytest.approx(2 * 4096 / 2.5e-3)


def test_gpus_flag_launches_that_many_ranks():
    """`bench.py --gpus 2` outside torchrun re-launches itself as two ranks (torch.distributed.run on
    127.0.0.1); the reference arm, which needs no GPU, shows it: rank 0 alone reports, with n_gpus 2."""
    import json
    import subprocess

    env = dict(os.environ)
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["n_gpus"] == 2 and line["impl"] == "reference" and line["steps"] == 1
    assert line["config"]["chunks"] == 4096 and line["config"]["parallelism"] == "replicas"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
