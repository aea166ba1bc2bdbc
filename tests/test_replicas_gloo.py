"""Replica timing across ranks (bench.py --gpus N under torchrun) with two gloo
processes on the CPU: the barrier, the max-over-ranks of the elapsed time that
every rank reports, and the whole-job throughput it implies. The reference arm
under torchrun runs on rank 0 only; another rank exits without output."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from stratusgfx_gb300 import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    replicas.barrier()
    elapsed = 10.0 + 5.0 * rank                      # rank 1 is the slower replica
    worst = replicas.max_over_ranks(elapsed)
    value = replicas.job_throughput(1000.0, world, worst)
    q.put((rank, worst, value))
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_with_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]        # both ranks see the slowest time
    assert [r[2] for r in res] == [2 * 1000.0 / 0.015] * 2


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    from stratusgfx_gb300 import replicas
    assert replicas.max_over_ranks(3.5) == 3.5
    replicas.barrier()
    assert replicas.job_throughput(10.0, 1, 1000.0) == 10.0
    with pytest.raises(ValueError):
        replicas.job_throughput(10.0, 1, 0.0)


def test_reference_arm_prints_only_on_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
