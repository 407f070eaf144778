"""bench.py's multi-GPU path (replicas, one process per GPU) on CPU with a
two-rank gloo group: barrier, max / sum over ranks, the whole-job throughput
(bonds of every rank's specimen x steps / slowest rank's time) on per-rank
specimens (seed = rank) stepped by the oracle, and the reference arm's rule
that only rank 0 runs and prints under torchrun."""
import os
import socket
import subprocess
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle as orc
    r = bench.Ranks(world, "cpu")
    r.barrier()
    mx, sm = r.max(float(rank + 1)), r.sum(float(rank + 1))
    p = bench.problem(40, seed=rank)
    o = orc.OracleFD(p)
    o.run(1)
    t0 = time.perf_counter()
    o.run(5)
    dt = time.perf_counter() - t0
    val = bench.throughput(o.nnz(), 5, dt, r)
    q.put((rank, mx, sm, val, r.sum(float(o.nnz())), r.max(dt), o.state()[0][:4].tolist()))
    r.barrier()
    dist.destroy_process_group()


def test_replicas_reduce_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(k, 2, port, q)) for k in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for rank, mx, sm, val, nnz_all, dt_max, u in res:
        assert mx == 2.0 and sm == 3.0
        assert val == pytest.approx(nnz_all * 5 / dt_max, rel=1e-12)
    assert res[0][3] == res[1][3]          # every rank reports the job's value
    assert res[0][6] != res[1][6]          # seed = rank: different specimens


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--gpus", "2", "--steps", "2", "--warmup", "1"],
                         env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == ""
