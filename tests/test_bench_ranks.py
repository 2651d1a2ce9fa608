"""bench.py's multi-rank host logic on CPU with two gloo ranks: each rank
simulates its own replica (distinct seeds, so distinct networks), timings are
combined as the maximum over ranks, and the reference arm's non-zero ranks
exit without work.  Nothing here needs a GPU."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    from eden_gb300 import lowering, workloads
    dist.init_process_group("gloo")
    seed = bench.replica_seed(1234, rank)
    low = lowering.lower(workloads.multicomp_net(n_cells=20, in_degree=5, length_ms=1.0, seed=seed))
    slowest = bench.max_over_ranks(10.0 + rank, dist)
    out[rank] = (seed, int(low.n_comp), slowest)
    dist.destroy_process_group()


def test_replicas_and_max_over_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    (s0, n0, m0), (s1, n1, m1) = out[0], out[1]
    assert s0 != s1 and n0 != n1          # two different replicas
    assert m0 == m1 == 11.0                # both ranks see the slowest rank's time


def test_reference_arm_other_ranks_exit_without_work():
    port = _free_port()
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK="1", WORLD_SIZE="2",
               LOCAL_RANK="1")
    # rank 1 alone: it must return before touching the process group's peers
    # or the CPU sample, printing nothing
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--cells', '20'];"
            "import torch.distributed as dist; dist.init_process_group = lambda *a, **k: None;"
            "runpy.run_path('bench.py', run_name='__main__')")
    p = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
