"""The replica path of bench.py on two CPU ranks (gloo): bench.Dist initialises from the torchrun
environment, its barrier returns on both ranks, its max-over-ranks reduction gives every rank the
largest value (the timing rule of the benchmark), and it closes cleanly. The solve itself does not
shard (one replica per GPU), so this is the whole multi-process path."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    os.environ["CUDA_VISIBLE_DEVICES"] = ""   # gloo on the host, whatever the machine has
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    assert d.world == world and d.rank == rank and d.pg is not None
    d.barrier()
    v = d.max(float(10 * rank + 1))
    d.barrier()
    d.close()
    out.put((rank, v))


def test_dist_two_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = dict(q.get(timeout=5) for _ in procs)
    assert got == {0: 11.0, 1: 11.0}


def test_bench_rejects_gpus_without_ranks():
    import subprocess
    env = dict(os.environ, WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "WORLD_SIZE" in r.stderr
