"""Multi-rank logic of bench.py (replicas, no data-path collective) on CPU
with the gloo backend, world size 2."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank), BGEMM_BENCH_BACKEND="gloo")
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, local = bench.dist_init(world)
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(w)
    # rank 1 is slower; the job rate is both ranks' work over the slower time
    ms = 10.0 if rank == 0 else 20.0
    tflops, ms_max = bench.whole_job_tflops(1e12, ms, w, device="cpu")
    q.put((rank, tflops, ms_max))
    dist.destroy_process_group()


def test_replica_timing_gloo_world2():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tflops, ms_max in out:
        assert ms_max == 20.0
        assert abs(tflops - 2 * 1e12 / 20e-3 / 1e12) < 1e-9


def test_single_rank_identity():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    tflops, ms = bench.whole_job_tflops(2e12, 4.0, 1)
    assert ms == 4.0 and abs(tflops - 500.0) < 1e-9
