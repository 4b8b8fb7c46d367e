"""bench.py's replica harness on two CPU processes (gloo): the barrier, the
max over ranks of the step time, and the whole-job value computed from it."""
import multiprocessing as mp
import os
import socket

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), QS_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    t_step = bench.max_over_ranks(w, 0.001 * (r + 1))   # rank 1 is the slow replica
    q.put((r, t_step, bench.replica_value(w, 5e8, t_step)))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_step, value in out:
        assert t_step == 0.002
        # two replicas of 0.5 GB per step in 2 ms each: 500 GB/s for the job
        assert abs(value - 500.0) < 1e-9


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1, 0.25) == 0.25
    assert abs(bench.replica_value(1, 1e9, 0.5) - 2.0) < 1e-12
