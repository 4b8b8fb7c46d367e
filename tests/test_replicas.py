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


def _reference_arm(extra_env, nproc):
    import json
    import subprocess
    import sys
    env = dict(os.environ, **extra_env)
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--workload", "j1j2_L24_k0_p1_z1",
           "--steps", "3", "--warmup", "3"]
    if nproc > 1:
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
               "--master-addr", "127.0.0.1", f"--master-port={_free_port()}"] + cmd[1:] + ["--gpus", str(nproc)]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference`: the oracle's restatement of the reference
    product on the host cores prints one JSON line with the arm's keys."""
    lines = _reference_arm({}, 1)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 3 and d["warmup"] >= 3
    assert d["config"]["N"] == 28968
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_under_two_ranks_prints_once():
    """Launched with two ranks (gloo here), rank 0 alone runs the reference
    arm and prints its line; the other rank exits 0 without work."""
    lines = _reference_arm({"QS_BENCH_BACKEND": "gloo"}, 2)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
