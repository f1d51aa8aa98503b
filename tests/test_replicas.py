"""The N > 1 path of bench.py, on the CPU with gloo (world size 2).

bench.py runs one independent solve per rank (replicas: a mesh is not
decomposed), takes the maximum of the timed region over ranks and reports the
aggregate.  These tests run its rank helpers in two gloo processes, and the
whole torchrun launch of the reference arm (host-only), which rank 0 alone
runs and prints.
"""

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    class A:
        pass

    w, r, local, dist = bench.dist_setup(A())
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(dist)
    got = bench.reduce_max(dist, 1.5 + rank)
    bench.barrier(dist)
    dist.destroy_process_group()
    out.put((rank, got))


def test_rank_helpers_two_gloo_processes():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, out))
             for k in range(2)]
    for p in procs:
        p.start()
    res = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 2.5, 1: 2.5}


def test_torchrun_reference_arm_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(_free_port()), "bench.py", "--impl",
           "reference", "--workload", "tube1d", "--gpus", "2",
           "--cpu-nside", "1001", "--steps", "3", "--warmup", "3"]
    run = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [json.loads(x) for x in run.stdout.splitlines()
             if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["metric"] == "point-steps/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_gpus_flag_launches_its_own_ranks():
    """``bench.py --gpus 2`` without a launcher starts its two ranks itself
    and prints one line for both."""
    pytest.importorskip("torch")
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR",
              "MASTER_PORT"):
        env.pop(k, None)
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--workload",
           "tube1d", "--gpus", "2", "--cpu-nside", "1001", "--steps", "3",
           "--warmup", "3"]
    run = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True,
                         timeout=600, env=env)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [json.loads(x) for x in run.stdout.splitlines()
             if x.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["n_gpus"] == 2 and lines[0]["impl"] == "reference"


def test_warmup_below_three_is_rejected():
    run = subprocess.run([sys.executable, "bench.py", "--impl", "reference",
                          "--workload", "tube1d", "--warmup", "2",
                          "--steps", "3"], cwd=ROOT, capture_output=True,
                         text=True, timeout=120)
    assert run.returncode != 0
    assert "--warmup must be at least 3" in run.stderr
