"""Multi-GPU is replicas only: each rank runs the whole workload on its own GPU
and the job's time is the slowest rank's (no data-path collective). The
host-side logic runs here as world_size-2 gloo ranks on CPU."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(times[rank], dist)
    dist.barrier()
    out.put((rank, got))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [1.25, 3.5]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 3.5, 1: 3.5}


def test_max_over_ranks_without_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.0, None) == 2.0


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--bursts", "1000"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


@pytest.mark.parametrize("rank", [0])
def test_reference_arm_rank0_prints_one_line(rank):
    import json
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--bursts", "2000"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def _replica_main(rank, world, port, out):
    """One replica: the whole (small) photon workload on this rank, the oracle
    standing in for the GPU engine, timed, then max over ranks."""
    import time

    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import build_oracle
    build_oracle.build()
    import orc

    from gsmfretda_gb300 import synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bs, n, args, md, S = synth.photon_3state(B=500, seed=2)
    m = orc.model(**md)
    dist.barrier()
    t0 = time.perf_counter()
    h, _ = orc.run_pda(bs.N, bs.T, n, args, m, 1, 8, 20_000, off_idx=bs.off_idx,
                       offsets=bs.offsets, nthreads=1)
    dt = time.perf_counter() - t0 + 0.05 * rank       # rank 1 is the slower one
    total = bench.max_over_ranks(dt, dist)
    value = bench.replica_value(bs.B * 8, 1, total, world)
    out.put((rank, h[0].tolist(), dt, total, value))
    dist.destroy_process_group()


def test_replicas_on_cpu_ranks_gloo_world2():
    """Two replica ranks run the same workload at the same seed: identical
    histograms, the job time is the slower rank's and the job value counts
    both ranks' units."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {r[0]: r[1:] for r in (q.get(timeout=180) for _ in procs)}
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] == res[1][0]
    slow = max(res[0][1], res[1][1])
    for r in (0, 1):
        assert res[r][2] == slow
        assert abs(res[r][3] - 2 * 500 * 8 / slow) < 1e-6 * res[r][3]
