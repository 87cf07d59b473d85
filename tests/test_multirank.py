"""The N > 1 path of the benchmark on CPU ranks (gloo): replicas only, so the only exchanges
are the barrier and the max-over-ranks reduction of the timed region; the whole-job rate counts
every rank's frames against the slowest rank's time.  The reference arm under torchrun runs on
rank 0 alone and prints one line; the other rank exits without work."""
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


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        dist.barrier()
        ms = 100.0 + 50.0 * rank                   # rank 1 is the slow replica
        slowest = bench.max_over_ranks(ms, ws, device="cpu")
        out.put((rank, slowest, bench.whole_job_rate(ws, 20, slowest)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate in res:
        assert slowest == 150.0
        assert rate == pytest.approx(2 * 20 / 0.150)


def test_single_rank_is_a_no_op():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(123.5, 1) == 123.5
    assert bench.whole_job_rate(1, 10, 500.0) == pytest.approx(20.0)


def test_reference_arm_on_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--width", "128", "--height", "72"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
