"""The multi-GPU form is replicas only: every rank renders its own frames and the job's
rate is all ranks' frames over the slowest rank's time.  Its host logic (the max over
ranks, the whole-job rate, the reference arm printing from rank 0 alone) runs here on
CPU with gloo ranks on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    # rank r took (r + 1) seconds for 10 frames and (2 - r) for the e2e leg
    times = bench.max_over_ranks([float(rank + 1), float(2 - rank)], "cpu", ws)
    rate = bench.whole_job_rate(10, ws, times[0])
    out.put((rank, times, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, rate in res:
        assert times == [2.0, 2.0]            # the slowest rank of each leg
        assert rate == pytest.approx(2 * 10 / 2.0)


def test_single_rank_is_a_no_op():
    import bench
    assert bench.max_over_ranks([1.5, 2.5], "cpu", 1) == [1.5, 2.5]
    assert bench.whole_job_rate(200, 1, 0.5) == 400.0


def test_reference_arm_prints_from_rank_zero_only():
    """`bench.py --impl reference` under torch.distributed.run with two ranks: rank 0
    times the CPU reference on a small sample and prints one line; rank 1 exits 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={free_port()}", str(ROOT / "bench.py"), "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--ref-sample-den", "8192",
           "--no-full-frame"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
