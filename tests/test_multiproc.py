"""CPU tests of the multi-process (N > 1) host logic of bench.py.  The path
runs independent replicas, one per GPU, so the only cross-rank step is the
job time: the slowest rank's, one max all-reduce.  gloo ranks on the CPU
stand in for the NCCL ranks of a multi-GPU run."""
import json
import multiprocessing as mp
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


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    try:
        q.put((rank, bench.replica_throughput(1000, 10.0 + 5.0 * rank, world)))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _ in out) == [0, 1]
    for _, (value, ms) in out:
        assert ms == 15.0                      # the slowest rank's time
        assert value == pytest.approx(2 * 1000 / 0.015)  # both ranks' units


def test_replica_throughput_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(1000, 10.0, 1) == (pytest.approx(1e5), 10.0)


def test_reference_arm_under_torchrun_prints_one_line():
    """Under torchrun with two ranks the reference arm runs on rank 0 only
    and prints one JSON line; the other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--config", "c1", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    for key in ("metric", "unit", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config"):
        assert key in d, key
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"],
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
