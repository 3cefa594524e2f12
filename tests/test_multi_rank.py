"""The multi-GPU contract on the host: replicas only (states, flamelets and
requests are independent, so no data-path collective), a barrier and a
max-over-ranks of the timings.  Two gloo ranks on the CPU exercise
``bench.py``'s process-group plumbing, and the reference arm under the
launcher the driver uses (``torch.distributed.run``, two ranks): rank 0
alone prints the one JSON line, the other rank exits 0 without work."""

import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world),
                       "LOCAL_RANK": str(rank), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.dist_info()
    dist = bench.init_dist(w)
    try:
        bench.barrier(dist)
        # each rank's "timing" differs; every rank sees the maximum
        got = bench.max_over_ranks(dist, 10.0 + r, torch.device("cpu"))
        q.put((r, w, got))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 2, 11.0), (1, 2, 11.0)]


def test_reference_arm_under_the_launcher():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cpu-seconds", "0.2"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
