"""The multi-process path of bench.py on CPU (gloo, world size 2): the
barrier and max-over-ranks helpers, and the reference arm under torchrun
(rank 0 alone measures and prints one line)."""
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


def _worker(rank, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, ws, local, dist = bench._dist()
    bench._barrier(dist)
    m = bench._allmax(dist, 1.5 + r)
    out.put((r, ws, local, m))
    dist.destroy_process_group()


def test_dist_helpers_world_size_2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 0, 2.5), (1, 2, 1, 2.5)]


def test_reference_arm_under_torchrun_prints_once(built):
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.5"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_failing_optional_form_is_reported_not_fatal():
    """An optional form (served, batched, precision, pipeline, the CPU leg)
    that raises becomes an error field of the line; the headline line is
    still printed."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench._optional(lambda: {"value": 1.0}) == {"value": 1.0}
    assert bench._optional(lambda x: 1 / x, 0) == {"error": "ZeroDivisionError: division by zero"}
