"""The N > 1 path of bench.py on CPU: world size 2 over gloo.

bench.py runs one independent replica per rank (no data-path collective); the
ranks meet only at the barrier around the timed region and in the max over
ranks of the step time.  These tests run those pieces as two real processes
with the gloo backend, and the reference arm under torchrun, where rank 0
alone does the work and prints the line."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_env()
    d = bench.Dist(ws)
    d.barrier()
    m = d.max(10.0 * rank + 1.5)  # rank 1's "step time" is the larger
    d.barrier()
    d.close()
    q.put((r, ws, m))


def test_dist_barrier_and_max_over_two_gloo_ranks():
    port = free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2, 11.5), (1, 2, 11.5)]


def test_reference_arm_under_torchrun_prints_one_line_from_rank0():
    pytest.importorskip("torch")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--case", "small"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["value"] > 0
    # the same config as the GPU arm's line at the same size and rank count
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.headline_config(2048, 2)
