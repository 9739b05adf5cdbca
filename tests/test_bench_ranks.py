"""bench.py across ranks, on the CPU (gloo): the replicas' timing protocol
(barriers, the maximum of the per-rank times, the whole-job throughput) and
the reference arm under torchrun with two ranks (rank 0 alone works and
prints one line; the other ranks exit 0)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r = bench.Ranks(world, "cpu")
    r.barrier()
    t = r.max(0.5 + rank)  # the slowest rank decides
    r.barrier()
    out.put((rank, t, bench.replicas_value(world, 3, t)))
    dist.destroy_process_group()


def test_ranks_max_and_value_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in res] == [1.5, 1.5]
    assert all(abs(v - 2 * 3 / 1.5) < 1e-12 for _, _, v in res)


def test_reference_arm_two_ranks():
    import __graft_entry__  # noqa: F401  (puts the repo on the path)
    import oracle
    oracle.build()
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1", "--nx", "16"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    # every step is a complete solve: the timed region is the steps themselves
    assert d["steps"] == 2 and d["warmup"] == 1 and len(d["step_s"]) == 2
    assert abs(d["ms_per_step"] / 1e3 - sum(d["step_s"]) / 2) < 0.05 * d["ms_per_step"] / 1e3 + 0.01
    # the config both arms print, for N = 2 replicas
    import bench
    assert d["config"] == json.loads(json.dumps(bench.bench_config(2)))
