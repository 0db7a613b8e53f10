"""The multi-rank path of bench.py on CPU (gloo, world size 2): one replica
per rank, no data-path collective; the whole-job rate is all ranks' cell
updates over the slowest rank's time, and the reference arm runs on rank 0
only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, _, dist = bench.dist_setup(world)
    assert (w, r) == (world, rank)
    # rank r did (r + 1) * 1e9 cell updates in (r + 1) * 0.5 s
    rate, t_max = bench.replica_throughput(dist, (rank + 1) * 1e9, (rank + 1) * 0.5)
    bench.barrier(dist)
    out.put((rank, rate, t_max))
    dist.destroy_process_group()


def test_replica_throughput_gloo():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, rate, t_max in res:
        assert t_max == pytest.approx(1.0)                 # slowest rank
        assert rate == pytest.approx(3e9 / 1.0)            # all ranks' updates / slowest time


def test_reference_arm_rank0_only():
    """bench.py --impl reference under torchrun (2 ranks, gloo): exactly one
    JSON line, from rank 0, and every rank exits 0."""
    oracle_so = ROOT / "oracle" / "liboracle.so"
    if not oracle_so.exists():
        pytest.skip("oracle not built")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--size", "256"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0
