"""Multi-process (replicas) path of bench.py on CPU with the gloo backend, world size 2.

The single-system step does not shard; several GPUs run independent replicas whose body-step
counts are summed and whose times are max-reduced over ranks. These tests run that host logic
without a GPU: the reductions themselves, and the reference arm under torchrun (rank 0 alone
works and prints one line; the other rank exits 0)."""
import json
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


def _worker(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    out[rank] = (d.max(rank + 1.5), d.sum(rank + 1.0), d.ws, d.rank)
    d.td.destroy_process_group()


def test_dist_reductions_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as mgr:
        out = mgr.dict()
        port = free_port()
        procs = [mp.Process(target=_worker, args=(r, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0][:3] == (2.5, 3.0, 2) and out[1][:3] == (2.5, 3.0, 2)
        assert {out[0][3], out[1][3]} == {0, 1}


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--gpus", "2",
           "--impl", "reference", "--workload", "plummer-16k", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["value"] > 0 and d["config"]["workload"] == "plummer-16k"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
