"""The multi-GPU path of bench.py is replicas only: N independent
processes, one per GPU, joined by gloo for the barrier and the max / sum of
their timings (no collective on the data path).  These tests run that
plumbing on the CPU with two gloo ranks."""
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


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_setup()
    bench.barrier(w)
    mx = bench.allreduce(float(r + 1), "max", w)
    sm = bench.allreduce(float(10 * (r + 1)), "sum", w)
    bench.barrier(w)
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump({"rank": r, "world": w, "local": local, "max": mx, "sum": sm}, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_gloo_max_and_sum_over_two_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        d = json.load(open(tmp_path / f"rank{r}.json"))
        assert d["world"] == 2 and d["local"] == r
        assert d["max"] == 2.0 and d["sum"] == 30.0


def test_reference_arm_under_torchrun_prints_one_line():
    """bench.py --impl reference launched through torchrun for N=2:
    rank 0 alone times the CPU reference and prints one JSON line; the
    other rank exits 0."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
