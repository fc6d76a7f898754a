"""The N > 1 path of bench.py on the CPU: world-size-2 gloo process groups.

Each rank of a replicas run times its own domain; rank 0 prints the whole
job's line from the maximum time over ranks and the sum of grid points.
These tests run the helpers bench.py uses for that (process group set-up,
max and sum reductions, barrier) in two real gloo ranks, and the reference
arm under torchrun, where rank 0 alone works and prints and the other rank
exits 0 without work."""
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


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      MOLOCH_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    dist, r, ws = bench.dist_setup()
    res = {"rank": r, "ws": ws,
           "max": bench.reduce_max(dist, 10.0 * (r + 1)),
           "sum": bench.reduce_sum(dist, 1e9 * (r + 1))}
    bench.barrier(dist)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump(res, f)


def test_replica_reductions_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in (0, 1):
        with open(tmp_path / f"rank{r}.json") as f:
            res = json.load(f)
        assert res["rank"] == r and res["ws"] == 2
        assert res["max"] == 20.0  # slowest rank's time
        assert res["sum"] == 3e9   # all ranks' grid points


def test_reference_arm_under_torchrun(oracle_mod):
    """torchrun with two ranks: exactly one JSON line, from rank 0, with the
    job's rank count; both ranks exit 0."""
    port = _free_port()
    env = dict(os.environ, MOLOCH_BENCH_BACKEND="gloo", OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(ln) for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
