"""The benchmark's multi-process path on CPU (gloo, world size 2).

bench.py runs one replica per rank: a barrier and max-over-ranks timing
around the timed region, and the whole-job value summed over ranks; the
reference arm runs on rank 0 alone.  Both are checked here with real
processes and the gloo backend, rendezvous on 127.0.0.1.
"""
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


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    mx = d.max(10.0 + rank)           # the slowest rank's time
    sm = d.sum(100 * (rank + 1))      # the whole job's units
    d.barrier()
    d.close()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as fh:
        json.dump({"max": mx, "sum": sm, "rank": d.rank, "world": d.world}, fh)


def test_dist_max_and_sum_over_two_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    for r in range(2):
        with open(tmp_path / ("rank%d.json" % r)) as fh:
            got = json.load(fh)
        assert got == {"max": 11.0, "sum": 300.0, "rank": r, "world": 2}


def test_reference_arm_prints_one_line_from_rank0():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--edge", "6", "--steps", "1",
           "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["cores"] >= 1
