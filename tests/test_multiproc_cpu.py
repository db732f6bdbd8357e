"""The N > 1 launch path of bench.py on CPU (gloo, world size 2).

Multi-GPU runs are replicas (no data-path collective): every rank steps its
own copy and the job time is the maximum over ranks.  These tests run two
ranks as CPU processes with the gloo backend: the max-over-ranks timing and
barrier helpers, and the reference arm launched by torchrun, where rank 0
alone prints the JSON line and the other rank exits 0.
"""
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
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": "2", "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, ws = bench.dist_init()
    assert (r, ws) == (rank, 2)
    bench.barrier(dist)
    # each rank's "time"; the job reports the maximum
    t = bench.reduce_max(dist, 1.5 + rank)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(t))
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, start_method="spawn")
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(2)]
    assert vals == [2.5, 2.5]


@pytest.mark.slow
def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--small", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-3000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
