"""Multi-process paths of bench.py on the CPU (gloo, world size 2).

The render path does not shard (every GPU runs an independent replica of the
step), so what runs across processes is the benchmark's own scaffolding:
the rank set-up from the torchrun environment, the barrier, the maximum of
the per-rank times, and the reference arm, which only rank 0 runs.
"""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    r, w, _ = bench.dist_setup(world)
    assert (r, w) == (rank, world)
    bench.barrier(w)
    value = bench.max_over_ranks(10.0 * (rank + 1), w)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(value))
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    port = _free_port()
    mp.start_processes(_max_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    values = [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(2)]
    assert values == [20.0, 20.0]


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun():
    """Rank 0 prints the reference arm's one JSON line; rank 1 exits 0 without
    work (the small configuration keeps the host run short)."""
    port = _free_port()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps",
           "1", "--warmup", "1", "--config", "small"]
    proc = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-3000:]
    lines = [line for line in proc.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1, proc.stdout
    record = json.loads(lines[0])
    assert record["impl"] == "reference" and record["value"] > 0
    assert record["e2e"]["h2d_bytes_per_step"] == 0 and record["cpu_baseline"]["kind"] == "port"
