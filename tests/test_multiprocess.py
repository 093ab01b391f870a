"""The multi-process path on the CPU (gloo, world size 2): bench.py's max-over-ranks timing reduction,
and the reference arm launched the way multi-GPU runs are (torchrun, one process per rank): rank 0
prints the single JSON line, the other ranks exit 0 without work. GPU runs use the same code with
NCCL; textures are independent, so ranks are replicas and exchange nothing but the timing maximum."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(world, float(10 * rank + 3))
        bench.barrier(world)
        with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
            f.write(repr(got))
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    vals = [float(open(tmp_path / f"r{r}.txt").read()) for r in range(2)]
    assert vals == [13.0, 13.0]


def test_reference_arm_under_torchrun_two_ranks(oracle):
    """torchrun --nproc-per-node 2 bench.py --impl reference: one JSON line from rank 0, exit 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--workload", "c2_small", "--steps", "1", "--warmup", "3", "--cpu-seconds", "0.2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
