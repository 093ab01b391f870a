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


# ---- textures of a batch across ranks (ntg.partition) ----

def test_partition_is_a_balanced_cover():
    sys.path.insert(0, os.path.join(ROOT, "nvidia-texture-tools_gb300"))
    from ntg import partition, synth
    specs = synth.batch_specs(1024, 0xC4, 7, 12)
    sizes = [(w, h) for (w, h, _f, _s) in specs]
    work = [partition.chain_texels(w, h) for (w, h) in sizes]
    for world in (1, 2, 3, 8):
        parts = partition.partition_textures(sizes, world)
        assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
        assert all(p == sorted(p) for p in parts)
        loads = [sum(work[i] for i in p) for p in parts]
        bound = max(max(work), sum(work) / world)   # no split can beat this
        assert max(loads) <= 4 / 3 * bound
    assert partition.partition([5, 1, 1, 1, 1, 1], 2) == [[0], [1, 2, 3, 4, 5]]
    with pytest.raises(ValueError):
        partition.partition([1], 0)


def _oracle_chain_bytes(oracle, w, h, fmt, seed):
    import numpy as np
    from ntg import synth
    img = synth.batch_texture(w, h, fmt, seed)
    _, enc = oracle.mip_chain(img, w, h, 1, 1.0, 0.0, 0.0, 2, 0, 0, 0, 2.2)
    return np.concatenate([oracle.bc1_image(l.reshape(-1), l.shape[2], l.shape[1], 0, 1) for l in enc])


def _partition_rank(rank, world, port, out_dir):
    import pickle
    import torch.distributed as dist
    sys.path[:0] = [ROOT, os.path.join(ROOT, "nvidia-texture-tools_gb300"), os.path.join(ROOT, "oracle")]
    import pyoracle
    from ntg import partition, synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        specs = synth.batch_specs(10, 0x5A, 3, 6)
        parts = partition.partition_textures([(w, h) for (w, h, _f, _s) in specs], world)
        oracle = pyoracle.Oracle()
        # this rank's textures, whole chains encoded by the CPU oracle (the test machine has no GPU)
        local = [_oracle_chain_bytes(oracle, *specs[i]) for i in parts[rank]]
        got = partition.gather(local, parts, rank, world)
        if rank == 0:
            with open(os.path.join(out_dir, "gathered.pkl"), "wb") as f:
                pickle.dump(got, f)
    finally:
        dist.destroy_process_group()


def test_partitioned_batch_gathers_to_the_one_rank_bytes(tmp_path, oracle):
    """Two gloo ranks each encode their part of a batch and gather on rank 0: the result is the
    one-rank batch's bytes, texture by texture, in the batch's order."""
    import pickle
    import numpy as np
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "nvidia-texture-tools_gb300"))
    from ntg import synth
    port = _free_port()
    mp.spawn(_partition_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    with open(tmp_path / "gathered.pkl", "rb") as f:
        got = pickle.load(f)
    specs = synth.batch_specs(10, 0x5A, 3, 6)
    assert len(got) == len(specs)
    for spec, g in zip(specs, got):
        assert np.array_equal(g, _oracle_chain_bytes(oracle, *spec))
