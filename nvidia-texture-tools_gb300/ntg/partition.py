"""Textures of a batch across GPUs: one process per GPU, a static partition, a host gather.

Textures are independent (the reference compresses one image per Compressor::process call,
src/nvtt/Context.cpp:217-346), so a batch splits across ranks with no exchange while it runs: each
rank builds the batch of its own textures on its own GPU, and the encoded bytes come back to one
rank on the host at the end. The split is the longest-processing-time rule over each texture's
work, the texels of its whole chain: textures in decreasing order of work, each to the rank with
the least work so far (ties to the lowest rank), which keeps every rank within 4/3 of the best
possible maximum.
"""
from __future__ import annotations


def chain_texels(w: int, h: int) -> int:
    """Texels of all levels of a full chain (nvtt::countMipmaps levels)."""
    n = 0
    while True:
        n += w * h
        if w == 1 and h == 1:
            return n
        w, h = max(1, w // 2), max(1, h // 2)


def partition(work, world: int):
    """Indices of the items per rank: largest first, each to the least-loaded rank; every rank's
    list is in increasing index order (the batch's own order)."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += work[i]
    return [sorted(p) for p in parts]


def partition_textures(sizes, world: int):
    """partition() over (w, h) texture sizes, by the texels of each texture's chain."""
    return partition([chain_texels(w, h) for (w, h) in sizes], world)


def gather(local, parts, rank: int, world: int, dst: int = 0):
    """Gathers each rank's outputs (`local`: this rank's outputs in its part's order, host arrays)
    into the batch's order on rank `dst` (a torch.distributed object gather; returns None on the
    other ranks). world 1 returns `local` unchanged."""
    if world == 1:
        return list(local)
    import torch.distributed as dist
    got = [None] * world if rank == dst else None
    dist.gather_object(list(local), got, dst=dst)
    if rank != dst:
        return None
    out = [None] * sum(len(p) for p in parts)
    for r, p in enumerate(parts):
        if len(got[r]) != len(p):
            raise RuntimeError(f"rank {r} returned {len(got[r])} outputs for {len(p)} textures")
        for i, v in zip(p, got[r]):
            out[i] = v
    return out
