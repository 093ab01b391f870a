"""The learned endpoint proposal for BC1: training data, training loop and evaluation.

Training blocks come from the two synthetic generators of the library's workloads (ntg.synth):
opaque colour textures with box mips in linear space, and sRGB colour textures with an alpha
field, Kaiser mips and transparency weighting. Every block of every level is a sample; its
target is what the plain cluster fit (icbc Level8, the full ordering search) encodes for it:
the two endpoints and log(1 + SSE). The network (ntg.MLP, tensor-core kernels) is trained with
Adam on shuffled batches; the CUDA graph of one step is replayed.

At inference, ntg.Context.compress_chain_learned runs features -> network -> pruned search ->
full fit of the blocks the network's error estimate flags, all on the GPU.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import (ALPHA_NONE, ALPHA_TRANSPARENCY, FILTER_BOX, FILTER_KAISER, FORMAT_BC1, FORMAT_BC3, MLP, QUALITY_NORMAL,
               XFORM_NONE, XFORM_SRGB, ChainOptions, Context, chain_levels, nblocks)
from . import synth


def generator_options(kind: int) -> ChainOptions:
    """BC1 blocks: kind 0: linear, box mips, opaque; kind 1: sRGB, Kaiser mips, transparency weighting;
    kind 2: linear, Kaiser mips, opaque (the batched workloads' BC1 textures). BC3 blocks: kind 3:
    linear, Kaiser mips, alpha field with transparency weighting (the batched workloads' BC3
    textures); kind 4: sRGB, Kaiser mips, transparency (the 4096x4096 workload's texture style)."""
    if kind == 3:
        return ChainOptions.make(format=FORMAT_BC3, quality=QUALITY_NORMAL, filter=FILTER_KAISER,
                                 alpha_mode=ALPHA_TRANSPARENCY, in_xform=XFORM_NONE, out_xform=XFORM_NONE)
    if kind == 4:
        return ChainOptions.make(format=FORMAT_BC3, quality=QUALITY_NORMAL, filter=FILTER_KAISER,
                                 alpha_mode=ALPHA_TRANSPARENCY, in_xform=XFORM_SRGB, out_xform=XFORM_SRGB)
    if kind == 2:
        return ChainOptions.make(format=FORMAT_BC1, quality=QUALITY_NORMAL, filter=FILTER_KAISER, alpha_mode=ALPHA_NONE,
                                 in_xform=XFORM_NONE, out_xform=XFORM_NONE)
    if kind == 0:
        return ChainOptions.make(format=FORMAT_BC1, quality=QUALITY_NORMAL, filter=FILTER_BOX, alpha_mode=ALPHA_NONE,
                                 in_xform=XFORM_NONE, out_xform=XFORM_NONE)
    return ChainOptions.make(format=FORMAT_BC1, quality=QUALITY_NORMAL, filter=FILTER_KAISER,
                             alpha_mode=ALPHA_TRANSPARENCY, in_xform=XFORM_SRGB, out_xform=XFORM_SRGB)


def generator_texture(kind: int, size: int, seed: int) -> np.ndarray:
    if kind == 0:
        return synth.colour_texture(size, size, seed, scale=size / 512.0)
    if kind == 2:
        return synth.batch_texture(size, size, FORMAT_BC1, seed)
    if kind == 3:
        return synth.batch_texture(size, size, FORMAT_BC3, seed)
    scale = 8.0 * size / 4096.0
    return synth.colour_texture(size, size, seed, scale=scale, alpha=synth.alpha_field(size, size, seed, scale=scale))


def _texture_job(job):
    return generator_texture(*job)


def _generate(jobs):
    """generator_texture(kind, size, seed) for every job, on every core (spawned processes)."""
    import multiprocessing as mp
    import os
    workers = min(len(jobs), os.cpu_count() or 1)
    if workers <= 1:
        return [_texture_job(j) for j in jobs]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_texture_job, jobs, chunksize=1)


def training_set(ctx: Context, n_blocks: int, seed: int = 0x5EED, size: int = 2048, kinds=(0, 1)):
    """(x [n x 48], t [n x 8]) float32 CUDA tensors from whole chains of seeded textures, cycling
    through the generators `kinds` (all of one format), until n_blocks samples."""
    import torch
    per = sum(nblocks(lw, lh) for lw, lh in chain_levels(size, size))
    count = (n_blocks + per - 1) // per
    imgs = _generate([(kinds[i % len(kinds)], size, seed + 7919 * i) for i in range(count)])
    xs, ts, have, i = [], [], 0, 0
    while have < n_blocks:
        kind = kinds[i % len(kinds)]
        img = imgs[i]
        opt = generator_options(kind)
        d = torch.from_numpy(img).cuda()
        blocks = ctx.compress_chain(d, size, size, opt)
        xs.append(ctx.chain_features(d, size, size, opt))
        ts.append(ctx.chain_targets(d, size, size, opt, blocks))
        have += xs[-1].shape[0]
        i += 1
    x = torch.cat(xs)[:n_blocks].contiguous()
    t = torch.cat(ts)[:n_blocks].contiguous()
    return x, t


def train(net: MLP, x, t, steps: int, batch: int = 8192, lr: float = 1e-3, seed: int = 1, log_every: int = 0):
    """Adam on shuffled batches (a new permutation each epoch); returns the per-step losses."""
    import torch
    n = x.shape[0]
    g = torch.Generator(device=x.device).manual_seed(seed)
    perm = torch.randperm(n, generator=g, device=x.device)
    xb = torch.empty((batch, x.shape[1]), dtype=torch.float32, device=x.device)
    tb = torch.empty((batch, t.shape[1]), dtype=torch.float32, device=x.device)
    losses = torch.zeros(steps, dtype=torch.float32, device=x.device)
    pos = 0
    for s in range(steps):
        if pos + batch > n:
            perm = torch.randperm(n, generator=g, device=x.device)
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        torch.index_select(x, 0, idx, out=xb)
        torch.index_select(t, 0, idx, out=tb)
        net.train_step(xb, tb, lr=lr, loss_out=losses[s:s + 1])
        if log_every and (s + 1) % log_every == 0:
            print(f"step {s + 1}: loss {losses[s].item():.5f}", flush=True)
    net.status()
    return losses.cpu().numpy()


def chain_rmse(ctx: Context, bgra, w: int, h: int, opt: ChainOptions, blocks) -> float:
    """RMSE of a BC1 chain's decoded levels against the levels the encoder read (linear chains:
    the mip levels themselves), over all texels of all levels."""
    import torch
    levels = ctx.mip_chain(bgra, w, h, opt)
    sse, texels, loff, boff = 0.0, 0, 0, 0
    for lw, lh in chain_levels(w, h, opt.max_levels):
        n = lw * lh
        nb = nblocks(lw, lh)
        ref = levels[loff:loff + 4 * n]
        dec = ctx.decode(FORMAT_BC1, blocks[boff:boff + 8 * nb], lw, lh)
        sums = ctx.error_sums(ref, dec, lw, lh, opt.alpha_mode)
        torch.cuda.synchronize()
        sse += float(sums[0].item())
        texels += n
        loff += 4 * n
        boff += 8 * nb
    return math.sqrt(sse / texels)


def chain_sse(ctx: Context, bgra, w: int, h: int, opt: ChainOptions, blocks_list):
    """Per blocks tensor of `blocks_list` (encodings of the same chain): the colour squared-error sum
    of its decoded levels against the levels the encoder read (linear chains: the mip levels
    themselves), over all texels of all levels - nvtt::rmsError's sum (alpha-weighted under
    transparency), in double. One mip chain, then every level's decode and error sums with no host
    round trip. Returns (list of sums, texels)."""
    import torch
    fmt = opt.format
    bb = 8 if fmt in (1, 2, 6) else 16
    levels = ctx.mip_chain(bgra, w, h, opt)
    lv = chain_levels(w, h, opt.max_levels)
    sums = torch.zeros((len(blocks_list), len(lv), 2), dtype=torch.float64, device=levels.device)
    texels, loff, boff = 0, 0, 0
    for li, (lw, lh) in enumerate(lv):
        n = lw * lh
        nb = nblocks(lw, lh)
        ref = levels[loff:loff + 4 * n]
        for k, blocks in enumerate(blocks_list):
            dec = ctx.decode(fmt, blocks[boff:boff + bb * nb], lw, lh)
            ctx.error_sums(ref, dec, lw, lh, opt.alpha_mode, out=sums[k, li])
        texels += n
        loff += 4 * n
        boff += bb * nb
    return [float(v) for v in sums[:, :, 0].sum(dim=1).cpu()], texels


def uniform_proposals(n: int, device="cuda"):
    """A proposal without the network: the orderings that split the block's weight evenly
    (quarters for four clusters, thirds for three), and an infinite error estimate (never falls back)."""
    import torch
    y = torch.zeros((n, 16), dtype=torch.float32, device=device)
    y[:, 0:5] = torch.tensor([0.25, 0.5, 0.75, 1 / 3, 2 / 3], device=device)
    y[:, 5] = float("inf")
    return y


def timed(fn, reps: int = 5):
    """Best of `reps` runs of fn() in milliseconds, CUDA events on the current stream."""
    import torch
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def _main(argv=None):
    """python -m ntg.learned infer --rows N: the fused network inference on N random blocks (an
    untrained network), for profiling; train --blocks N --steps S: a short training run."""
    import argparse
    import torch
    ap = argparse.ArgumentParser(prog="python -m ntg.learned")
    ap.add_argument("mode", choices=["infer", "train"])
    ap.add_argument("--rows", type=int, default=1 << 20)
    ap.add_argument("--blocks", type=int, default=1 << 20)
    ap.add_argument("--steps", type=int, default=128)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    net = MLP(seed=1)
    if a.mode == "infer":
        g = torch.Generator(device="cuda").manual_seed(1)
        x = torch.rand((a.rows, 48), generator=g, device="cuda")
        y = net.infer(x)
        ms = timed(lambda: net.infer(x, out=y), reps=a.reps)
        flop = a.rows * 2 * (48 * 256 + 256 * 256 + 256 * 16)
        print(f"infer {a.rows} rows: {ms:.3f} ms, {flop / ms / 1e9:.1f} TFLOP/s")
    else:
        ctx = Context(0)
        x, t = training_set(ctx, a.blocks, size=1024)
        t0 = time.perf_counter()
        losses = train(net, x, t, steps=a.steps)
        print(f"train {a.steps} steps: {time.perf_counter() - t0:.2f} s, loss {losses[0]:.4f} -> {losses[-1]:.4f}")
        ctx.close()
    net.close()


if __name__ == "__main__":
    _main()
