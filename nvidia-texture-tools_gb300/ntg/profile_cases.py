"""Runs every kernel of libntg.so on a small case, for a profiler's launch list and captures.

    cd nvidia-texture-tools_gb300 && python -m ntg.profile_cases [--case NAME ...] [--size N] [--once]

Each case makes its inputs, runs one warm-up call, then the call itself (--once: the call alone, for
a profiler that captures every launch and flushes the caches between its passes anyway). Inputs are
sized above the 129 MB L2 where the kernel reads DRAM in production (images of 2048 x 2048 texels by
default) and hold a few GB of device memory at most. The learned cases use an untrained network and
no fallback (the pruned search's cost does not depend on the proposal's quality). Kernels per case:

  mips_kaiser_srgb   k_tile2x_u8, k_tile2x, k_mip_tail           (Kaiser, sRGB in and out, BC3 levels)
  mips_tma           k_tile2x_f32                                (one Kaiser 2:1 step from a 2N x N FP32 level)
  mips_odd           k_poly, k_mip_tail                          (odd sizes: the general scale kernel)
  mips_box           k_set_image, k_fast_down                    (box filter)
  bc1                k_bc1<7> (Normal)     bc1_fastest  k_bc1<0>     bc1_production  k_bc1<8>
  bc3                k_bc3<1>              bc1a         k_bc1a       bc4  k_bc4<1>    bc5  k_bc5<1>
  decode_rms         k_decode, k_error_sums
  learned_bc1        chain mips, k_bc1_features, k_mlp_infer, k_bc1_learned, k_bc1<7> over the list
  learned_bc3        chain mips, k_bc3_features, k_mlp_infer, k_bc3_learned, k_bc3<1> over the list
  train              k_to_bf16, k_gemm (forward, backward, split-K), k_loss, k_colsum, k_adam, k_refresh
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from . import (ALPHA_NONE, ALPHA_TRANSPARENCY, BLOCK_BYTES, FILTER_BOX, FILTER_KAISER, FORMAT_BC1, FORMAT_BC1A,
               FORMAT_BC3, FORMAT_BC4, FORMAT_BC5, MLP, NTG_PROPOSAL_DESCENT, QUALITY_FASTEST, QUALITY_NORMAL,
               QUALITY_PRODUCTION, XFORM_SRGB, ChainOptions, Context, chain_bytes, chain_levels, nblocks)
from . import learned, synth

CASES = ["mips_kaiser_srgb", "mips_tma", "mips_odd", "mips_box", "bc1", "bc1_fastest", "bc1_production", "bc3", "bc1a", "bc4", "bc5",
         "decode_rms", "learned_bc1", "learned_bc3", "train"]
ONCE = False


def _calls(fn):
    import torch
    if not ONCE:
        fn()
        torch.cuda.synchronize()
    fn()
    torch.cuda.synchronize()


def run(case: str, size: int, ctx: Context):
    import torch
    dev = "cuda"
    if case == "mips_tma":
        # a source of 2N x N FP32 texels: large enough for the TMA-staged tile kernel
        w, h = 2 * size, size
        img = torch.from_numpy(synth.colour_texture(w, h, 9, scale=4.0)).to(dev)
        src = torch.empty(4 * w * h, dtype=torch.float32, device=dev)
        ctx.set_image(img, w, h, out=src)
        out = torch.empty(4 * (w // 2) * (h // 2), dtype=torch.float32, device=dev)
        _calls(lambda: ctx.mip_level(src, w, h, filter=FILTER_KAISER, params=(4.0, 1.0), out=out))
        return
    if case.startswith("mips"):
        w, h = (size - 3, size - 5) if case == "mips_odd" else (size, size)
        img = synth.colour_texture(w, h, 7, scale=4.0, alpha=synth.alpha_field(w, h, 7, scale=4.0))
        d = torch.from_numpy(img).to(dev)
        if case == "mips_box":
            opt = ChainOptions.make(format=FORMAT_BC1, filter=FILTER_BOX)
        else:
            opt = ChainOptions.make(format=FORMAT_BC3, filter=FILTER_KAISER, alpha_mode=ALPHA_TRANSPARENCY,
                                    in_xform=XFORM_SRGB, out_xform=XFORM_SRGB)
        out = torch.empty(sum(4 * lw * lh for lw, lh in chain_levels(w, h)), dtype=torch.float32, device=dev)
        _calls(lambda: ctx.mip_chain(d, w, h, opt, out=out))
        return
    if case in ("bc1", "bc1_fastest", "bc1_production", "bc3", "bc1a", "bc4", "bc5", "decode_rms"):
        w = h = size
        fmt, q = {"bc1": (FORMAT_BC1, QUALITY_NORMAL), "bc1_fastest": (FORMAT_BC1, QUALITY_FASTEST),
                  "bc1_production": (FORMAT_BC1, QUALITY_PRODUCTION), "bc3": (FORMAT_BC3, QUALITY_NORMAL),
                  "bc1a": (FORMAT_BC1A, QUALITY_NORMAL), "bc4": (FORMAT_BC4, QUALITY_NORMAL),
                  "bc5": (FORMAT_BC5, QUALITY_NORMAL), "decode_rms": (FORMAT_BC3, QUALITY_NORMAL)}[case]
        if case == "bc1_production":  # Level9 is slow: a quarter of the blocks
            h = size // 4
        levels = torch.from_numpy(np.random.default_rng(3).random(4 * w * h, dtype=np.float32)).to(dev)
        am = ALPHA_TRANSPARENCY if fmt == FORMAT_BC3 else ALPHA_NONE
        out = torch.empty(BLOCK_BYTES[fmt] * nblocks(w, h), dtype=torch.uint8, device=dev)
        if case == "decode_rms":
            ctx.encode(fmt, levels, w, h, quality=q, alpha_mode=am, out=out)
            dec = torch.empty(4 * w * h, dtype=torch.float32, device=dev)
            sums = torch.empty(2, dtype=torch.float64, device=dev)
            _calls(lambda: (ctx.decode(fmt, out, w, h, out=dec), ctx.error_sums(levels, dec, w, h, am, out=sums)))
            return
        _calls(lambda: ctx.encode(fmt, levels, w, h, quality=q, alpha_mode=am, out=out))
        return
    if case in ("learned_bc1", "learned_bc3"):
        kind = 2 if case == "learned_bc1" else 3
        img = learned.generator_texture(kind, size, 11)
        opt = learned.generator_options(kind)
        d = torch.from_numpy(img).to(dev)
        net = MLP(seed=5)
        out = torch.empty(chain_bytes(size, size, opt), dtype=torch.uint8, device=dev)
        search = NTG_PROPOSAL_DESCENT | 4 if kind == 2 else 2
        _calls(lambda: ctx.compress_chain_learned(net, d, size, size, opt, radius=search, margin=float("inf"), out=out,
                                                  stats=False))
        net.close()
        return
    if case == "train":
        net = MLP(seed=5)
        rng = np.random.default_rng(1)
        x = torch.from_numpy(rng.random((8192, 48), dtype=np.float32)).to(dev)
        t = torch.from_numpy(rng.random((8192, 8), dtype=np.float32)).to(dev)
        _calls(lambda: net.train_step(x, t))
        net.close()
        return
    raise ValueError(case)


def main(argv=None):
    global ONCE
    ap = argparse.ArgumentParser(prog="python -m ntg.profile_cases")
    ap.add_argument("--case", action="append", choices=CASES)
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--once", action="store_true", help="one call per case, no warm-up")
    a = ap.parse_args(argv)
    ONCE = a.once
    ctx = Context(0)
    for c in a.case or CASES:
        run(c, a.size, ctx)
        print(f"case {c} done", file=sys.stderr, flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
