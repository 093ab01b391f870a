"""GPU parity at the workloads' own sizes, bit-exact against the oracle.

The small cases of test_gpu_parity.py leave some production code unexercised:
  * the BGRA8 level-1 kernel is persistent (one CTA per SM over 64 x 16 output tiles): only a level
    with more tiles than SMs makes a CTA walk several tiles and swap its double buffer (fetch tile
    i+1 while filtering tile i and running tile i-1's Y taps);
  * batches merge the same depth of many textures into one launch, so a batch of large textures has
    thousands of tiles per launch;
  * the 4096x4096 sRGB / Kaiser / BC3 chain runs every kernel variant of the chain at full size.
Each case runs the product through the C ABI and the oracle on the host cores, then compares every
FP32 level (bit patterns) and every block byte.
"""
import os

import numpy as np
import pytest

import ntg
import ntg.synth as synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

THREADS = os.cpu_count() or 4
TILE_W, TILE_H, SMS = 64, 16, 152   # the BGRA8 tile kernel's output tile and the GB300's SM count


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def oracle_blocks(oracle, enc_levels, fmt, quality, am):
    out = []
    for lv in enc_levels:
        lw, lh = lv.shape[2], lv.shape[1]
        flat = lv.reshape(-1)
        if fmt == ntg.FORMAT_BC1:
            out.append(oracle.bc1_image(flat, lw, lh, am, quality, threads=THREADS))
        elif fmt == ntg.FORMAT_BC3:
            out.append(oracle.bc3_image(flat, lw, lh, am, quality, threads=THREADS))
        else:
            out.append(oracle.bc5_image(flat, lw, lh, quality, threads=THREADS))
    return np.concatenate(out)


def oracle_chain(oracle, bgra, w, h, opt, max_levels=64):
    width = {0: 0.5, 1: 1.0, 2: 3.0}[opt.filter]
    lin, enc = oracle.mip_chain(bgra, w, h, opt.filter, width, 4.0, 1.0, opt.wrap, opt.alpha_mode, opt.in_xform,
                                opt.out_xform, 2.2, max_levels)
    return np.concatenate([l.reshape(-1) for l in lin]), oracle_blocks(oracle, enc, opt.format, opt.quality,
                                                                        opt.alpha_mode)


def level1_tiles(w, h):
    return ((w // 2 + TILE_W - 1) // TILE_W) * ((h // 2 + TILE_H - 1) // TILE_H)


def test_c1_full_chain_matches_oracle(ctx, oracle):
    """The 4096x4096 sRGB texture with its alpha field, Kaiser (3, 4, 1) mips with sRGB in and out,
    transparency, BC3 Normal, all 13 levels: every FP32 level and all 1,398,103 blocks."""
    w = h = 4096
    bgra = synth.texture_c1()
    opt = ntg.ChainOptions.make(format=ntg.FORMAT_BC3, quality=ntg.QUALITY_NORMAL, filter=ntg.FILTER_KAISER,
                                wrap=ntg.WRAP_MIRROR, alpha_mode=ntg.ALPHA_TRANSPARENCY, in_xform=ntg.XFORM_SRGB,
                                out_xform=ntg.XFORM_SRGB)
    d = dev(bgra)
    levels = host(ctx.mip_chain(d, w, h, opt))
    blocks = host(ctx.compress_chain(d, w, h, opt))
    ref_levels, ref_blocks = oracle_chain(oracle, bgra, w, h, opt)
    assert blocks.size == 1398103 * 16
    assert np.array_equal(levels.view(np.uint32), ref_levels.view(np.uint32))
    assert np.array_equal(blocks, ref_blocks)


# (w, h, format, filter, alpha_mode, in_xform, out_xform): level 1 filtered from the BGRA8 input.
# 2048x2048 gives 1,024 tiles (6.7 per CTA), 4096x1024 gives 1,024 in a wide shape, 1024x4096 in a
# tall one; BC3/BC5 also write the quantised BGRA8 copy of the level the encoders read.
LEVEL1 = [
    (2048, 2048, ntg.FORMAT_BC3, ntg.FILTER_KAISER, 1, ntg.XFORM_SRGB, ntg.XFORM_SRGB),
    (2048, 2048, ntg.FORMAT_BC1, ntg.FILTER_TRIANGLE, 0, ntg.XFORM_NONE, ntg.XFORM_NONE),
    (4096, 1024, ntg.FORMAT_BC3, ntg.FILTER_TRIANGLE, 1, ntg.XFORM_GAMMA, ntg.XFORM_GAMMA),
    (1024, 4096, ntg.FORMAT_BC1, ntg.FILTER_KAISER, 0, ntg.XFORM_NONE, ntg.XFORM_NONE),
]


@pytest.mark.parametrize("wrap", [ntg.WRAP_CLAMP, ntg.WRAP_REPEAT, ntg.WRAP_MIRROR])
@pytest.mark.parametrize("case", LEVEL1)
def test_level1_tile_loop_matches_oracle(ctx, oracle, case, wrap):
    """One buildNextMipmap step from the BGRA8 input at sizes where every CTA of the persistent tile
    kernel walks several tiles, under each wrap mode: level 1 bit-exact, and both levels' blocks."""
    w, h, fmt, filt, am, ix, ox = case
    assert level1_tiles(w, h) >= 3 * SMS
    bgra = synth.colour_texture(w, h, 0x11 + w + 3 * h + wrap, scale=4.0,
                                alpha=synth.alpha_field(w, h, 7 + wrap, scale=4.0) if am else None)
    opt = ntg.ChainOptions.make(format=fmt, quality=ntg.QUALITY_NORMAL, filter=filt, wrap=wrap, alpha_mode=am,
                                in_xform=ix, out_xform=ox, gamma=2.2, max_levels=2)
    d = dev(bgra)
    levels = host(ctx.mip_chain(d, w, h, opt))
    blocks = host(ctx.compress_chain(d, w, h, opt))
    ref_levels, ref_blocks = oracle_chain(oracle, bgra, w, h, opt, max_levels=2)
    assert np.array_equal(levels.view(np.uint32), ref_levels.view(np.uint32))
    assert np.array_equal(blocks, ref_blocks)


def _batch_sample(specs, filt, seed):
    """The batched workloads' textures (linear colour, BC3 with transparency, fBm normal maps for
    BC5, Normal quality, mirror wrap), one image per texture."""
    out = []
    for i, (w, h, fmt, s) in enumerate(specs):
        img = synth.batch_texture(w, h, fmt, seed ^ (w * 131 + h * 7 + fmt) ^ i)
        opt = ntg.ChainOptions.make(format=fmt, quality=ntg.QUALITY_NORMAL, filter=filt, wrap=ntg.WRAP_MIRROR,
                                    alpha_mode=ntg.ALPHA_TRANSPARENCY if fmt == ntg.FORMAT_BC3 else ntg.ALPHA_NONE)
        out.append((w, h, opt, img))
    return out


def _pick(specs, n_per_format, largest):
    """The `largest` biggest textures of the spec list plus the first `n_per_format` of each format."""
    by_size = sorted(range(len(specs)), key=lambda i: -specs[i][0] * specs[i][1])
    chosen = list(by_size[:largest])
    for fmt in (ntg.FORMAT_BC1, ntg.FORMAT_BC3, ntg.FORMAT_BC5):
        chosen += [i for i, s in enumerate(specs) if s[2] == fmt and i not in chosen][:n_per_format]
    return [specs[i] for i in sorted(set(chosen))]


def _check_batch(ctx, oracle, sample, tmp_path, monkeypatch):
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    textures = []
    for (w, h, opt, img) in sample:
        out = dev(np.zeros(ntg.chain_bytes(w, h, opt), np.uint8))
        textures.append((dev(img.reshape(-1).view(np.uint32)), w, h, opt, out))
    b = ntg.Batch(ctx, textures)
    try:
        for t in textures:
            t[4].zero_()
        b.launch()
        for (w, h, opt, img), t in zip(sample, textures):
            _, ref = oracle_chain(oracle, img, w, h, opt)
            assert np.array_equal(host(t[4]), ref), (w, h, opt.format)
    finally:
        b.close()


def test_batch_c2_sample_matches_oracle(ctx, oracle, tmp_path, monkeypatch):
    """A sample of the 256-texture batch (sizes 64..2048, 50/30/20 BC1/BC3/BC5, Triangle mips): its
    largest textures and some of each format, as one batch. The merged level-1 launch has well over
    one tile per SM, so the persistent tile loop runs across textures."""
    specs = synth.batch_specs(256, 0xC2, 6, 11)
    sample = _batch_sample(_pick(specs, 4, 6), ntg.FILTER_TRIANGLE, 0xC2)
    assert len(sample) >= 12
    assert {s[2].format for s in sample} == {1, 4, 7}
    assert sum(level1_tiles(w, h) for (w, h, _, _) in sample) >= 3 * SMS
    _check_batch(ctx, oracle, sample, tmp_path, monkeypatch)


def test_batch_c4_sample_matches_oracle(ctx, oracle, tmp_path, monkeypatch):
    """A sample of the 1024-texture batch (sizes 128..4096, Kaiser mips): its largest textures (4096
    px) and some of each format, as one batch."""
    specs = synth.batch_specs(1024, 0xC4, 7, 12)
    sample = _batch_sample(_pick(specs, 3, 3), ntg.FILTER_KAISER, 0xC4)
    assert max(w * h for (w, h, _, _) in sample) == 4096 * 4096
    assert {s[2].format for s in sample} == {1, 4, 7}
    _check_batch(ctx, oracle, sample, tmp_path, monkeypatch)
