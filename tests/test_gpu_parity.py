"""GPU parity: every kernel of libntg.so, called through its C ABI, against the oracle (the C
restatement pinned to the reference) on the same seeded inputs, bit-exact (the sRGB curves on
float levels included: the device corrects its powf to the host libm's results)."""
import ctypes

import numpy as np
import pytest

import ntg
import ntg.synth as synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def float_image(w, h, seed, lo=0.0, hi=1.0, alpha_zero_frac=0.0):
    rng = np.random.default_rng(seed)
    img = (rng.random(4 * w * h) * (hi - lo) + lo).astype(np.float32)
    if alpha_zero_frac:
        a = img[3 * w * h:]
        a[rng.random(w * h) < alpha_zero_frac] = 0.0
    return img


def blocky_image(w, h, seed):
    """A float image tiled from the synthetic 4x4 block kinds (flat, few-colour, gradients, noise)."""
    bw, bh = (w + 3) // 4, (h + 3) // 4
    blocks = synth.random_blocks(bw * bh, seed).reshape(bh, bw, 4, 4, 4).astype(np.float32) / 255.0
    img = blocks.transpose(0, 2, 1, 3, 4).reshape(bh * 4, bw * 4, 4)[:h, :w]
    bgra_planar = img.transpose(2, 0, 1)  # b, g, r, a planes
    return np.concatenate([bgra_planar[2].ravel(), bgra_planar[1].ravel(), bgra_planar[0].ravel(),
                           bgra_planar[3].ravel()]).astype(np.float32)


# ---------------------------------------------------------------------------------------------
# block encoders

@pytest.mark.parametrize("quality", [0, 1, 2])
@pytest.mark.parametrize("alpha_mode", [0, 1])
def test_bc1_encode_matches_oracle(ctx, oracle, quality, alpha_mode):
    for (w, h, seed) in [(64, 64, 1), (37, 23, 2), (4, 4, 3), (1, 1, 4), (2, 7, 5)]:
        for img in (float_image(w, h, seed, alpha_zero_frac=0.2), blocky_image(w, h, seed + 50),
                    float_image(w, h, seed + 9, lo=-0.2, hi=1.3)):
            ours = host(ctx.encode(ntg.FORMAT_BC1, dev(img), w, h, quality=quality, alpha_mode=alpha_mode))
            ref = oracle.bc1_image(img, w, h, alpha_mode, quality, threads=4)
            assert np.array_equal(ours, ref), (w, h, seed)


def test_bc1_colour_weights_and_nan(ctx, oracle):
    w, h = 32, 16
    img = float_image(w, h, 77)
    img[5] = np.nan
    img[w * h + 40] = np.inf
    for cw in [(1.0, 1.0, 1.0), (0.3, 0.59, 0.11), (2.0, 0.5, 1.0)]:
        ours = host(ctx.encode(ntg.FORMAT_BC1, dev(img), w, h, quality=1, cw=cw))
        assert np.array_equal(ours, oracle.bc1_image(img, w, h, 0, 1, cw=cw, threads=4))


@pytest.mark.parametrize("quality", [0, 1, 2, 3])
@pytest.mark.parametrize("alpha_mode", [0, 1])
def test_bc3_encode_matches_oracle(ctx, oracle, quality, alpha_mode):
    for (w, h, seed) in [(64, 32, 1), (13, 7, 2), (3, 5, 3), (1, 1, 4)]:
        for img in (float_image(w, h, seed, alpha_zero_frac=0.3), blocky_image(w, h, seed + 20),
                    float_image(w, h, seed + 5, lo=-0.3, hi=1.4)):
            ours = host(ctx.encode(ntg.FORMAT_BC3, dev(img), w, h, quality=quality, alpha_mode=alpha_mode))
            ref = oracle.bc3_image(img, w, h, alpha_mode, quality, threads=4)
            assert np.array_equal(ours, ref), (w, h, seed)


@pytest.mark.parametrize("quality", [1, 2])
def test_bc5_encode_matches_oracle(ctx, oracle, quality):
    for (w, h, seed) in [(64, 32, 1), (13, 7, 2), (1, 3, 3)]:
        for img in (float_image(w, h, seed), blocky_image(w, h, seed + 7)):
            ours = host(ctx.encode(ntg.FORMAT_BC5, dev(img), w, h, quality=quality))
            assert np.array_equal(ours, oracle.bc5_image(img, w, h, quality, threads=4))


@pytest.mark.parametrize("quality", [1, 2, 3])
@pytest.mark.parametrize("alpha_mode", [0, 1])
def test_bc1a_encode_matches_oracle(ctx, oracle, quality, alpha_mode):
    """CompressorDXT1a: three-colour fit with transparent texels (alpha 0 after ColorBlock's
    truncation), four-colour fit as well where there are none."""
    for (w, h, seed) in [(64, 32, 1), (13, 7, 2), (3, 5, 3), (1, 1, 4)]:
        for img in (float_image(w, h, seed, alpha_zero_frac=0.3), blocky_image(w, h, seed + 20),
                    float_image(w, h, seed + 5, lo=-0.3, hi=1.4), float_image(w, h, seed + 8, alpha_zero_frac=1.0)):
            ours = host(ctx.encode(ntg.FORMAT_BC1A, dev(img), w, h, quality=quality, alpha_mode=alpha_mode))
            ref = oracle.bc1a_image(img, w, h, alpha_mode, threads=4)
            assert np.array_equal(ours, ref), (w, h, seed)


def test_bc1a_colour_weights(ctx, oracle):
    w, h = 32, 16
    img = float_image(w, h, 78, alpha_zero_frac=0.25)
    for cw in [(0.3, 0.59, 0.11), (2.0, 0.5, 1.0)]:
        ours = host(ctx.encode(ntg.FORMAT_BC1A, dev(img), w, h, quality=1, cw=cw))
        assert np.array_equal(ours, oracle.bc1a_image(img, w, h, 0, cw=cw, threads=4))


def test_bc1a_fastest_is_refused(ctx):
    with pytest.raises(ntg.NtgError) as e:
        ctx.encode(ntg.FORMAT_BC1A, dev(np.zeros(64, np.float32)), 4, 4, quality=0)
    assert e.value.code == 2


@pytest.mark.parametrize("quality", [0, 1, 2, 3])
def test_bc4_encode_matches_oracle(ctx, oracle, quality):
    for (w, h, seed) in [(64, 32, 1), (13, 7, 2), (1, 3, 3)]:
        for img in (float_image(w, h, seed), blocky_image(w, h, seed + 7)):
            ours = host(ctx.encode(ntg.FORMAT_BC4, dev(img), w, h, quality=quality))
            assert np.array_equal(ours, oracle.bc4_image(img, w, h, quality, threads=4))


def _tiled(blocks64):
    """BGRA8 image whose 4x4 blocks, in raster order, are the given 64-byte blocks (one row of blocks)."""
    n = len(blocks64)
    b = np.asarray(blocks64, np.uint8).reshape(n, 4, 4, 4)
    return np.ascontiguousarray(b.transpose(1, 0, 2, 3).reshape(4, 4 * n, 4))


def test_bc1a_bc4_golden_blocks(ctx):
    """The reference's own BC1a and BC4 blocks (tests/golden/bc1a_bc4_blocks.npz), encoded here from
    the same bytes through the 8-bit path of a one-level chain."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "bc1a_bc4_blocks.npz"))
    inputs = g["inputs"]
    img = _tiled(inputs)
    w, h = 4 * len(inputs), 4
    for key in g.files:
        if key == "inputs":
            continue
        kind, param = key.split("_")
        if kind == "bc1a":
            opt = ntg.ChainOptions.make(format=ntg.FORMAT_BC1A, quality=1, alpha_mode=int(param), max_levels=1)
        else:
            opt = ntg.ChainOptions.make(format=ntg.FORMAT_BC4, quality=int(param), max_levels=1)
        out = host(ctx.compress_chain(dev(img), w, h, opt)).reshape(-1, 8)
        assert np.array_equal(out, g[key]), key


@pytest.mark.parametrize("fmt", [ntg.FORMAT_BC1, ntg.FORMAT_BC3])
@pytest.mark.parametrize("out_xform", [ntg.XFORM_GAMMA, ntg.XFORM_SRGB])
def test_encode_with_output_transform(ctx, oracle, fmt, out_xform):
    """Compressor::compress after toGamma(2.2) / toSrgb of the level: BC3 through the quantiser
    tables, BC1 on the float level through the device's corrected sRGB curve; every block exact."""
    w, h = 96, 64
    img = float_image(w, h, 31)
    enc = img.copy()
    n = w * h
    enc[:3 * n] = oracle.powf_5_11(img[:3 * n]) if out_xform == ntg.XFORM_GAMMA else oracle.to_srgb(img[:3 * n])
    for q in (0, 1, 2):
        ours = host(ctx.encode(fmt, dev(img), w, h, quality=q, out_xform=out_xform, gamma=2.2))
        ref = oracle.bc1_image(enc, w, h, 0, q, threads=4) if fmt == 1 else oracle.bc3_image(enc, w, h, 0, q, threads=4)
        assert np.array_equal(ours, ref), q


def _domain(lo_bits, hi_bits, margin):
    """Every float from lo_bits - margin to hi_bits + margin, plus zeros, negatives, 2 and NaN."""
    u = np.arange(lo_bits - margin, hi_bits + margin + 1, dtype=np.uint64).astype(np.uint32)
    extra = np.array([0.0, -0.0, -1e-8, -0.5, 2.0, np.inf, np.nan, 1.0000001], np.float32).view(np.uint32)
    return np.concatenate([u, extra]).view(np.float32)


@pytest.mark.parametrize("kind", [ntg.TRANSFORM_TO_SRGB, ntg.TRANSFORM_FROM_SRGB])
def test_srgb_curves_exact_over_their_domains(ctx, oracle, kind):
    """toSrgb over every float of its power segment (0.0031308, 1] and toLinearFromSrgb over every float
    of [0.04045, 1] (70.4 M and 39.5 M values, with a margin either side and special values): the
    device's corrected curves equal the host libm's, bit for bit."""
    lo = 0x3B4D2E1C if kind == ntg.TRANSFORM_TO_SRGB else 0x3D25AEE6
    vals = _domain(lo, 0x3F800000, 4096)
    n = -(-vals.size // 3)
    planes = np.zeros(4 * n, np.float32)
    planes[:vals.size] = vals                      # R, G, B planes hold the domain in order
    d = dev(planes)
    ntg._check(ntg.lib().ntg_transform(ctx.h, d.data_ptr(), n, 1, kind, ctypes.c_float(2.2), None))
    ours = host(d)[:vals.size]
    ref = oracle.to_srgb(vals) if kind == ntg.TRANSFORM_TO_SRGB else oracle.from_srgb(vals)
    bad = np.flatnonzero(ours.view(np.uint32) != ref.view(np.uint32))
    assert bad.size == 0, (bad.size, vals[bad[:5]], ours[bad[:5]], ref[bad[:5]])


# ---------------------------------------------------------------------------------------------
# mip filtering

@pytest.mark.parametrize("size", [(64, 64), (33, 17), (1, 9), (9, 1), (2, 2), (5, 7), (128, 32)])
@pytest.mark.parametrize("filt", [ntg.FILTER_BOX, ntg.FILTER_TRIANGLE, ntg.FILTER_KAISER])
def test_mip_level_matches_oracle(ctx, oracle, size, filt):
    w, h = size
    params = (4.0, 1.0)
    for wrap in (0, 1, 2):
        for am in (0, 1):
            img = float_image(w, h, w * 7 + h + wrap, lo=-0.1, hi=1.1)
            ours = host(ctx.mip_level(dev(img), w, h, filter=filt, params=params, wrap=wrap, alpha_mode=am))
            dw, dh = max(1, w // 2), max(1, h // 2)
            width = {0: 0.5, 1: 1.0, 2: 3.0}[filt]
            if filt == 0 and am == 0:
                ref = oracle.fast_downsample(img, w, h)
            else:
                ref = oracle.resize(img, w, h, dw, dh, filt, width, 4.0, 1.0, wrap)
            assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), (size, filt, wrap, am)


@pytest.mark.parametrize("filt", [ntg.FILTER_TRIANGLE, ntg.FILTER_KAISER])
def test_weighted_mip_level_matches_oracle(ctx, oracle, filt):
    for (w, h) in [(32, 32), (17, 9), (64, 16)]:
        img = float_image(w, h, 3 + w, alpha_zero_frac=0.3)
        width = 1.0 if filt == 1 else 3.0
        ours = host(ctx.mip_level(dev(img), w, h, filter=filt, params=(4.0, 1.0), wrap=2, weighted=1))
        ref = oracle.resize_weighted(img, w, h, max(1, w // 2), max(1, h // 2), filt, width, 4.0, 1.0, 2)
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


# 2:1 steps between FP32 levels: sources of at least 2048 x 2048 with enough tiles run on the
# persistent TMA-staged tile kernel (one TMA box per window; boxes at the level's edges read through
# remapped indices with the clamp and mirror wraps, and are copied by the threads with the repeat
# wrap); the others on the one-tile-per-CTA kernel. Sizes give both kernels, partial tiles on the
# right and bottom (4100 x 2050, 1000 x 600) and each tile height the planner picks (16, 8, 4 rows).
@pytest.mark.parametrize("size", [(4096, 2048), (2048, 4096), (4100, 2050), (1024, 1024), (1000, 600), (192, 96)])
@pytest.mark.parametrize("filt", [ntg.FILTER_TRIANGLE, ntg.FILTER_KAISER])
def test_fp32_tile_mip_level_matches_oracle(ctx, oracle, size, filt):
    w, h = size
    width = 1.0 if filt == ntg.FILTER_TRIANGLE else 3.0
    for wrap in (0, 1, 2):
        img = float_image(w, h, w + 3 * h + wrap, lo=-0.1, hi=1.1)
        ours = host(ctx.mip_level(dev(img), w, h, filter=filt, params=(4.0, 1.0), wrap=wrap))
        ref = oracle.resize(img, w, h, w // 2, h // 2, filt, width, 4.0, 1.0, wrap)
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), (size, filt, wrap)


def test_mip_level_unaligned_source_matches_oracle(ctx, oracle):
    """A source level 4 bytes past a 16-byte boundary gets no tensor map: the TMA tile kernel's
    windows are all copied by the threads."""
    w, h = 4096, 2048
    img = float_image(w, h, 31)
    buf = dev(np.concatenate([np.zeros(1, np.float32), img]))
    ours = host(ctx.mip_level(buf[1:], w, h, filter=ntg.FILTER_KAISER, params=(4.0, 1.0), wrap=ntg.WRAP_MIRROR))
    ref = oracle.resize(img, w, h, w // 2, h // 2, ntg.FILTER_KAISER, 3.0, 4.0, 1.0, ntg.WRAP_MIRROR)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_mip_waits_run_out_without_a_fault(ctx):
    """The TMA-staged FP32 tile kernel's mbarrier waits are bounded: with a limit of zero polls every
    wait for a TMA box gives up at once, with nothing faulting; the kernel records it, lets the box land
    and returns. With the default limit back, the same calls give the same levels and blocks as before
    (the 4096 x 2048 FP32 step takes TMA boxes; the chain's steps run beside it, unaffected)."""
    w = h = 1024
    bgra = synth.colour_texture(w, h, 5, alpha=synth.alpha_field(w, h, 5))
    fw, fh = 4096, 2048
    img = float_image(fw, fh, 9)
    opt = ntg.ChainOptions.make(format=ntg.FORMAT_BC3, quality=ntg.QUALITY_NORMAL, filter=ntg.FILTER_KAISER,
                                wrap=ntg.WRAP_MIRROR, alpha_mode=ntg.ALPHA_TRANSPARENCY, in_xform=ntg.XFORM_SRGB,
                                out_xform=ntg.XFORM_SRGB, max_levels=3)
    d_bgra, d_img = dev(bgra), dev(img)

    def run():
        lv = host(ctx.mip_level(d_img, fw, fh, filter=ntg.FILTER_KAISER, params=(4.0, 1.0), wrap=ntg.WRAP_MIRROR))
        return lv, host(ctx.mip_chain(d_bgra, w, h, opt)), host(ctx.compress_chain(d_bgra, w, h, opt))

    before = run()
    assert ctx.mip_status() == 0
    ctx.set_mip_wait_limit(0)
    try:
        run()
        assert ctx.mip_status() == 1
    finally:
        ctx.set_mip_wait_limit(-1)
    after = run()
    assert ctx.mip_status() == 0
    for a, b in zip(before, after):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


CHAINS = [
    # (w, h, format, quality, filter, alpha_mode, in_xform, out_xform, wrap)
    (128, 128, 1, 1, 0, 0, 0, 0, 2),    # the box/BC1/linear workload at reduced size
    (256, 256, 4, 1, 2, 1, 2, 2, 2),    # the Kaiser/sRGB/BC3/transparency workload at reduced size
    (64, 32, 7, 1, 1, 0, 0, 0, 1),      # BC5 normal map, triangle
    (96, 40, 4, 1, 1, 1, 1, 1, 0),      # gamma 2.2, triangle, clamp
    (37, 19, 1, 1, 2, 0, 1, 1, 2),      # odd sizes, Kaiser, BC1 + gamma
    (1, 64, 4, 1, 0, 1, 0, 0, 2),       # 1-D, box polyphase (transparency)
    (64, 1, 1, 0, 0, 0, 0, 0, 2),       # 1-D fast box, range fit
    (31, 31, 4, 3, 2, 0, 2, 2, 1),      # odd, Highest quality alpha
    (96, 64, 2, 1, 2, 1, 2, 2, 2),      # BC1a, Kaiser/sRGB, transparency
    (45, 27, 2, 2, 0, 0, 0, 0, 1),      # BC1a, box, odd sizes
    (64, 48, 6, 1, 1, 0, 0, 0, 2),      # BC4, triangle
    (37, 37, 6, 2, 2, 0, 1, 1, 0),      # BC4 Production, Kaiser, gamma
    (1, 4096, 4, 1, 2, 0, 0, 0, 2),     # 1-wide and tall: the tail's X plane keeps the full height
    (4096, 1, 1, 1, 2, 1, 2, 2, 1),     # 1-high and wide, sRGB
    (256, 192, 1, 1, 2, 1, 2, 2, 2),    # BC1 on float levels through the sRGB curve, transparency weights
    # level 1 from the BGRA8 input: tiles whose window lies inside the level take whole-vector copies
    (384, 128, 4, 1, 2, 1, 2, 2, 2),    # Kaiser / sRGB / BC3, interior tiles at (64, 16) and (64, 32)
    (320, 96, 1, 1, 1, 0, 0, 0, 1),     # triangle, repeat, BC1, interior tiles
    (50, 18, 4, 1, 2, 1, 2, 2, 2),      # rows of 50 words (not 16-byte multiples): wrapped copies only
]


def oracle_chain(oracle, bgra, w, h, fmt, quality, filt, am, ix, ox, wrap):
    width = {0: 0.5, 1: 1.0, 2: 3.0}[filt]
    lin, enc = oracle.mip_chain(bgra, w, h, filt, width, 4.0, 1.0, wrap, am, ix, ox, 2.2)
    out = []
    for l in enc:
        lw, lh = l.shape[2], l.shape[1]
        flat = l.reshape(-1)
        if fmt == 1:
            out.append(oracle.bc1_image(flat, lw, lh, am, quality, threads=8))
        elif fmt == 2:
            out.append(oracle.bc1a_image(flat, lw, lh, am, threads=8))
        elif fmt == 6:
            out.append(oracle.bc4_image(flat, lw, lh, quality, threads=8))
        elif fmt == 4:
            out.append(oracle.bc3_image(flat, lw, lh, am, quality, threads=8))
        else:
            out.append(oracle.bc5_image(flat, lw, lh, quality, threads=8))
    return lin, np.concatenate(out)


@pytest.mark.parametrize("case", CHAINS)
def test_chain_matches_oracle(ctx, oracle, case):
    w, h, fmt, quality, filt, am, ix, ox, wrap = case
    if fmt == 7:
        bgra = synth.normal_map(w, h, 5)
    else:
        bgra = synth.colour_texture(w, h, 11, scale=max(1.0, w / 512),
                                    alpha=synth.alpha_field(w, h, 11) if am else None)
    opt = ntg.ChainOptions.make(format=fmt, quality=quality, filter=filt, wrap=wrap, alpha_mode=am, in_xform=ix,
                                out_xform=ox, gamma=2.2)
    d_bgra = dev(bgra)
    levels = host(ctx.mip_chain(d_bgra, w, h, opt))
    blocks = host(ctx.compress_chain(d_bgra, w, h, opt))
    lin, ref_blocks = oracle_chain(oracle, bgra, w, h, fmt, quality, filt, am, ix, ox, wrap)
    ref_levels = np.concatenate([l.reshape(-1) for l in lin])
    assert np.array_equal(levels.view(np.uint32), ref_levels.view(np.uint32))
    assert np.array_equal(blocks, ref_blocks)


def test_chain_host_variant_matches_device_variant(ctx):
    w, h = 200, 120
    bgra = synth.colour_texture(w, h, 3, alpha=synth.alpha_field(w, h, 3))
    opt = ntg.ChainOptions.make(format=4, quality=1, filter=2, alpha_mode=1, in_xform=2, out_xform=2)
    a = host(ctx.compress_chain(dev(bgra), w, h, opt))
    b = ctx.compress_chain_host(bgra, w, h, opt)
    assert np.array_equal(a, b)


def test_chains_host_pipeline_matches_single_calls(ctx):
    """ntg_compress_chains_host (copies overlapped with the chains, double-buffered slots) gives each
    image exactly what its own ntg_compress_chain_host call gives."""
    w, h = 160, 96
    opt = ntg.ChainOptions.make(format=4, quality=1, filter=2, alpha_mode=1, in_xform=2, out_xform=2)
    imgs = [synth.colour_texture(w, h, 30 + i, alpha=synth.alpha_field(w, h, 30 + i)) for i in range(5)]
    outs = ctx.compress_chains_host(imgs, w, h, opt)
    for img, out in zip(imgs, outs):
        assert np.array_equal(out, ctx.compress_chain_host(img, w, h, opt))
    assert ctx.compress_chains_host([], w, h, opt) == []


def test_chain_golden_fixture(ctx):
    """The GPU chain against the reference's own bytes (tests/golden/chain_c0.npz)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "chain_c0.npz"))
    w, h = int(g["w"]), int(g["h"])
    opt = ntg.ChainOptions.make(format=1, quality=1, filter=0)
    out = host(ctx.compress_chain(dev(g["image"]), w, h, opt))
    assert np.array_equal(out, g["blocks"])


def test_srgb_quantizer_bucket_table_is_exact(ctx):
    """The mip kernels' sRGB quantiser (bucket table + one comparison) against the plain step search,
    on all 2^32 float bit patterns."""
    assert ctx.selftest_srgb_quantizer() == 0


# ---------------------------------------------------------------------------------------------
# resize (Surface::resize, the InputOptions resize step)

@pytest.mark.parametrize("w,h,dw,dh", [(61, 37, 64, 64), (100, 60, 40, 24), (64, 64, 16, 16), (4096 // 16, 48, 10, 7),
                                       (13, 9, 16, 16), (7, 3, 8, 4), (3, 200, 1, 50), (40, 40, 40, 10)])
@pytest.mark.parametrize("filt,width,p0,p1", [(0, 0.5, 0, 0), (1, 1.0, 0, 0), (2, 3.0, 4.0, 1.0)])
def test_resize_matches_oracle(ctx, oracle, w, h, dw, dh, filt, width, p0, p1):
    img = float_image(w, h, w * 7 + h + filt)
    for wrap in (0, 1, 2):
        ours = host(ctx.resize(dev(img), w, h, dw, dh, filter=filt, width=width, params=(p0, p1), wrap=wrap))
        ref = oracle.resize(img, w, h, dw, dh, filt, width, p0, p1, wrap)
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), wrap


def test_resize_to_same_extent_is_a_copy(ctx):
    img = float_image(9, 5, 3)
    assert np.array_equal(host(ctx.resize(dev(img), 9, 5, 9, 5)), img)


# ---------------------------------------------------------------------------------------------
# decode and error

@pytest.mark.parametrize("fmt", [1, 2, 4, 6, 7])
def test_decode_and_error_sums(ctx, oracle, fmt):
    w, h = 45, 27
    img = float_image(w, h, fmt, alpha_zero_frac=0.2)
    blocks = {1: lambda: oracle.bc1_image(img, w, h), 2: lambda: oracle.bc1a_image(img, w, h),
              4: lambda: oracle.bc3_image(img, w, h, 1), 6: lambda: oracle.bc4_image(img, w, h),
              7: lambda: oracle.bc5_image(img, w, h)}[fmt]()
    dec = host(ctx.decode(fmt, dev(blocks), w, h))
    assert np.array_equal(dec.view(np.uint32), oracle.decode(fmt, blocks, w, h).view(np.uint32))
    am = 1 if fmt == 4 else 0
    sums = host(ctx.error_sums(dev(img), dev(dec), w, h, alpha_mode=am))
    rc, ra = oracle.rms(fmt, img, blocks, w, h, am)
    assert abs(np.sqrt(sums[0] / (w * h)) - rc) <= 1e-6 * max(1.0, rc)
    assert abs(np.sqrt(sums[1] / (w * h)) - ra) <= 1e-6 * max(1.0, ra)


# ---------------------------------------------------------------------------------------------
# errors are reported, not hidden

def test_invalid_arguments_report_errors(ctx):
    opt = ntg.ChainOptions.make(format=3)  # BC2 (DXT3) is outside the path
    with pytest.raises(ntg.NtgError) as e:
        ctx.compress_chain(dev(np.zeros((4, 4, 4), np.uint8)), 4, 4, opt)
    assert e.value.code == 2
    with pytest.raises(ntg.NtgError) as e:
        ctx.mip_level(dev(np.zeros(4, np.float32)), 1, 1)
    assert e.value.code == 1
