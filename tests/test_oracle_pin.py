"""Pins the oracle (C restatement, oracle/ntg_oracle.c) to the reference.

Two anchors: (1) the reference library compiled from its own sources (oracle/_ref), compared on
fresh seeded cases wherever the reference tree exists; (2) the committed golden fixtures in
tests/golden/, written by tests/golden/make_golden.py from that same reference build, compared
everywhere."""
import os

import numpy as np
import pytest

import ntg.synth as synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _blocks_float(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(n):
        k = t % 4
        if k == 0:
            c = rng.random((16, 4), dtype=np.float32)
        elif k == 1:
            c = (rng.integers(0, 256, (16, 4)) / 255.0).astype(np.float32)
        elif k == 2:
            c = np.clip(rng.random(4) + rng.normal(0, 0.02, (16, 4)), -0.1, 1.1).astype(np.float32)
        else:
            c = rng.random((3, 4))[rng.integers(0, 3, 16)].astype(np.float32)
        w = np.ones(16, np.float32)
        if t % 5 == 0:
            w = rng.random(16).astype(np.float32)
        if t % 7 == 0:
            w[rng.integers(0, 16, 5)] = 0
        out.append((c, w))
    return out


@pytest.mark.parametrize("level", [0, 7, 8])
def test_bc1_blocks_vs_reference(oracle, reference, level):
    for c, w in _blocks_float(600, 11 + level):
        a, ea = oracle.bc1_block(level, c, w)
        b, eb = reference.bc1_block(level, c, w)
        assert np.array_equal(a, b)
        assert ea == eb


@pytest.mark.parametrize("quality", [0, 1, 3])
@pytest.mark.parametrize("alpha_mode", [0, 1])
def test_bc3_blocks_vs_reference(oracle, reference, quality, alpha_mode):
    for blk in synth.random_blocks(400, 7 + quality):
        b = blk.reshape(64)
        assert np.array_equal(oracle.bc3_block(b, alpha_mode, quality), reference.bc3_block(b, alpha_mode, quality))


@pytest.mark.parametrize("quality", [1, 2])
def test_bc5_blocks_vs_reference(oracle, reference, quality):
    for blk in synth.random_blocks(300, 3):
        b = blk.reshape(64)
        assert np.array_equal(oracle.bc5_block(b, quality), reference.bc5_block(b, quality))


def _transparent_blocks(n, seed):
    rng = np.random.default_rng(seed)
    out = synth.random_blocks(n, seed).reshape(n, 64).copy()
    for t in range(n):
        a = out[t, 3::4]
        if t % 4 == 1:
            a[rng.integers(0, 16, 2)] = 0
        elif t % 4 == 2:
            a[rng.random(16) < 0.5] = 0
        elif t % 4 == 3:
            a[:] = 0
        out[t, 3::4] = a
    return out


@pytest.mark.parametrize("alpha_mode", [0, 1])
def test_bc1a_blocks_vs_reference(oracle, reference, alpha_mode):
    """CompressorDXT1a: transparent texels left out of the colour set, three-colour fit first,
    four-colour fit only without transparency, single colour through the midpoint tables."""
    for b in _transparent_blocks(600, 31 + alpha_mode):
        assert np.array_equal(oracle.bc1a_block(b, alpha_mode), reference.bc1a_block(b, alpha_mode))


def test_bc1a_single_colour_vs_reference(oracle, reference):
    rng = np.random.default_rng(8)
    for t in range(300):
        b = np.tile(rng.integers(0, 256, 4).astype(np.uint8), 16)
        b[3::4][rng.random(16) < (t % 3) * 0.4] = 0
        assert np.array_equal(oracle.bc1a_block(b, 0), reference.bc1a_block(b, 0))


@pytest.mark.parametrize("quality", [0, 1, 2, 3])
def test_bc4_blocks_vs_reference(oracle, reference, quality):
    for blk in synth.random_blocks(300, 41 + quality):
        b = blk.reshape(64)
        assert np.array_equal(oracle.bc4_block(b, quality), reference.bc4_block(b, quality))


def test_alpha_and_single_colour_vs_reference(oracle, reference):
    rng = np.random.default_rng(5)
    for t in range(800):
        a = rng.integers(0, 256, 16).astype(np.uint8)
        if t % 3 == 0:
            a = np.clip(rng.integers(100, 140) + rng.integers(-10, 10, 16), 0, 255).astype(np.uint8)
        if t % 5 == 0:
            a[rng.integers(0, 16, 4)] = rng.choice([0, 255])
        assert np.array_equal(oracle.dxt5a_quick(a), reference.dxt5a_quick(a))
        if t % 8 == 0:
            assert np.array_equal(oracle.dxt5a_optimal(a), reference.dxt5a_optimal(a))
    for r in range(0, 256, 5):
        for g in range(0, 256, 7):
            b = (r * 3 + g) % 256
            assert np.array_equal(oracle.dxt1_single_color(r, g, b), reference.dxt1_single_color(r, g, b))


@pytest.mark.parametrize("filt,width,p0,p1", [(0, 0.5, 0, 0), (1, 1.0, 0, 0), (2, 3.0, 4.0, 1.0), (2, 3.0, 2.0, 0.8)])
def test_polyphase_vs_reference(oracle, reference, filt, width, p0, p1):
    for src in [1, 2, 3, 5, 8, 13, 17, 64, 255, 256, 1000, 4096]:
        dst = max(1, src // 2)
        a = oracle.polyphase(filt, width, p0, p1, src, dst)
        b = reference.polyphase(filt, width, p0, p1, src, dst)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_gamma_vs_reference(oracle, reference):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.random(50000).astype(np.float32) * 2,
                        np.array([0, 1e-40, 1e-30, -1, np.inf, np.nan, 1e30, 3.4e38], np.float32),
                        (rng.standard_normal(5000) * 1e10).astype(np.float32)])
    for name in ("powf_11_5", "powf_5_11"):
        a, b = getattr(oracle, name)(x), getattr(reference, name)(x)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("size", [(16, 16), (17, 9), (1, 8), (8, 1), (13, 13), (5, 7), (64, 32)])
@pytest.mark.parametrize("filt,width,p0,p1", [(0, 0.5, 0, 0), (1, 1.0, 0, 0), (2, 3.0, 4.0, 1.0)])
def test_mip_chains_vs_reference(oracle, reference, size, filt, width, p0, p1):
    w, h = size
    rng = np.random.default_rng(w * 31 + h)
    for am in (0, 1):
        for ix, ox in ((0, 0), (1, 1), (2, 2)):
            wrap = (w + h + am + ix) % 3
            bgra = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
            la, ea = oracle.mip_chain(bgra, w, h, filt, width, p0, p1, wrap, am, ix, ox)
            lb, eb = reference.mip_chain(bgra, w, h, filt, width, p0, p1, wrap, am, ix, ox)
            assert len(la) == len(lb)
            for u, v in zip(la + ea, lb + eb):
                assert np.array_equal(u.view(np.uint32), v.view(np.uint32))


def test_weighted_resize_vs_reference(oracle, reference):
    rng = np.random.default_rng(9)
    for (w, h, dw, dh) in [(16, 16, 8, 8), (17, 9, 8, 4), (64, 32, 32, 16)]:
        for filt, width, p0, p1 in [(1, 1.0, 0, 0), (2, 3.0, 4.0, 1.0)]:
            img = rng.random(4 * w * h).astype(np.float32)
            a = oracle.resize_weighted(img, w, h, dw, dh, filt, width, p0, p1, 2)
            b = reference.resize_weighted(img, w, h, dw, dh, filt, width, p0, p1, 2)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("fmt,quality,alpha_mode", [(1, 1, 0), (1, 0, 1), (1, 2, 0), (4, 1, 1), (4, 0, 0), (7, 1, 0),
                                                    (2, 1, 0), (2, 2, 1), (6, 0, 0), (6, 1, 0)])
def test_images_vs_reference(oracle, reference, fmt, quality, alpha_mode):
    """Whole-image encodes through the reference's Compressor (gather, edges, dispatch). BC4/BC5 at
    Production are left to the block tests: OptimalCompress::compressDXT5A starts from the error
    of whatever the reference's output buffer held (src/nvtt/OptimalCompressDXT.cpp:546), so its
    whole-image output varies from run to run."""
    rng = np.random.default_rng(fmt * 10 + quality)
    for (w, h) in [(16, 16), (13, 7), (1, 1), (3, 5), (32, 20)]:
        img = rng.random(4 * w * h).astype(np.float32)
        img[3 * w * h:] = np.where(rng.random(w * h) < 0.3, 0.0, img[3 * w * h:])
        ref = reference.compress(img, w, h, fmt, quality, alpha_mode)
        if fmt == 1:
            ours = oracle.bc1_image(img, w, h, alpha_mode, quality, threads=2)
        elif fmt == 2:
            ours = oracle.bc1a_image(img, w, h, alpha_mode, threads=2)
        elif fmt == 6:
            ours = oracle.bc4_image(img, w, h, quality, threads=2)
        elif fmt == 4:
            ours = oracle.bc3_image(img, w, h, alpha_mode, quality, threads=2)
        else:
            ours = oracle.bc5_image(img, w, h, quality, threads=2)
        assert np.array_equal(ours, ref)


def test_target_extent_vs_reference(oracle, reference):
    """nv::getTargetExtent for every round mode, with and without a maximum extent (the library's
    own ntg_target_extent is held to the same values, and ntg_target_extent_ex for cube maps and arrays)."""
    import ntg
    for w in list(range(1, 40)) + [63, 64, 65, 100, 127, 1000, 4095]:
        for h in (1, 2, 3, 7, 64, 300):
            for me in (0, 1, 5, 16, 48, 64, 1000):
                for rm in range(7):
                    ref = reference.target_extent(w, h, me, rm)
                    assert oracle.target_extent(w, h, me, rm) == ref
                    assert ntg.target_extent(w, h, me, rm) == ref
                    for tt in (1, 3):  # cube map (square faces), array
                        assert ntg.target_extent(w, h, me, rm, tt) == reference.target_extent(w, h, me, rm, tt)


@pytest.mark.parametrize("alpha_mode", [0, 1])
def test_resize_vs_reference(oracle, reference, alpha_mode):
    """FloatImage::resize through Surface::resize, down and up, every wrap mode."""
    rng = np.random.default_rng(12)
    for (w, h, dw, dh) in [(61, 37, 64, 32), (64, 64, 16, 16), (100, 50, 64, 32), (13, 9, 16, 16), (7, 3, 8, 4)]:
        img = rng.random(4 * w * h).astype(np.float32)
        for filt, width, p0, p1 in [(0, 0.5, 0, 0), (1, 1.0, 0, 0), (2, 3.0, 4.0, 1.0)]:
            for wrap in (0, 1, 2):
                a = oracle.resize(img, w, h, dw, dh, filt, width, p0, p1, wrap)
                b = reference.surface_resize(img, w, h, dw, dh, filt, width, p0, p1, wrap, alpha_mode)
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_decode_and_rms_vs_reference(oracle, reference):
    rng = np.random.default_rng(4)
    for fmt in (1, 2, 4, 6, 7):
        w, h = 24, 12
        img = rng.random(4 * w * h).astype(np.float32)
        img[3 * w * h:][rng.random(w * h) < 0.2] = 0.0
        blocks = reference.compress(img, w, h, fmt, 1, 1 if fmt == 4 else 0)
        # the reference's Surface::setImage2D does not take BC1a; the block layout is BC1's
        dfmt = 1 if fmt == 2 else fmt
        assert np.array_equal(oracle.decode(fmt, blocks, w, h).view(np.uint32),
                              reference.decode(dfmt, blocks, w, h).view(np.uint32))
        am = 1 if fmt == 4 else 0
        assert oracle.rms(fmt, img, blocks, w, h, am) == reference.rms(dfmt, img, blocks, w, h, am)


# ---- golden fixtures (run everywhere) ----

def _golden(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail(f"missing golden fixture {name}; run tests/golden/make_golden.py")
    return np.load(path)


def test_golden_bc1_blocks(oracle):
    g = _golden("bc1_blocks.npz")
    for level in (0, 7, 8):
        cols, wts, outs = g[f"colors_{level}"], g[f"weights_{level}"], g[f"blocks_{level}"]
        for c, w, o in zip(cols, wts, outs):
            assert np.array_equal(oracle.bc1_block(level, c, w)[0], o)


def test_golden_bc3_bc5_blocks(oracle):
    g = _golden("bc3_bc5_blocks.npz")
    for key in g.files:
        if not key.startswith("bc3_"):
            continue
        _, q, am = key.split("_")
        for b, o in zip(g["inputs"], g[key]):
            assert np.array_equal(oracle.bc3_block(b, int(am), int(q)), o)
    for q in (1, 2):
        for b, o in zip(g["inputs"], g[f"bc5_{q}"]):
            assert np.array_equal(oracle.bc5_block(b, q), o)


def test_golden_bc1a_bc4_blocks(oracle):
    g = _golden("bc1a_bc4_blocks.npz")
    for am in (0, 1):
        for b, o in zip(g["inputs"], g[f"bc1a_{am}"]):
            assert np.array_equal(oracle.bc1a_block(b, am), o)
    for q in (1, 2):
        for b, o in zip(g["inputs"], g[f"bc4_{q}"]):
            assert np.array_equal(oracle.bc4_block(b, q), o)


def test_golden_mip_chains(oracle):
    g = _golden("mip_chains.npz")
    for key in g.files:
        if not key.startswith("case_"):
            continue
        w, h, filt, width, p0, p1, wrap, am, ix, ox = g[key]
        w, h, filt, wrap, am, ix, ox = (int(v) for v in (w, h, filt, wrap, am, ix, ox))
        bgra = g["img_" + key[5:]]
        lin, enc = oracle.mip_chain(bgra, w, h, filt, float(width), float(p0), float(p1), wrap, am, ix, ox)
        flat_lin = np.concatenate([v.reshape(-1) for v in lin])
        flat_enc = np.concatenate([v.reshape(-1) for v in enc])
        assert np.array_equal(flat_lin.view(np.uint32), g["lin_" + key[5:]].view(np.uint32))
        if ox != 2:  # sRGB encode goes through the host libm's powf, which may differ by machine
            assert np.array_equal(flat_enc.view(np.uint32), g["enc_" + key[5:]].view(np.uint32))


def test_golden_chain_c0(oracle):
    """The 512x512 box-filtered BC1 chain (the CPU-runnable workload), end to end."""
    g = _golden("chain_c0.npz")
    bgra, w, h = g["image"], int(g["w"]), int(g["h"])
    lin, _ = oracle.mip_chain(bgra, w, h, 0, 0.5, 0.0, 0.0, 2, 0, 0, 0)
    out = np.concatenate([oracle.bc1_image(l.reshape(-1), l.shape[2], l.shape[1], 0, 1, threads=4) for l in lin])
    assert np.array_equal(out, g["blocks"])
