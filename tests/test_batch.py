"""Batches (ntg_batch_*): many textures' chains in one CUDA graph. Every texture's blocks must equal
what the single-chain path (ntg_compress_chain, itself pinned to the oracle) gives with the same
options, and a few are checked against the oracle directly; graph replays, new inputs written into
the same buffers, and the autotuner's launch shapes must not change a byte."""
import json
import os

import numpy as np
import pytest

import ntg
import ntg.synth as synth
from test_gpu_parity import oracle_chain

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


# (w, h, format, quality, filter, alpha_mode, in_xform, out_xform, wrap, weighted)
MIXED = [
    (256, 256, 4, 1, 2, 1, 2, 2, 2, 0),   # the Kaiser / sRGB / BC3 / transparency chain
    (128, 128, 1, 1, 0, 0, 0, 0, 2, 0),   # box / BC1 / linear (fast box path, level 0 materialised)
    (64, 32, 7, 1, 1, 0, 0, 0, 1, 0),     # BC5 normal map, triangle, repeat
    (96, 40, 4, 1, 1, 1, 1, 1, 0, 0),     # gamma 2.2, triangle, clamp
    (37, 19, 1, 1, 2, 0, 1, 1, 2, 0),     # odd sizes, Kaiser, BC1 + gamma
    (1, 64, 4, 1, 0, 1, 0, 0, 2, 0),      # 1-D, polyphase box (transparency)
    (64, 1, 1, 0, 0, 0, 0, 0, 2, 0),      # 1-D fast box, range fit
    (31, 31, 4, 3, 2, 0, 2, 2, 1, 0),     # odd, Highest quality alpha
    (16, 16, 1, 2, 2, 0, 2, 2, 2, 0),     # smaller than the tail threshold from level 0, Production
    (512, 64, 4, 0, 1, 1, 2, 2, 2, 0),    # non-square, Fastest BC3
    (8, 8, 7, 2, 1, 0, 0, 0, 2, 0),       # tiny BC5 Production
    (64, 64, 4, 1, 2, 1, 0, 0, 2, 1),     # alpha-weighted Kaiser taps
    (128, 32, 1, 1, 1, 1, 2, 2, 2, 1),    # alpha-weighted triangle, BC1 + sRGB
    (256, 128, 1, 1, 2, 0, 2, 2, 0, 0),   # Kaiser clamp, BC1 + sRGB
    (128, 64, 2, 1, 2, 1, 2, 2, 2, 0),    # BC1a, Kaiser / sRGB / transparency
    (64, 64, 6, 1, 1, 0, 0, 0, 2, 0),     # BC4, triangle
    (32, 48, 6, 2, 0, 0, 0, 0, 2, 0),     # BC4 Production, box
]


def options(c):
    w, h, fmt, q, filt, am, ix, ox, wrap, weighted = c
    return ntg.ChainOptions.make(format=fmt, quality=q, filter=filt, wrap=wrap, alpha_mode=am, in_xform=ix,
                                 out_xform=ox, gamma=2.2, weighted=weighted)


def image(c, seed):
    w, h, fmt = c[0], c[1], c[2]
    if fmt == 7:
        return synth.normal_map(w, h, seed)
    rng = np.random.default_rng(seed)
    return synth.colour_texture(w, h, seed, scale=0.25, alpha=rng.integers(0, 256, (h, w)).astype(np.uint8))


def make_batch(ctx, cases, seed0):
    imgs, textures, refs = [], [], []
    for i, c in enumerate(cases):
        img = image(c, seed0 + i)
        d_in = dev(img.reshape(-1).view(np.uint32))
        opt = options(c)
        out = dev(np.zeros(ntg.chain_bytes(c[0], c[1], opt), np.uint8))
        imgs.append(img)
        textures.append((d_in, c[0], c[1], opt, out))
        refs.append(host(ctx.compress_chain(d_in, c[0], c[1], opt)))
    return imgs, textures, refs


def test_batch_matches_single_chains(ctx, tmp_path, monkeypatch):
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    _, textures, refs = make_batch(ctx, MIXED, 100)
    b = ntg.Batch(ctx, textures)
    try:
        for t, r in zip(textures, refs):  # build() ran the sequence once
            assert np.array_equal(host(t[4]), r)
        for t in textures:
            t[4].zero_()
        b.launch()
        b.launch()  # replays are idempotent
        for t, r in zip(textures, refs):
            assert np.array_equal(host(t[4]), r)
        info = b.info()
        assert info["texels"] == sum(sum(lw * lh for lw, lh in ntg.chain_levels(c[0], c[1])) for c in MIXED)
        assert info["launches"] < 4 * 10 + 8  # grouped by depth, not one launch per texture level
    finally:
        b.close()


def test_batch_new_inputs_in_same_buffers(ctx, tmp_path, monkeypatch):
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    cases = MIXED[:6]
    _, textures, _ = make_batch(ctx, cases, 200)
    b = ntg.Batch(ctx, textures)
    try:
        refs = []
        for i, (c, t) in enumerate(zip(cases, textures)):
            img = image(c, 900 + i)
            t[0].copy_(dev(img.reshape(-1).view(np.uint32)))
            refs.append(host(ctx.compress_chain(t[0], c[0], c[1], t[3])))
        b.launch()
        for t, r in zip(textures, refs):
            assert np.array_equal(host(t[4]), r)
    finally:
        b.close()


def test_alternate_binding(ctx, tmp_path, monkeypatch):
    """A second set of inputs and outputs with its own graph: each binding encodes its own images,
    replays of either leave the other's outputs alone, and autotuning recaptures both."""
    import torch
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    cases = MIXED[:8]
    _, textures, refs = make_batch(ctx, cases, 400)
    b = ntg.Batch(ctx, textures)
    try:
        alt_in, alt_out, alt_refs = [], [], []
        for i, (c, t) in enumerate(zip(cases, textures)):
            img = image(c, 1400 + i)
            alt_in.append(dev(img.reshape(-1).view(np.uint32)))
            alt_out.append(torch.zeros_like(t[4]))
            alt_refs.append(host(ctx.compress_chain(alt_in[-1], c[0], c[1], t[3])))
        b.bind_alternate(alt_in, alt_out)
        for y in alt_out:
            y.zero_()
        for t in textures:
            t[4].zero_()
        b.launch(alternate=True)
        for y, r in zip(alt_out, alt_refs):
            assert np.array_equal(host(y), r)
        for t in textures:
            assert not host(t[4]).any()
        b.launch()
        for t, r in zip(textures, refs):
            assert np.array_equal(host(t[4]), r)
        b.autotune()
        for y in alt_out:
            y.zero_()
        b.launch(alternate=True)
        b.launch()
        for y, r in zip(alt_out, alt_refs):
            assert np.array_equal(host(y), r)
        for t, r in zip(textures, refs):
            assert np.array_equal(host(t[4]), r)
    finally:
        b.close()


@pytest.mark.parametrize("alternate", [False, True])
def test_process_host_sets(ctx, tmp_path, monkeypatch, alternate):
    """ntg_batch_process_host: several sets of host images through the batch, each set's host blocks
    equal to the single-chain encodes of its images, with one binding (sets in turn) and with two
    (copies beside the neighbouring sets' graphs; page-locked and pageable host buffers)."""
    import torch
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    cases = MIXED[:6]
    _, textures, _ = make_batch(ctx, cases, 500)
    b = ntg.Batch(ctx, textures)
    try:
        if alternate:
            b.bind_alternate([torch.empty_like(t[0]) for t in textures], [torch.empty_like(t[4]) for t in textures])
        sets, refs = [], []
        for k in range(5):
            ins, outs, rs = [], [], []
            for i, (c, t) in enumerate(zip(cases, textures)):
                img = image(c, 2000 + 10 * k + i).reshape(-1).view(np.uint32)
                x = torch.from_numpy(img.copy())
                ins.append(x.pin_memory() if k % 2 == 0 else x)
                y = torch.zeros(t[4].numel(), dtype=torch.uint8)
                outs.append(y.pin_memory() if k % 2 == 0 else y)
                rs.append(host(ctx.compress_chain(dev(img), c[0], c[1], t[3])))
            sets.append((ins, outs))
            refs.append(rs)
        b.process_host(sets)
        for (ins, outs), rs in zip(sets, refs):
            for y, r in zip(outs, rs):
                assert np.array_equal(y.numpy(), r)
    finally:
        b.close()


def test_autotune_keeps_results_and_caches_shape(ctx, tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("NTG_TUNE_CACHE", str(cache))
    _, textures, refs = make_batch(ctx, MIXED, 300)
    b = ntg.Batch(ctx, textures)
    try:
        b.autotune()
        shape = b.info()["shape"]
        for t in textures:
            t[4].zero_()
        b.launch()
        for t, r in zip(textures, refs):
            assert np.array_equal(host(t[4]), r)
    finally:
        b.close()
    entries = json.loads(cache.read_text())["entries"]
    assert len(entries) == 1 and entries[0]["strip"] == shape["strip"] and entries[0]["bc3"] == shape["bc3_blocks_per_cta"]
    b2 = ntg.Batch(ctx, textures)  # same device and textures: the cached shape is used
    try:
        assert b2.info()["shape"] == shape
    finally:
        b2.close()


def test_batch_c2_mix_matches_oracle(ctx, oracle, tmp_path, monkeypatch):
    """The batched workload's mix (BC1/BC3/BC5, triangle mips, fBm normal maps) at small sizes,
    checked against the oracle itself."""
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    specs = synth.batch_specs(12, 77, 3, 7)
    textures = []
    for (w, h, fmt, seed) in specs:
        img = synth.batch_texture(w, h, fmt, seed)
        opt = ntg.ChainOptions.make(format=fmt, quality=1, filter=ntg.FILTER_TRIANGLE, wrap=ntg.WRAP_MIRROR,
                                    alpha_mode=ntg.ALPHA_TRANSPARENCY if fmt == 4 else ntg.ALPHA_NONE,
                                    in_xform=ntg.XFORM_SRGB if fmt != 7 else ntg.XFORM_NONE,
                                    out_xform=ntg.XFORM_SRGB if fmt != 7 else ntg.XFORM_NONE)
        out = dev(np.zeros(ntg.chain_bytes(w, h, opt), np.uint8))
        textures.append((dev(img.reshape(-1).view(np.uint32)), w, h, opt, out, img))
    b = ntg.Batch(ctx, [t[:5] for t in textures])
    try:
        b.launch()
        for (d_in, w, h, opt, out, img) in textures:
            if opt.format == 1:
                continue  # BC1 levels after a float sRGB transform use the device powf (checked elsewhere)
            _, ref = oracle_chain(oracle, img, w, h, opt.format, 1, 1, opt.alpha_mode, opt.in_xform, opt.out_xform, 2)
            assert np.array_equal(host(out), ref), (w, h, opt.format)
    finally:
        b.close()


def test_batch_rejects_bad_input(ctx):
    with pytest.raises(ntg.NtgError):
        ntg.Batch(ctx, [])


def test_batch_learned_proposal_wide_radius_is_exact(ctx, tmp_path, monkeypatch):
    """With the proposal's search covering every ordering, the batch's BC1 blocks through the
    learned path equal the full fit's; clearing the proposal restores the plain graph."""
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    _, textures, refs = make_batch(ctx, MIXED, 500)
    net = ntg.MLP(seed=4)
    b = ntg.Batch(ctx, textures)
    try:
        launches = b.info()["launches"]
        b.set_proposal(net, radius=16, margin=float("inf"))
        assert b.info()["launches"] == launches + 3
        for t in textures:
            t[4].zero_()
        b.launch()
        for t, r in zip(textures, refs):
            assert np.array_equal(host(t[4]), r)
        st = b.proposal_stats()
        assert st["kept"] > 0 and st["full_fit"] == 0
        b.set_proposal(None)
        assert b.info()["launches"] == launches
    finally:
        b.close()
        net.close()


@pytest.mark.gpu
def test_count_work_orderings(ctx, tmp_path, monkeypatch):
    """ntg_batch_count_work: a block of 16 distinct bright colours evaluates every ordering (968 four-
    cluster, 152 three-cluster); with eight black colours among its 16, the three-cluster fit runs over
    the other eight (44 orderings); a solid block runs no fit."""
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    w, h = 12, 4  # three blocks, level 0 only
    img = np.zeros((h, w, 4), np.uint8)  # B, G, R, A
    img[..., 3] = 255
    for k in range(16):
        y, x = k // 4, k % 4
        img[y, x] = (100, 200, 64 + 8 * k, 255)                  # block 0: bright, distinct
        img[y, 4 + x] = (0, 0, 3 * k, 255) if k < 8 else (100, 200, 64 + 8 * k, 255)  # block 1: 8 black
        img[y, 8 + x] = (30, 60, 90, 255)                        # block 2: one colour
    opt = ntg.ChainOptions.make(format=ntg.FORMAT_BC1, quality=ntg.QUALITY_NORMAL, max_levels=1)
    d_in = dev(img.reshape(-1).view(np.uint32))
    out = dev(np.zeros(ntg.chain_bytes(w, h, opt), np.uint8))
    b = ntg.Batch(ctx, [(d_in, w, h, opt, out)])
    try:
        assert b.count_work() == (968 + 968, 152 + 44)
    finally:
        b.close()
