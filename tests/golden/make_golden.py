"""Writes the golden fixtures of tests/golden/ from the reference library built from its own
sources (oracle/ref/Makefile -> oracle/_ref/libnvtt_ref.so). Run where the reference tree exists:

    python tests/golden/make_golden.py [--ref /root/reference]

Inputs are seeded synthetic blocks and images (ntg.synth); outputs are exactly what the
reference produces for them. The fixtures let the oracle be checked on machines without the
reference tree."""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "nvidia-texture-tools_gb300")]

import pyoracle  # noqa: E402
import ntg.synth as synth  # noqa: E402


def float_blocks(n, seed):
    rng = np.random.default_rng(seed)
    cols, wts = [], []
    for t in range(n):
        k = t % 4
        if k == 0:
            c = rng.random((16, 4), dtype=np.float32)
        elif k == 1:
            c = (rng.integers(0, 256, (16, 4)) / 255.0).astype(np.float32)
        elif k == 2:
            c = np.clip(rng.random(4) + rng.normal(0, 0.03, (16, 4)), -0.1, 1.1).astype(np.float32)
        else:
            c = rng.random((2 + t % 3, 4))[rng.integers(0, 2 + t % 3, 16)].astype(np.float32)
        w = np.ones(16, np.float32)
        if t % 5 == 0:
            w = rng.random(16).astype(np.float32)
        if t % 7 == 0:
            w[rng.integers(0, 16, 6)] = 0
        if t % 23 == 0:
            c[:, :3] *= 0.05  # near-black blocks exercise the transparent-black three-colour path
        cols.append(c)
        wts.append(w)
    return np.array(cols), np.array(wts)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference source tree (default: $NTG_REFERENCE_ROOT, else the recipe's)")
    ap.add_argument("--only", choices=["blocks", "dds", "bc1a_bc4"],
                    help="write only the block/chain, the DDS or the BC1a/BC4 block fixtures")
    args = ap.parse_args()
    path = pyoracle.build_reference(args.ref)
    if path is None:
        sys.exit("reference source tree not found")
    R = pyoracle.Reference(path)
    if args.only in (None, "blocks"):
        write_block_fixtures(R)
    if args.only in (None, "dds"):
        write_dds_fixtures(R)
    if args.only in (None, "bc1a_bc4"):
        write_bc1a_bc4_fixtures(R)
    print("fixtures written to", HERE)


def transparent_blocks(n, seed):
    """Synthetic 4x4 BGRA8 blocks with zero-alpha texels planted: none, a seeded few, about a
    third, or all sixteen (the BC1a cases)."""
    rng = np.random.default_rng(seed)
    blocks = synth.random_blocks(n, seed).reshape(n, 64).copy()
    for t in range(n):
        a = blocks[t, 3::4]
        k = t % 4
        if k == 1:
            a[rng.integers(0, 16, 3)] = 0
        elif k == 2:
            a[rng.random(16) < 0.35] = 0
        elif k == 3:
            a[:] = 0
        blocks[t, 3::4] = a
    return blocks


def write_bc1a_bc4_fixtures(R):
    blocks = transparent_blocks(400, 77)
    out = {"inputs": blocks}
    for am in (0, 1):
        out[f"bc1a_{am}"] = np.array([R.bc1a_block(b, am) for b in blocks])
    for q in (1, 2):
        out[f"bc4_{q}"] = np.array([R.bc4_block(b, q) for b in blocks])
    np.savez_compressed(os.path.join(HERE, "bc1a_bc4_blocks.npz"), **out)


def write_block_fixtures(R):

    out = {}
    for level in (0, 7, 8):
        cols, wts = float_blocks(240, 100 + level)
        out[f"colors_{level}"] = cols
        out[f"weights_{level}"] = wts
        out[f"blocks_{level}"] = np.array([R.bc1_block(level, c, w)[0] for c, w in zip(cols, wts)])
    np.savez_compressed(os.path.join(HERE, "bc1_blocks.npz"), **out)

    blocks = synth.random_blocks(300, 2024).reshape(300, 64)
    out = {"inputs": blocks}
    for q in (0, 1, 3):
        for am in (0, 1):
            out[f"bc3_{q}_{am}"] = np.array([R.bc3_block(b, am, q) for b in blocks])
    for q in (1, 2):
        out[f"bc5_{q}"] = np.array([R.bc5_block(b, q) for b in blocks])
    np.savez_compressed(os.path.join(HERE, "bc3_bc5_blocks.npz"), **out)

    cases = [
        (16, 16, 0, 0.5, 0, 0, 2, 0, 0, 0), (17, 9, 0, 0.5, 0, 0, 2, 0, 1, 1), (32, 16, 1, 1.0, 0, 0, 0, 0, 0, 0),
        (13, 13, 1, 1.0, 0, 0, 1, 1, 2, 2), (32, 32, 2, 3.0, 4.0, 1.0, 2, 1, 2, 2), (24, 20, 2, 3.0, 4.0, 1.0, 2, 0, 1, 1),
        (5, 7, 2, 3.0, 4.0, 1.0, 0, 0, 0, 0), (1, 16, 1, 1.0, 0, 0, 2, 0, 0, 0), (16, 1, 0, 0.5, 0, 0, 2, 0, 0, 0),
    ]
    rng = np.random.default_rng(77)
    out = {}
    for i, c in enumerate(cases):
        w, h = c[0], c[1]
        img = synth.colour_texture(w, h, 500 + i, scale=0.125, alpha=rng.integers(0, 256, (h, w)).astype(np.uint8))
        lin, enc = R.mip_chain(img, w, h, c[2], c[3], c[4], c[5], c[6], c[7], c[8], c[9])
        out[f"case_{i}"] = np.array(c, np.float64)
        out[f"img_{i}"] = img
        out[f"lin_{i}"] = np.concatenate([v.reshape(-1) for v in lin])
        out[f"enc_{i}"] = np.concatenate([v.reshape(-1) for v in enc])
    np.savez_compressed(os.path.join(HERE, "mip_chains.npz"), **out)

    w = h = 128
    img = synth.texture_c0(seed=0x4E565454, w=w, h=h)
    lin, _ = R.mip_chain(img, w, h, 0, 0.5, 0.0, 0.0, 2, 0, 0, 0)
    blocks = np.concatenate([R.compress(l.reshape(-1), l.shape[2], l.shape[1], 1, 1, 0) for l in lin])
    np.savez_compressed(os.path.join(HERE, "chain_c0.npz"), image=img, w=w, h=h, blocks=blocks)


def write_dds_fixtures(R):
    out = {}
    for i, case in enumerate(DDS_CASES):
        data = dds_input(i, case)
        res = R.process_ex(data, case["w"], case["h"], case["format"], **{k: v for k, v in case.items()
                                                                         if k not in ("w", "h", "format")})
        out[f"params_{i}"] = np.array(json.dumps(case))
        out[f"input_{i}"] = data
        out[f"dds_{i}"] = res if isinstance(res, np.ndarray) else np.array([res], np.int64)
        if case.get("input_format", 0) == 0 and case["format"] in (1, 4, 6, 7):
            # rmsError / rmsAlphaError of level 0 encoded without transforms, against its input
            w, h = case["w"], case["h"]
            bgra = data[:4 * w * h].reshape(h, w, 4)
            planar = np.stack([bgra[..., c].astype(np.float32) / np.float32(255) for c in (2, 1, 0, 3)])
            am = case.get("alpha_mode", 0)
            blocks = R.compress(planar.reshape(-1), w, h, case["format"], case.get("quality", 1), am,
                                case.get("cw", (1, 1, 1, 1)))
            out[f"rms_{i}"] = np.array(R.rms(case["format"], planar.reshape(-1), blocks, w, h, am), np.float32)
    np.savez_compressed(os.path.join(HERE, "dds_process.npz"), **out)


# Compressor::process cases for the nvtt:: drop-in API: containers, header flags, filters, gammas,
# source mipmaps, float input, one format the DDS container rejects (BC7 -> Error 6), and BC1a /
# BC4 (BC4 at Normal and Fastest only: the reference's Production BC4 varies from run to run), and the
# InputOptions resize step (max extent, round modes).
DDS_CASES = [
    dict(w=61, h=37, format=1, quality=1, mip_filter=0),
    dict(w=64, h=64, format=4, quality=1, mip_filter=2, alpha_mode=1, srgb=1, version=7),
    dict(w=48, h=40, format=7, quality=2, mip_filter=1, gamma=(1.0, 1.0), container=1, normal_map=1, normalize_mips=0),
    dict(w=32, h=32, format=1, quality=0, max_level=0, container=1, srgb=1),
    dict(w=40, h=24, format=4, quality=0, max_level=3, wrap=0, cw=(0.5, 1.0, 0.25, 1.0)),
    dict(w=32, h=32, format=1, quality=2, nsrc_levels=2),
    dict(w=24, h=24, format=4, quality=1, mip_filter=1, input_format=2),
    dict(w=16, h=16, format=1, quality=1, mip_filter=2, input_format=1, gamma=(1.0, 1.0), kaiser=(2.0, 6.0, 0.75)),
    dict(w=17, h=9, format=4, quality=1, mip_filter=2, alpha_mode=1, wrap=1, header=False),
    dict(w=3, h=5, format=1, quality=1),
    dict(w=20, h=12, format=7, quality=1, mip_filter=0, normal_map=1, normalize_mips=0),
    dict(w=16, h=16, format=11, quality=1),
    dict(w=40, h=28, format=2, quality=1, mip_filter=2, alpha_mode=1),
    dict(w=32, h=20, format=2, quality=2, container=1, srgb=1),
    dict(w=36, h=36, format=6, quality=1, mip_filter=1),
    dict(w=16, h=24, format=6, quality=0, container=1),
    dict(w=61, h=37, format=1, quality=1, mip_filter=2, round_mode=1),                 # up to 64 x 64
    dict(w=100, h=60, format=4, quality=1, mip_filter=1, alpha_mode=1, max_extent=40),  # down to 40 x 24
    dict(w=70, h=50, format=7, quality=1, max_extent=64, round_mode=3, wrap=1),         # 64 x 32 after rounding
    dict(w=23, h=41, format=1, quality=0, round_mode=4, gamma=(1.0, 1.0), container=1),  # 24 x 44
    dict(w=30, h=18, format=2, quality=1, round_mode=2, alpha_mode=1),                  # 32 x 16
    dict(w=45, h=27, format=4, quality=1, round_mode=5, max_level=1),                   # unchanged (reference quirk)
    dict(w=3, h=9, format=1, quality=1, round_mode=6),                                  # width 0: rejected
    # cube maps (six faces, each a whole chain, face by face) and texture arrays
    dict(w=32, h=32, format=1, quality=1, mip_filter=2, texture_type=1),
    dict(w=24, h=24, format=4, quality=1, mip_filter=1, alpha_mode=1, texture_type=1, container=1, srgb=1),
    dict(w=40, h=24, format=7, quality=1, texture_type=1, max_extent=16, round_mode=1),   # (40+24)/2 -> 16
    dict(w=20, h=12, format=4, quality=1, mip_filter=2, texture_type=3, layers=3, container=1),
    dict(w=16, h=16, format=1, quality=2, texture_type=3, layers=2),                    # array in a DDS9 file
    dict(w=16, h=16, format=4, quality=1, mip_filter=1, alpha_mode=1, texture_type=1, nsrc_levels=2),  # faces' own mips
    dict(w=12, h=20, format=1, quality=1, texture_type=3, layers=2, input_format=2, container=1, srgb=1),
    dict(w=8, h=8, format=7, quality=1, texture_type=1, max_level=1),                   # one level: no mipmap caps
]


def dds_input(i, case):
    """Seeded input of DDS case i: BGRA8 levels (source mipmaps included) or interleaved float RGBA."""
    w, h = case["w"], case["h"]
    levels = pyoracle.level_sizes(w, h)[:case.get("nsrc_levels", 1)]
    fmt = case.get("input_format", 0)
    tt = case.get("texture_type", 0)
    faces = 6 if tt == 1 else (case.get("layers", 1) if tt == 3 else 1)
    parts = []
    for f in range(faces):  # face (or layer) by face, each with its source levels
        for j, (lw, lh) in enumerate(levels):
            s = 9000 + 10 * i + j + 100 * f
            rng = np.random.default_rng(s)
            img = synth.colour_texture(lw, lh, s - 8100, scale=0.2, alpha=rng.integers(0, 256, (lh, lw)).astype(np.uint8))
            if fmt == 0:
                parts.append(img.reshape(-1))
            else:
                rgba = img[..., [2, 1, 0, 3]].astype(np.float32) / 255.0 + rng.normal(0, 0.01, (lh, lw, 4)).astype(np.float32)
                rgba = np.clip(rgba, 0, 1).astype(np.float32)
                parts.append((rgba.astype(np.float16) if fmt == 1 else rgba).reshape(-1).view(np.uint8))
    return np.concatenate(parts)


if __name__ == "__main__":
    main()
