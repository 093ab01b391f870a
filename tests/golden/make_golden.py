"""Writes the golden fixtures of tests/golden/ from the reference library built from its own
sources (oracle/ref/Makefile -> oracle/_ref/libnvtt_ref.so). Run where the reference tree exists:

    python tests/golden/make_golden.py [--ref /root/reference]

Inputs are seeded synthetic blocks and images (ntg.synth); outputs are exactly what the
reference produces for them. The fixtures let the oracle be checked on machines without the
reference tree."""
import argparse
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
    ap.add_argument("--ref", default=pyoracle.REF_SRC)
    args = ap.parse_args()
    path = pyoracle.build_reference(args.ref)
    if path is None:
        sys.exit("reference source tree not found")
    R = pyoracle.Reference(path)

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
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
