"""Seeded synthetic textures of the benchmark workloads (stand-ins: no dataset is used).

All images are returned as (h, w, 4) uint8 in BGRA order, the layout nvtt's InputFormat_BGRA_8UB
expects. Generators are deterministic per seed on a given machine.

  colour_texture  -- sum of 4 sinusoid octaves (1/256 .. 1/32 px^-1, divided by `scale`), seeded
                     orientation/phase, 12 hard-edged rectangles, uniform noise of +-8, alpha 255
  alpha_field     -- value noise in 0..255 with 30% of texels (seeded mask) snapped to 0 or 255
  normal_map      -- 5-octave fBm height -> central differences -> normalised -> RG8
  batch_specs     -- the mixed batches: power-of-two sizes drawn per axis, 80% square, formats
                     50% BC1 / 30% BC3 / 20% BC5
"""
from __future__ import annotations

import numpy as np

TWO_PI = 2.0 * np.pi


def colour_texture(w: int, h: int, seed: int, scale: float = 1.0, alpha: np.ndarray | None = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    xs = np.arange(w, dtype=np.float32)[None, :]
    ys = np.arange(h, dtype=np.float32)[:, None]
    rgb = np.full((h, w, 3), 128.0, np.float32)
    for o in range(4):
        f = (1.0 / 256.0) * (2 ** o) / scale
        amp = 56.0 / (2 ** o)
        theta = rng.uniform(0, TWO_PI)
        proj = (xs * np.float32(np.cos(theta)) + ys * np.float32(np.sin(theta))) * np.float32(TWO_PI * f)
        for c in range(3):
            rgb[..., c] += np.float32(amp) * np.sin(proj + np.float32(rng.uniform(0, TWO_PI)))
    for _ in range(12):
        rw = int(rng.integers(16, 129) * scale)
        rh = int(rng.integers(16, 129) * scale)
        x0 = int(rng.integers(0, max(1, w - min(rw, w) + 1)))
        y0 = int(rng.integers(0, max(1, h - min(rh, h) + 1)))
        rgb[y0:y0 + rh, x0:x0 + rw, :] = rng.integers(0, 256, 3).astype(np.float32)
    rgb += rng.uniform(-8.0, 8.0, size=rgb.shape).astype(np.float32)
    out = np.empty((h, w, 4), np.uint8)
    q = np.clip(np.rint(rgb), 0, 255).astype(np.uint8)
    out[..., 0], out[..., 1], out[..., 2] = q[..., 2], q[..., 1], q[..., 0]
    out[..., 3] = 255 if alpha is None else alpha
    return out


def _value_noise(w: int, h: int, cell: float, rng) -> np.ndarray:
    gw, gh = int(np.ceil(w / cell)) + 2, int(np.ceil(h / cell)) + 2
    lattice = rng.random((gh, gw), dtype=np.float32)
    fx = np.arange(w, dtype=np.float32) / np.float32(cell)
    fy = np.arange(h, dtype=np.float32) / np.float32(cell)
    ix, iy = fx.astype(np.int64), fy.astype(np.int64)
    tx, ty = fx - ix, fy - iy
    tx = tx * tx * (3 - 2 * tx)
    ty = ty * ty * (3 - 2 * ty)
    a = lattice[iy][:, ix]
    b = lattice[iy][:, ix + 1]
    c = lattice[iy + 1][:, ix]
    d = lattice[iy + 1][:, ix + 1]
    top = a + (b - a) * tx[None, :]
    bot = c + (d - c) * tx[None, :]
    return top + (bot - top) * ty[:, None]


def alpha_field(w: int, h: int, seed: int, scale: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed ^ 0x5A5A5A5A)
    v = _value_noise(w, h, 32.0 * scale, rng) * 0.65 + _value_noise(w, h, 8.0 * scale, rng) * 0.35
    a = np.clip(np.rint(v * 255.0), 0, 255).astype(np.uint8)
    snap = rng.random((h, w), dtype=np.float32) < 0.3
    a[snap] = np.where(a[snap] < 128, 0, 255).astype(np.uint8)
    return a


def normal_map(w: int, h: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed ^ 0x3C3C3C3C)
    height = np.zeros((h, w), np.float32)
    amp = 1.0
    for o in range(5):
        cell = max(2.0, min(w, h) / (4.0 * 2 ** o))
        height += np.float32(amp) * _value_noise(w, h, cell, rng)
        amp *= 0.5
    k = np.float32(4.0)
    dx = (np.roll(height, -1, axis=1) - np.roll(height, 1, axis=1)) * k
    dy = (np.roll(height, -1, axis=0) - np.roll(height, 1, axis=0)) * k
    nz = np.ones_like(dx)
    inv = 1.0 / np.sqrt(dx * dx + dy * dy + nz * nz)
    nx, ny = -dx * inv, -dy * inv
    out = np.empty((h, w, 4), np.uint8)
    out[..., 2] = np.clip(np.rint((nx * 0.5 + 0.5) * 255.0), 0, 255).astype(np.uint8)
    out[..., 1] = np.clip(np.rint((ny * 0.5 + 0.5) * 255.0), 0, 255).astype(np.uint8)
    out[..., 0] = 0
    out[..., 3] = 255
    return out


def texture_c0(seed: int = 0x4E565454, w: int = 512, h: int = 512) -> np.ndarray:
    """512x512 opaque colour texture (BC1, box mips, linear)."""
    return colour_texture(w, h, seed)


def texture_c1(seed: int = 0x47423330, w: int = 4096, h: int = 4096) -> np.ndarray:
    """4096x4096 sRGB colour texture at 8x scale with an independent alpha field (BC3, Kaiser)."""
    scale = 8.0 * w / 4096.0
    return colour_texture(w, h, seed, scale=scale, alpha=alpha_field(w, h, seed, scale=scale))


def batch_specs(count: int, seed: int, kmin: int, kmax: int):
    """(w, h, format, seed) per texture: sizes 2^k per axis, 80% square; 50/30/20 BC1/BC3/BC5."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        kw = int(rng.integers(kmin, kmax + 1))
        kh = kw if rng.random() < 0.8 else int(rng.integers(kmin, kmax + 1))
        u = rng.random()
        fmt = 1 if u < 0.5 else (4 if u < 0.8 else 7)
        specs.append((1 << kw, 1 << kh, fmt, int(rng.integers(0, 2 ** 31))))
    return specs


def batch_texture(w: int, h: int, fmt: int, seed: int) -> np.ndarray:
    if fmt == 7:
        return normal_map(w, h, seed)
    scale = max(1.0, min(w, h) / 512.0)
    if fmt == 4:
        return colour_texture(w, h, seed, scale=scale, alpha=alpha_field(w, h, seed, scale=scale))
    return colour_texture(w, h, seed, scale=scale)


def _batch_image(args):
    w, h, fmt, seed = args
    return batch_texture(w, h, fmt, seed)


def batch_workload(count: int, seed: int, kmin: int, kmax: int, workers: int = 0):
    """The textures of a mixed batch: (w, h, format, image) per texture, in batch_specs order. One
    seeded image per distinct (size, format), shared by the textures that have both; the distinct
    images are generated by `workers` processes (0: every core; spawned, so that callers may already
    hold a GPU context)."""
    import os
    specs = batch_specs(count, seed, kmin, kmax)
    keys = sorted({(w, h, fmt) for (w, h, fmt, _s) in specs}, key=lambda k: (-k[0] * k[1], k))
    jobs = [(w, h, fmt, seed ^ (w * 131 + h * 7 + fmt)) for (w, h, fmt) in keys]
    workers = workers or os.cpu_count() or 1
    if workers > 1 and len(jobs) > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(workers, len(jobs))) as pool:
            imgs = pool.map(_batch_image, jobs, chunksize=1)
    else:
        imgs = [_batch_image(j) for j in jobs]
    by_key = dict(zip(keys, imgs))
    return [(w, h, fmt, by_key[(w, h, fmt)]) for (w, h, fmt, _s) in specs]


def random_blocks(n: int, seed: int, kind: str = "mixed") -> np.ndarray:
    """n random 4x4 BGRA8 blocks (n, 16, 4) covering smooth, noisy, few-colour and flat cases."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 16, 4), np.uint8)
    for i in range(n):
        k = i % 6 if kind == "mixed" else 0
        if k == 0:
            out[i] = rng.integers(0, 256, (16, 4))
        elif k == 1:
            base = rng.integers(0, 256, 4)
            out[i] = np.clip(base + rng.integers(-6, 7, (16, 4)), 0, 255)
        elif k == 2:
            pal = rng.integers(0, 256, (3, 4))
            out[i] = pal[rng.integers(0, 3, 16)]
        elif k == 3:
            out[i] = rng.integers(0, 256, 4)[None, :]
        elif k == 5:
            # few RGB colours, alpha varying per texel (duplicate colours with unequal weights)
            pal = rng.integers(0, 256, (2 + i % 3, 3))
            out[i, :, :3] = pal[rng.integers(0, len(pal), 16)]
            out[i, :, 3] = rng.integers(0, 256, 16)
        else:
            t = np.linspace(0, 1, 16)[:, None]
            a, b = rng.integers(0, 256, 4), rng.integers(0, 256, 4)
            out[i] = np.clip(np.rint(a + (b - a) * t) + rng.integers(-2, 3, (16, 4)), 0, 255)
    return out
