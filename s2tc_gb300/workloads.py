"""Seeded synthetic inputs with the shapes and value distributions of the
encoder's benchmark workloads (numpy only; used by bench.py and the tests).

* ``plain_rgba``      -- 1024x1024 RGBA8: left half iid noise, right half an RGB
                          gradient with +-8 jitter, alpha 255.
* ``value_noise_rgba``-- 4096x4096 RGBA8: 4-octave value noise per channel,
                          hard-edged alpha mask with 10% noisy texels.
* ``mip_textures``    -- 256 textures, log-uniform sizes 4..2048 (aspect <= 4:1),
                          full box-filtered mip chains (the reduction of the
                          reference tool's Image_MipReduce32,
                          s2tc_compress.c:427-493), formats and component
                          counts cycling.
* ``normal_map``      -- tangent-space normal maps from a 3-octave value-noise
                          heightfield (RGB8).
* ``serving_requests``-- request sizes/formats/metrics for the serving loop.
"""
from __future__ import annotations

import numpy as np

DXT1_RGBA, DXT3, DXT5 = 0x83F1, 0x83F2, 0x83F3


def _value_noise(rng: np.random.Generator, w: int, h: int, period: int) -> np.ndarray:
    """Bilinear value noise on a random u8 lattice with the given period."""
    gw, gh = w // period + 2, h // period + 2
    lat = rng.integers(0, 256, (gh, gw)).astype(np.float32)
    x = np.arange(w)
    ix, fx = x // period, (x % period).astype(np.float32) / period
    rows = lat[:, ix] * (1 - fx) + lat[:, ix + 1] * fx          # (gh, w)
    y = np.arange(h)
    iy, fy = y // period, ((y % period).astype(np.float32) / period)[:, None]
    return rows[iy] * (1 - fy) + rows[iy + 1] * fy             # (h, w)


def plain_rgba(seed: int = 1, w: int = 1024, h: int = 1024) -> np.ndarray:
    """Left half iid uniform noise; right half a linear RGB gradient plus
    uniform jitter in [-8, 8]; alpha 255.  Returns (h, w, 4) uint8."""
    rng = np.random.default_rng(seed)
    img = np.empty((h, w, 4), np.uint8)
    half = w // 2
    img[:, :half, :3] = rng.integers(0, 256, (h, half, 3), dtype=np.uint8)
    xs = np.arange(half, w)[None, :].astype(np.float64)
    ys = np.arange(h)[:, None].astype(np.float64)
    grad = np.stack(np.broadcast_arrays(xs * 255 / max(1, w - 1), ys * 255 / max(1, h - 1),
                                        (xs + ys) * 255 / max(1, w + h - 2)), axis=-1)
    jit = rng.integers(-8, 9, grad.shape)
    img[:, half:, :3] = np.clip(np.rint(grad) + jit, 0, 255).astype(np.uint8)
    img[:, :, 3] = 255
    return img


def value_noise_rgba(seed: int = 2, w: int = 4096, h: int = 4096) -> np.ndarray:
    """RGB: 4-octave value noise (periods 256/64/16/4, weights .5/.25/.15/.1).
    Alpha: 255 where the first octave of the red noise exceeds 128, else 0,
    then 10% of texels set to uniform u8.  Returns (h, w, 4) uint8."""
    rng = np.random.default_rng(seed)
    img = np.empty((h, w, 4), np.uint8)
    first = None
    for c in range(3):
        acc = np.zeros((h, w), np.float32)
        for period, wt in ((256, 0.5), (64, 0.25), (16, 0.15), (4, 0.1)):
            n = _value_noise(rng, w, h, period)
            if c == 0 and period == 256:
                first = n
            acc += wt * n
        img[:, :, c] = np.clip(np.rint(acc), 0, 255).astype(np.uint8)
    alpha = np.where(first > 128, 255, 0).astype(np.uint8)
    mask = rng.random((h, w)) < 0.10
    alpha[mask] = rng.integers(0, 256, int(mask.sum()), dtype=np.uint8)
    img[:, :, 3] = alpha
    return img


def mip_reduce(img: np.ndarray) -> np.ndarray:
    """One level of the reference tool's mip reduction: 2x2 (or 2x1 / 1x2 when
    one side is already 1) box average with truncating shifts; an odd last
    row/column is dropped (s2tc_compress.c:427-493)."""
    h, w = img.shape[:2]
    a = img.astype(np.uint16)
    if w > 1 and h > 1:
        a = a[: (h // 2) * 2, : (w // 2) * 2]
        s = a[0::2, 0::2] + a[0::2, 1::2] + a[1::2, 0::2] + a[1::2, 1::2]
        return (s >> 2).astype(np.uint8)
    if w > 1:
        a = a[:, : (w // 2) * 2]
        return ((a[:, 0::2] + a[:, 1::2]) >> 1).astype(np.uint8)
    if h > 1:
        a = a[: (h // 2) * 2]
        return ((a[0::2] + a[1::2]) >> 1).astype(np.uint8)
    return img.copy()


def mip_chain(img: np.ndarray) -> list[np.ndarray]:
    """Levels from the base down to 1x1 (s2tc_compress.c:722-733)."""
    levels = [img]
    while levels[-1].shape[0] > 1 or levels[-1].shape[1] > 1:
        levels.append(mip_reduce(levels[-1]))
    return levels


def mip_textures(seed: int = 3, count: int = 256, lo: int = 4, hi: int = 2048):
    """Uneven mip-chain batch: list of dicts with keys ``levels`` (list of
    (h, w, srccomps) uint8 arrays), ``fmt`` and ``srccomps``.  Base sizes are
    log-uniform in [lo, hi] with aspect at most 4:1; formats cycle DXT1 /
    DXT3 / DXT5 by thirds; RGB8 and RGBA8 inputs alternate."""
    rng = np.random.default_rng(seed)
    fmts = (DXT1_RGBA, DXT3, DXT5)
    out = []
    for i in range(count):
        while True:
            w = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
            h = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
            if max(w, h) <= 4 * min(w, h):
                break
        comps = 3 if i % 2 == 0 else 4
        base = np.empty((h, w, 4), np.uint8)
        base[:, :, :3] = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        base[:, :, 3] = rng.integers(0, 256, (h, w), dtype=np.uint8)
        levels = [lvl[:, :, :comps].copy() for lvl in mip_chain(base)]
        out.append({"levels": levels, "fmt": fmts[(i * 3) // count], "srccomps": comps})
    return out


def normal_map(seed: int = 4, w: int = 2048, h: int = 2048) -> np.ndarray:
    """Tangent-space normal map: 3-octave value-noise heightfield scaled 0..4,
    central-difference gradient, normalised, n*127.5+127.5 rounded.
    Returns (h, w, 3) uint8."""
    rng = np.random.default_rng(seed)
    hf = np.zeros((h, w), np.float32)
    for period, wt in ((128, 0.6), (32, 0.3), (8, 0.1)):
        hf += wt * _value_noise(rng, w, h, period)
    hf *= 4.0 / 255.0
    gx = (np.roll(hf, -1, axis=1) - np.roll(hf, 1, axis=1)) * 0.5
    gy = (np.roll(hf, -1, axis=0) - np.roll(hf, 1, axis=0)) * 0.5
    n = np.stack([-gx, -gy, np.ones_like(hf)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.clip(np.rint(n * 127.5 + 127.5), 0, 255).astype(np.uint8)


def serving_requests(seed: int = 5, count: int = 20000, lo: int = 64, hi: int = 4096):
    """Request descriptors (width, height, fmt, metric, pixel seed) for the
    serving workload; pixels follow ``plain_rgba`` with the request's seed."""
    rng = np.random.default_rng(seed)
    metrics = (5, 3, 7)  # WAVG, SRGB_MIXED, NORMALMAP
    reqs = []
    for i in range(count):
        w = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        h = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        reqs.append({"width": w, "height": h, "fmt": DXT1_RGBA if rng.random() < 0.5 else DXT5,
                     "metric": int(metrics[rng.integers(0, 3)]), "seed": int(seed * 1000003 + i)})
    return reqs
