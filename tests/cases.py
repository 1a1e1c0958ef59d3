"""Seeded encoder test cases shared by the CPU and GPU parity tests."""
from __future__ import annotations

import numpy as np

FORMATS = (0x83F0, 0x83F1, 0x83F2, 0x83F3)
NRANDOM = (-1, 0, 1, 2, 7, 16)


# 8-bit colours whose 5:6:5 truncations are magenta-like and green-like
# extremes; the SRGB metric's int32 arithmetic wraps between such colours and
# gives negative distances (e.g. (31,0,31) vs (5,60,3)).
SRGB_WRAP_COLOURS = np.array([[248, 0, 248], [40, 240, 24], [248, 44, 248], [8, 244, 8], [16, 240, 0],
                              [248, 76, 248], [0, 252, 0], [248, 16, 240]], np.uint8)


def image(rng: np.random.Generator, w: int, h: int, sc: int, kind: int | None = None) -> np.ndarray:
    """Small test image with one of several value distributions (uniform,
    extremes, coarse levels, flat, alpha-heavy, SRGB wrap-around colours)."""
    kind = int(rng.integers(0, 6)) if kind is None else kind
    if kind == 5:
        img = np.empty((w * h, sc), np.uint8)
        img[:, :3] = SRGB_WRAP_COLOURS[rng.integers(0, len(SRGB_WRAP_COLOURS), w * h)]
        if sc == 4:
            img[:, 3] = rng.choice(np.array([255, 255, 0, 128], np.uint8), w * h)
        return img.reshape(-1)
    n = w * h * sc
    if kind == 0:
        return rng.integers(0, 256, n, dtype=np.uint8)
    if kind == 1:
        return rng.choice(np.array([0, 1, 2, 127, 128, 253, 254, 255], np.uint8), n)
    if kind == 2:
        return (rng.integers(0, 4, n) * 85).astype(np.uint8)
    if kind == 3:
        return np.full(n, int(rng.integers(0, 256)), np.uint8)
    img = rng.integers(0, 256, (w * h, sc), dtype=np.uint8)
    if sc == 4:
        img[:, 3] = rng.choice(np.array([0, 0, 255, 255, 128, 7], np.uint8), w * h)
    return img.reshape(-1)


def random_cases(seed: int, count: int, max_size: int = 17):
    """(w, h, sc, fmt, dither, metric, nrandom, refine, img, seed) tuples."""
    rng = np.random.default_rng(seed)
    for i in range(count):
        w = int(rng.integers(1, max_size + 1))
        h = int(rng.integers(1, max_size + 1))
        sc = int(rng.choice([3, 4]))
        fmt = int(rng.choice(FORMATS))
        yield (w, h, sc, fmt, int(rng.integers(0, 3)), int(rng.integers(0, 8)), int(rng.choice(NRANDOM)),
               int(rng.integers(0, 3)), image(rng, w, h, sc), seed * 100000 + i + 1)


def is_unpinned_corner(w: int, h: int, fmt: int, metric: int, nrandom: int) -> bool:
    """A 1x1 DXT5 image in the all-texels mode without random candidates: the
    reference reads an uninitialised stack slot for its second alpha
    candidate, so its output is not determined by its inputs."""
    return w == 1 and h == 1 and fmt == 0x83F3 and nrandom <= 0 and (nrandom >= 0 or metric == 7)
