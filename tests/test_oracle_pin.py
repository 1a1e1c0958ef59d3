"""Pin the oracle (the C restatement) against the reference encoder compiled
from its own sources.  Runs only where those sources were available."""
import struct
from pathlib import Path

import numpy as np
import pytest

import cases
import pyoracle


def _both(oracle, reference, w, h, sc, fmt, dither, metric, nr, refine, img, seed, stride=0):
    a = reference.compress(sc, w, h, img, fmt, dither, metric, nr, refine, dst_row_stride=stride, seed=seed)
    b = oracle.compress(sc, w, h, img, fmt, dither, metric, nr, refine, dst_row_stride=stride, seed=seed)
    return a, b


def test_random_sweep(oracle, reference):
    bad = []
    for c in cases.random_cases(11, 3000):
        w, h, sc, fmt, dither, metric, nr, refine, img, seed = c
        if cases.is_unpinned_corner(w, h, fmt, metric, nr):
            continue
        a, b = _both(oracle, reference, *c)
        if not np.array_equal(a, b):
            bad.append((w, h, sc, hex(fmt), dither, metric, nr, refine))
    assert not bad, bad[:10]


@pytest.mark.parametrize("fmt", cases.FORMATS)
def test_every_small_size(oracle, reference, fmt):
    """Every (w, h) in [1, 9]^2, cycling through the modes."""
    rng = np.random.default_rng(fmt)
    k = 0
    for w in range(1, 10):
        for h in range(1, 10):
            for _ in range(3):
                sc = 3 + (k & 1)
                metric, refine, dither = k % 8, (k // 8) % 3, (k // 24) % 3
                nr = cases.NRANDOM[k % len(cases.NRANDOM)]
                k += 1
                if cases.is_unpinned_corner(w, h, fmt, metric, nr):
                    continue
                img = cases.image(rng, w, h, sc)
                a, b = _both(oracle, reference, w, h, sc, fmt, dither, metric, nr, refine, img, k)
                assert np.array_equal(a, b), (w, h, sc, metric, nr, refine, dither)


@pytest.mark.parametrize("dither", [0, 1, 2])
def test_rgb565_image(oracle, reference, dither):
    rng = np.random.default_rng(dither)
    for _ in range(60):
        w, h = int(rng.integers(1, 70)), int(rng.integers(1, 70))
        sc, ab = int(rng.choice([3, 4])), int(rng.choice([1, 4, 8]))
        img = cases.image(rng, w, h, sc)
        assert np.array_equal(reference.rgb565_image(img, w, h, sc, ab, dither),
                              oracle.rgb565_image(img, w, h, sc, ab, dither)), (w, h, sc, ab)


def test_row_stride(oracle, reference):
    """dstRowStride: padded rows, packed fallback and overlapping rows."""
    rng = np.random.default_rng(5)
    for fmt in cases.FORMATS:
        bs = 8 if fmt < 0x83F2 else 16
        for w, h in ((5, 6), (8, 8), (13, 3)):
            img = cases.image(rng, w, h, 4, 0)
            row = ((w + 3) // 4) * bs
            for stride in (0, row, row + 12, w * (bs // 4), row - 4):
                size = row * ((h + 3) // 4) + max(0, stride - row) * ((h + 3) // 4) + 64
                da = np.full(size, 0xAB, np.uint8)
                db = np.full(size, 0xAB, np.uint8)
                reference.compress(4, w, h, img, fmt, 1, 5, -1, 1, dst_row_stride=stride, dest=da)
                oracle.compress(4, w, h, img, fmt, 1, 5, -1, 1, dst_row_stride=stride, dest=db)
                assert np.array_equal(da, db), (fmt, w, h, stride)


def test_corner_leftover_rule(oracle, reference):
    """A single-texel DXT5 block reads the alpha endpoint the previous block of
    the same call left behind; the oracle restates that for the reference's
    own build."""
    rng = np.random.default_rng(9)
    for _ in range(200):
        w, h = int(rng.choice([1, 5, 9, 13])), int(rng.choice([1, 5, 9]))
        if w * h == 1:
            continue
        img = cases.image(rng, w, h, 4)
        metric, refine = int(rng.integers(0, 8)), int(rng.integers(0, 3))
        nr = 0 if metric != 7 else int(rng.choice([0, -1]))
        a, b = _both(oracle, reference, w, h, 4, 0x83F3, int(rng.integers(0, 3)), metric, nr, refine, img, 1)
        assert np.array_equal(a, b), (w, h, metric, refine, nr)


def test_srgb_wraparound(oracle, reference):
    """Images of colours whose SRGB distances wrap negative: exercises the
    reference's `bestsum < 0` rule and its wrap-around arithmetic."""
    rng = np.random.default_rng(17)
    for it in range(300):
        w, h = int(rng.integers(1, 13)), int(rng.integers(1, 13))
        fmt = int(rng.choice(cases.FORMATS))
        nr = int(rng.choice([-1, 0, 3, 40]))
        metric = int(rng.choice([2, 2, 3]))
        if cases.is_unpinned_corner(w, h, fmt, metric, nr):
            continue
        img = cases.image(rng, w, h, 4, 5)
        a, b = _both(oracle, reference, w, h, 4, fmt, 0, metric, nr, int(rng.integers(0, 3)), img, it + 1)
        assert np.array_equal(a, b), (w, h, hex(fmt), metric, nr)


def test_wrapv_twin_agrees(reference):
    """The reference built with -fwrapv gives the same bytes, so gcc does not
    exploit the SRGB metric's signed overflow: the encoder's arithmetic is
    plain 32-bit wrap-around.  (The two builds differ only on the
    uninitialised slot read by a single-texel DXT5 block after a NEVER-mode
    block, which is excluded.)"""
    if not pyoracle.REF_WRAPV_SO.exists():
        pytest.skip("no -fwrapv build")
    twin = pyoracle.Reference(pyoracle.REF_WRAPV_SO)
    rng = np.random.default_rng(13)
    for _ in range(400):
        w, h = int(rng.integers(1, 16)), int(rng.integers(1, 16))
        fmt = int(rng.choice(cases.FORMATS))
        nr = int(rng.choice(cases.NRANDOM))
        metric = int(rng.choice([2, 2, 3, 0, 7]))
        refine = int(rng.integers(0, 3))
        if fmt == 0x83F3 and w % 4 == 1 and h % 4 == 1 and (nr == 0 or (nr < 0 and metric == 7)):
            continue
        img = cases.image(rng, w, h, 4, 0)
        a = reference.compress(4, w, h, img, fmt, 1, metric, nr, refine, seed=3)
        b = twin.compress(4, w, h, img, fmt, 1, metric, nr, refine, seed=3)
        assert np.array_equal(a, b), (w, h, hex(fmt), metric, nr, refine)


def _load_tga(path: Path) -> np.ndarray:
    """Uncompressed (type 2) or RLE (type 10) true-colour TGA -> (h, w, 4) RGBA,
    top row first."""
    d = path.read_bytes()
    idlen, cmap, itype = d[0], d[1], d[2]
    w, h, bpp, desc = struct.unpack("<HHBB", d[12:18])
    assert cmap == 0 and itype in (2, 10) and bpp in (24, 32)
    n = bpp // 8
    p = 18 + idlen
    px = np.empty((w * h, n), np.uint8)
    if itype == 2:
        px[:] = np.frombuffer(d, np.uint8, w * h * n, p).reshape(-1, n)
    else:
        i = 0
        while i < w * h:
            hdr = d[p]
            p += 1
            cnt = (hdr & 0x7F) + 1
            if hdr & 0x80:
                px[i:i + cnt] = np.frombuffer(d, np.uint8, n, p)
                p += n
            else:
                px[i:i + cnt] = np.frombuffer(d, np.uint8, cnt * n, p).reshape(-1, n)
                p += cnt * n
            i += cnt
    img = np.full((w * h, 4), 255, np.uint8)
    img[:, 0], img[:, 1], img[:, 2] = px[:, 2], px[:, 1], px[:, 0]
    if n == 4:
        img[:, 3] = px[:, 3]
    img = img.reshape(h, w, 4)
    if not desc & 0x20:
        img = img[::-1]
    return np.ascontiguousarray(img)


def test_reference_fixture_images(oracle, reference):
    """The reference's own test images (tests/*.tga), cropped, in the three
    configurations its visual test script runs."""
    from s2tc_gb300 import build
    ref = build.reference_dir()
    files = sorted((ref / "tests").glob("*.tga")) if ref is not None else []
    if not files:
        pytest.skip("reference test images not present")
    for f in files:
        img = _load_tga(f)[:64, :96]
        h, w = img.shape[:2]
        for fmt in (0x83F1, 0x83F3):
            for dither, metric, nr, refine in ((2, 3, 32, 2), (1, 5, -1, 1), (1, 5, -1, 2), (2, 7, 32, 2)):
                a, b = _both(oracle, reference, w, h, 4, fmt, dither, metric, nr, refine, img.reshape(-1), 77)
                assert np.array_equal(a, b), (f.name, hex(fmt), dither, metric, nr, refine)
