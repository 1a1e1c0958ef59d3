"""GPU versions of the reference's command-line tools against the oracle:
s2tc_compress (mip chain + DDS), s2tc_decompress (whole-image decode, TGA) and
s2tc_from_s3tc (block rewrite)."""
import struct

import numpy as np
import pytest

import pyoracle
import s2tc_gb300 as s2
from s2tc_gb300 import workloads

pytestmark = pytest.mark.gpu

FMTS = (0x83F1, 0x83F2, 0x83F3)


def synthetic(seed, w, h, opaque):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    img[:, : w // 2, 0] = (xx[:, : w // 2] * 7 + yy[:, : w // 2] * 3) % 256
    if opaque:
        img[:, :, 3] = 255
    return img


MODES = [(1, 5, -1, 1), (1, 5, -1, 2), (2, 3, 32, 2), (0, 7, 8, 0), (1, 2, 0, 2), (2, 1, -1, 1), (1, 3, 0, 1)]


@pytest.mark.parametrize("fmt", FMTS)
def test_compress_dds_matches_oracle(lib, oracle, fmt):
    sizes = [(2, 1), (1, 9), (5, 3), (16, 16), (37, 23), (64, 4), (3, 70), (100, 60)]
    for k, (w, h) in enumerate(sizes):
        for opaque in (False, True):
            img = synthetic(100 + k, w, h, opaque)
            for dither, metric, nr, refine in MODES:
                opt = s2.options(dither, metric, nr, refine)
                pyoracle.srand(1)
                got = s2.compress_dds(img, w, h, fmt, opt)
                want = oracle.dds(img, w, h, fmt, dither, metric, nr, refine, seed=1)
                assert got == want, (w, h, hex(fmt), opaque, dither, metric, nr, refine)
    assert s2.dds_size(37, 23, fmt) == oracle.dds_size(37, 23, fmt)


def test_compress_dds_large(lib, oracle):
    w, h = 1024, 768
    img = workloads.value_noise_rgba(9, w, h)
    for fmt, mode in ((0x83F1, (1, 5, -1, 1)), (0x83F3, (1, 3, 0, 2))):
        opt = s2.options(*mode)
        got = s2.compress_dds(img, w, h, fmt, opt)
        want = oracle.dds(img, w, h, fmt, *mode, seed=1)
        assert got == want, (hex(fmt), mode)


def test_compress_dds_reads_env(lib, oracle):
    img = synthetic(5, 40, 24, False)
    s2.set_env(2, 3, -1, 2)
    assert s2.compress_dds(img, 40, 24, 0x83F3) == oracle.dds(img, 40, 24, 0x83F3, 2, 3, -1, 2)


def _random_blocks(seed, w, h, fmt):
    rng = np.random.default_rng(seed)
    bs = 8 if fmt in (0x83F0, 0x83F1) else 16
    return rng.integers(0, 256, ((w + 3) // 4) * ((h + 3) // 4) * bs, dtype=np.uint8)


@pytest.mark.parametrize("fmt", (0x83F0, 0x83F1, 0x83F2, 0x83F3))
def test_gpu_decode_matches_fetch(lib, oracle, fmt):
    torch = pytest.importorskip("torch")
    dxt = 0 if fmt in (0x83F0, 0x83F1) else 1 if fmt == 0x83F2 else 2
    for k, (w, h) in enumerate([(1, 1), (3, 5), (8, 8), (29, 14), (64, 33)]):
        blocks = _random_blocks(20 + k, w, h, fmt)
        want = np.zeros((h, w, 4), np.uint8)
        for j in range(h):
            for i in range(w):
                want[j, i] = oracle.fetch(dxt, int(fmt != 0x83F0), w, blocks, i, j)
        d_blk = torch.from_numpy(blocks).cuda()
        for pitch, bgra in ((0, False), (w * 4 + 12, True)):
            p = pitch or w * 4
            d_out = torch.zeros(p * h, dtype=torch.uint8, device="cuda")
            s2.gpu_decode(d_blk, fmt, w, h, d_out, pitch, bgra)
            s2.gpu_synchronize(None)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy().reshape(h, p)[:, : w * 4].reshape(h, w, 4)
            exp = want[:, :, [2, 1, 0, 3]] if bgra else want
            assert np.array_equal(got, exp), (hex(fmt), w, h, pitch, bgra)


def test_round_trip_decode(lib, oracle):
    """Encode with tx_compress_dxtn, decode on the GPU: every texel equals the
    reference decoder's."""
    torch = pytest.importorskip("torch")
    w, h = 512, 384
    img = workloads.plain_rgba(3, w, h).reshape(-1)
    for fmt in FMTS:
        s2.set_env(1, 5, -1, 1)
        blocks = s2.tx_compress_dxtn(4, w, h, img, fmt)
        d_out = torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda")
        s2.gpu_decode(torch.from_numpy(blocks).cuda(), fmt, w, h, d_out)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().reshape(h, w, 4)
        dxt = FMTS.index(fmt)
        for j in list(range(0, h, 37)) + [h - 1]:
            row = np.stack([oracle.fetch(dxt, 1, w, blocks, i, j) for i in range(w)])
            assert np.array_equal(got[j], row), (hex(fmt), j)


def test_decompress_dds_matches_oracle(lib, oracle):
    for fmt in FMTS:
        for k, (w, h) in enumerate([(1, 1), (7, 5), (37, 23), (128, 64)]):
            img = synthetic(300 + k, w, h, False)
            dds = s2.compress_dds(img, w, h, fmt, s2.options(1, 5, -1, 1))
            assert s2.decompress_dds(dds) == oracle.decompress(dds), (hex(fmt), w, h)
    rng = np.random.default_rng(7)
    for fourcc, bs in (("DXT1", 8), ("DXT3", 16), ("DXT5", 16)):
        w, h = 29, 14
        hdr = bytearray(128)
        hdr[0:4] = b"DDS "
        struct.pack_into("<II", hdr, 12, h, w)
        hdr[84:88] = fourcc.encode()
        dds = bytes(hdr) + rng.integers(0, 256, ((w + 3) // 4) * ((h + 3) // 4) * bs, dtype=np.uint8).tobytes()
        assert s2.decompress_dds(dds) == oracle.decompress(dds), fourcc
    bad = bytearray(dds)
    bad[84:88] = b"ATI2"
    with pytest.raises(s2.S2tcError):
        s2.decompress_dds(bytes(bad))


def test_from_s3tc_matches_oracle(lib, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    for fmt, dxt, bs in ((0x83F1, 0, 8), (0x83F2, 1, 16), (0x83F3, 2, 16)):
        n = 5000
        blocks = rng.integers(0, 256, n * bs, dtype=np.uint8)
        want = oracle.from_s3tc_blocks(blocks, dxt)
        d_src = torch.from_numpy(blocks).cuda()
        d_dst = torch.zeros_like(d_src)
        s2.gpu_from_s3tc(d_src, d_dst, n, fmt)
        torch.cuda.synchronize()
        assert np.array_equal(d_dst.cpu().numpy(), want), hex(fmt)
        s2.gpu_from_s3tc(d_src, d_src, n, fmt)  # in place
        torch.cuda.synchronize()
        assert np.array_equal(d_src.cpu().numpy(), want), hex(fmt)
        for tail in (0, 5):
            hdr = bytearray(128)
            hdr[0:4] = b"DDS "
            hdr[84:88] = ("DXT1", "DXT3", "DXT5")[dxt].encode()
            f = bytes(hdr) + rng.integers(0, 256, 333 * bs + tail, dtype=np.uint8).tobytes()
            assert s2.from_s3tc_dds(f) == oracle.from_s3tc(f), (hex(fmt), tail)
