"""s2tc_gpu_compress_noalloc: the entry point for callers that cannot call
cudaMalloc (its scratch lives in a fixed device array of the library).  Its
bytes must equal s2tc_gpu_compress's on two calls in a row, where the second
call finds the first call's leftovers in the shared array.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import numpy as np
import pytest

import s2tc_gb300 as s2
from s2tc_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_noalloc_matches_gpu_compress_twice(lib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    calls = [
        # 2048x2048 RGBA -> DXT5, SRGB_MIXED all-16 search, LOOP, SIMPLE dither (the size limit)
        (workloads.value_noise_rgba(11, 2048, 2048), 2048, 2048, 0x83F3, s2.options(1, s2.SRGB_MIXED, 0, 2)),
        # 1000x613 RGBA -> DXT1, WAVG quick selection, ALWAYS, Floyd-Steinberg
        (workloads.plain_rgba(12, 1000, 613), 1000, 613, 0x83F1, s2.options(2, s2.WAVG, -1, 1)),
        # 2048x2048 RGBA -> DXT1, Floyd-Steinberg with its alpha pass (the size limit)
        (workloads.plain_rgba(13, 2048, 2048), 2048, 2048, 0x83F1, s2.options(2, s2.WAVG, -1, 1)),
    ]
    for img, w, h, fmt, opt in calls:
        d_src = torch.from_numpy(img.reshape(-1).copy()).cuda()
        n = s2.compressed_size(w, h, fmt)
        d_want = torch.zeros(n, dtype=torch.uint8, device="cuda")
        d_got = torch.full((n,), 0x5A, dtype=torch.uint8, device="cuda")
        s2.gpu_compress(4, w, h, d_src, fmt, d_want, opt=opt, stream=stream.cuda_stream)
        s2.gpu_synchronize(stream.cuda_stream)
        st = s2.gpu_compress_noalloc(4, w, h, d_src, fmt, d_got, opt=opt, stream=stream.cuda_stream)
        assert st == 0, s2.last_error()
        assert np.array_equal(d_got.cpu().numpy(), d_want.cpu().numpy())


def test_noalloc_rejects_oversize(lib):
    torch = pytest.importorskip("torch")
    d_src = torch.zeros(16, dtype=torch.uint8, device="cuda")
    d_dst = torch.zeros(16, dtype=torch.uint8, device="cuda")
    # 4097 x 1024 texels is above the 4 Mi limit: rejected before any device work
    assert s2.gpu_compress_noalloc(4, 4097, 1024, d_src, 0x83F1, d_dst, opt=s2.options()) == 6


def test_noalloc_rejects_wide_floyd_steinberg(lib):
    """65536x64 is under the 4 Mi texel limit, but its Floyd-Steinberg carry
    rows do not fit the fixed scan region: rejected before any device work.
    The same image with SIMPLE dither is not rejected for that reason."""
    torch = pytest.importorskip("torch")
    d_src = torch.zeros(16, dtype=torch.uint8, device="cuda")
    d_dst = torch.zeros(16, dtype=torch.uint8, device="cuda")
    assert s2.gpu_compress_noalloc(4, 65536, 64, d_src, 0x83F1, d_dst, opt=s2.options(2, s2.WAVG, -1, 1)) == 6


def test_noalloc_random_candidates_and_rgb_twice(lib):
    """RANDOM_COLORS > 0 with the caller's replayed words (d_rand), and an
    RGB8 (3-component) source, each on two calls in a row, against
    s2tc_gpu_compress given the same words; and no device memory is taken
    by a call on a warm context."""
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    cases = [
        (workloads.plain_rgba(14, 300, 200).reshape(-1), 4, 300, 200, 0x83F3, s2.options(1, s2.WAVG, 16, 1)),
        (workloads.normal_map(15, 256, 256).reshape(-1), 3, 256, 256, 0x83F1, s2.options(1, s2.NORMALMAP, 8, 2)),
        (workloads.normal_map(16, 1000, 700).reshape(-1), 3, 1000, 700, 0x83F1, s2.options(1, s2.SRGB_MIXED, 0, 1)),
    ]
    for img, sc, w, h, fmt, opt in cases:
        words = s2.rand_words(w, h, fmt, opt)
        d_rand = torch.randint(0, 2**31 - 1, (max(1, words),), dtype=torch.int32, device="cuda") if words else None
        d_src = torch.from_numpy(img.copy()).cuda()
        n = s2.compressed_size(w, h, fmt)
        d_want = torch.zeros(n, dtype=torch.uint8, device="cuda")
        s2.gpu_compress(sc, w, h, d_src, fmt, d_want, opt=opt, d_rand=d_rand, stream=stream.cuda_stream)
        s2.gpu_synchronize(stream.cuda_stream)
        for call in range(2):
            d_got = torch.full((n,), 0x5A, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            st = s2.gpu_compress_noalloc(sc, w, h, d_src, fmt, d_got, opt=opt, d_rand=d_rand,
                                         stream=stream.cuda_stream)
            free_after = torch.cuda.mem_get_info()[0]
            assert st == 0, s2.last_error()
            assert np.array_equal(d_got.cpu().numpy(), d_want.cpu().numpy()), (sc, w, h, call)
            if call == 1:  # the first call may load kernels it had not run yet
                assert free_after >= free_before, (free_before, free_after)
