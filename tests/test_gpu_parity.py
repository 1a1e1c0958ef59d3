"""GPU encoder (through the C ABI) against the oracle and the golden vectors:
byte-for-byte, every mode."""
import numpy as np
import pytest

import cases
import pyoracle
import s2tc_gb300 as s2
from golden import golden
from s2tc_gb300 import workloads

pytestmark = pytest.mark.gpu


def gpu_compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed=1, stride=0, dest=None):
    s2.set_env(dither, metric, nr, refine)
    pyoracle.srand(seed)
    return s2.tx_compress_dxtn(sc, w, h, img, fmt, stride, dest)


def test_golden_vectors(lib):
    n = 0
    for c in golden.encode_cases():
        out = gpu_compress(c["sc"], c["w"], c["h"], c["src"], c["fmt"], c["dither"], c["metric"], c["nrandom"],
                           c["refine"], c["seed"], c["stride"])
        assert np.array_equal(out, c["out"]), {k: v for k, v in c.items() if k not in ("src", "out")}
        n += 1
    assert n > 500


def test_golden_dither(lib):
    for c in golden.dither_cases():
        out = s2.rgb565_image(c["src"], c["w"], c["h"], c["sc"], c["alphabits"], c["dither"])
        assert np.array_equal(out, c["out"]), {k: v for k, v in c.items() if k not in ("src", "out")}


def test_random_sweep(lib, oracle):
    for c in cases.random_cases(21, 1500):
        w, h, sc, fmt, dither, metric, nr, refine, img, seed = c
        if cases.is_unpinned_corner(w, h, fmt, metric, nr):
            continue
        a = gpu_compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed)
        b = oracle.compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed=seed)
        assert np.array_equal(a, b), (w, h, sc, hex(fmt), dither, metric, nr, refine)


def test_srgb_wraparound(lib, oracle):
    """SRGB distances that wrap negative: the full-block kernel, the warp
    kernel's sequential fallback and the thread kernel all keep the
    reference's `bestsum < 0` rule."""
    rng = np.random.default_rng(23)
    for it in range(200):
        w, h = int(rng.integers(1, 24)), int(rng.integers(1, 24))
        fmt = int(rng.choice(cases.FORMATS))
        nr = int(rng.choice([-1, 0, 3, 40]))
        metric = int(rng.choice([2, 2, 3]))
        refine = int(rng.integers(0, 3))
        img = cases.image(rng, w, h, 4, 5)
        if cases.is_unpinned_corner(w, h, fmt, metric, nr):
            continue
        a = gpu_compress(4, w, h, img, fmt, 0, metric, nr, refine, it + 1)
        b = oracle.compress(4, w, h, img, fmt, 0, metric, nr, refine, seed=it + 1)
        assert np.array_equal(a, b), (w, h, hex(fmt), metric, nr, refine)


def _pair_sums(oracle, metric, t565, bx, by, iw):
    """The reference's 120 pair sums of one whole block's 16 inputs
    (s2tc_algorithm.cpp:363-414), from the oracle's distance."""
    px = t565.reshape(-1, 4)
    ins = [tuple(int(v) for v in px[(by * 4 + y) * iw + bx * 4 + x][:3]) for x in range(4) for y in range(4)]
    d = [[0 if i == k else oracle.color_dist(metric, ins[min(i, k)], ins[max(i, k)]) for k in range(16)]
         for i in range(16)]
    return [sum(min(d[i][k], d[j][k]) for k in range(16)) for i in range(16) for j in range(i + 1, 16)]


def test_srgb_negative_pair_sums_whole_blocks(lib, oracle):
    """Whole 4x4 blocks of the SRGB wrap-around colours, all-texels search:
    pair sums go negative, where the reference keeps the last pair
    (`bestsum < 0` takes every later pair), against blocks of non-negative
    sums, where it keeps the first smallest."""
    rng = np.random.default_rng(31)
    w, h = 64, 32
    rgb = cases.SRGB_WRAP_COLOURS[rng.integers(0, len(cases.SRGB_WRAP_COLOURS), (h, w))]
    # every other block row: two colours only, half and half, so more sums are negative
    two = cases.SRGB_WRAP_COLOURS[[0, 6]][rng.integers(0, 2, (h, w))]
    rows = (np.arange(h) // 4) % 2 == 1
    rgb[rows] = two[rows]
    img = np.concatenate([rgb, np.full((h, w, 1), 255, np.uint8)], axis=2).reshape(-1)
    t565 = oracle.rgb565_image(img, w, h, 4, 8, 0)
    neg = sum(min(_pair_sums(oracle, 2, t565, bx, by, w)) < 0 for by in range(2) for bx in range(0, 16, 3))
    assert 0 < neg < 12, neg  # both kinds of block occur
    for fmt in (0x83F0, 0x83F1, 0x83F2, 0x83F3):
        for refine in range(3):
            a = gpu_compress(4, w, h, img, fmt, 0, 2, 0, refine, 5)
            b = oracle.compress(4, w, h, img, fmt, 0, 2, 0, refine, seed=5)
            assert np.array_equal(a, b), (hex(fmt), refine)


@pytest.mark.parametrize("nr", [64, 300, 700])
def test_many_random_candidates(lib, oracle, nr):
    """Random-candidate counts served by the warp kernel (shared-memory
    candidate lists) and, past its shared-memory limit, by the thread kernel."""
    rng = np.random.default_rng(nr)
    for fmt in (0x83F1, 0x83F2, 0x83F3):
        for metric in (5, 3, 7, 2):
            w, h = int(rng.integers(5, 20)), int(rng.integers(5, 20))
            img = cases.image(rng, w, h, 4)
            refine = int(rng.integers(0, 3))
            a = gpu_compress(4, w, h, img, fmt, 1, metric, nr, refine, 7)
            b = oracle.compress(4, w, h, img, fmt, 1, metric, nr, refine, seed=7)
            assert np.array_equal(a, b), (hex(fmt), metric, refine)


@pytest.mark.parametrize("fmt", cases.FORMATS)
def test_every_small_size(lib, oracle, fmt):
    rng = np.random.default_rng(fmt + 1)
    k = 0
    for w in range(1, 10):
        for h in range(1, 10):
            for _ in range(2):
                sc = 3 + (k & 1)
                metric, refine, dither = k % 8, (k // 8) % 3, (k // 24) % 3
                nr = cases.NRANDOM[k % len(cases.NRANDOM)]
                k += 1
                img = cases.image(rng, w, h, sc)
                if cases.is_unpinned_corner(w, h, fmt, metric, nr):
                    continue
                a = gpu_compress(sc, w, h, img, fmt, dither, metric, nr, refine, k)
                b = oracle.compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed=k)
                assert np.array_equal(a, b), (w, h, sc, metric, nr, refine, dither)


@pytest.mark.parametrize("fmt", [0x83F1, 0x83F2, 0x83F3])
def test_every_mode_combination(lib, oracle, fmt):
    rng = np.random.default_rng(fmt)
    w, h = 37, 29
    for metric in range(8):
        for nr in (-1, 0, 5):
            for refine in range(3):
                for dither in range(3):
                    img = cases.image(rng, w, h, 4, int(rng.integers(0, 5)))
                    a = gpu_compress(4, w, h, img, fmt, dither, metric, nr, refine, 99)
                    b = oracle.compress(4, w, h, img, fmt, dither, metric, nr, refine, seed=99)
                    assert np.array_equal(a, b), (metric, nr, refine, dither)


@pytest.mark.parametrize("dither", [0, 1, 2])
def test_rgb565_image_many_tiles(lib, oracle, dither):
    """Images that span many scan tiles and Floyd-Steinberg strips and clusters."""
    rng = np.random.default_rng(40 + dither)
    for w, h in ((1000, 613), (3, 2000), (4099, 37), (257, 300)):
        for sc, ab in ((4, 1), (4, 4), (3, 8), (4, 8)):
            img = cases.image(rng, w, h, sc, 0)
            a = s2.rgb565_image(img, w, h, sc, ab, dither)
            b = oracle.rgb565_image(img, w, h, sc, ab, dither)
            assert np.array_equal(a, b), (w, h, sc, ab)


def test_fs_strip_edges(lib, oracle):
    """Floyd-Steinberg heights around the 32-row strips, odd widths (unaligned
    rows), one-row and one-column images, all alpha variants."""
    rng = np.random.default_rng(77)
    for w, h in ((31, 32), (33, 64), (64, 33), (2, 129), (1, 100), (100, 1), (7, 31), (5, 63), (130, 96)):
        for sc, ab in ((4, 1), (4, 4), (4, 8), (3, 1), (3, 4)):
            img = cases.image(rng, w, h, sc, 0)
            a = s2.rgb565_image(img, w, h, sc, ab, 2)
            b = oracle.rgb565_image(img, w, h, sc, ab, 2)
            assert np.array_equal(a, b), (w, h, sc, ab)


def test_fs_unaligned_device_source(lib, oracle):
    """Floyd-Steinberg from device sources 1, 2 and 4 bytes past an aligned
    address (byte loads, byte loads, 4-byte copies) and at the aligned one."""
    import torch
    rng = np.random.default_rng(78)
    for w, h in ((70, 45), (33, 40)):
        img = cases.image(rng, w, h, 4, 0)
        for fmt in (0x83F1, 0x83F3):
            want = oracle.compress(4, w, h, img, fmt, 2, 5, -1, 1)
            for off in (0, 1, 2, 4):
                buf = torch.zeros(off + img.size, dtype=torch.uint8, device="cuda")
                buf[off:] = torch.from_numpy(img).cuda()
                d_dst = torch.zeros(s2.compressed_size(w, h, fmt), dtype=torch.uint8, device="cuda")
                s2.gpu_compress(4, w, h, buf.data_ptr() + off, fmt, d_dst, opt=s2.options(2, 5, -1, 1))
                torch.cuda.synchronize()
                assert np.array_equal(d_dst.cpu().numpy(), want), (w, h, hex(fmt), off)


def test_row_stride(lib, oracle):
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
                gpu_compress(4, w, h, img, fmt, 1, 5, -1, 1, stride=stride, dest=da)
                oracle.compress(4, w, h, img, fmt, 1, 5, -1, 1, dst_row_stride=stride, dest=db)
                assert np.array_equal(da, db), (fmt, w, h, stride)


def test_encode_block_func(lib, oracle):
    """The per-block API: same bytes as the oracle's block encoder, including
    the leftover alpha endpoint carried from call to call."""
    rng = np.random.default_rng(6)
    t565 = np.zeros(8 * 8 * 4, np.uint8)
    for it in range(300):
        t = rng.integers(0, 256, (8 * 8, 4)).astype(np.uint8)
        t[:, 0] &= 31
        t[:, 1] &= 63
        t[:, 2] &= 31
        dxt = int(rng.integers(0, 3))
        if dxt == 0:
            t[:, 3] = rng.integers(0, 2, 64)
        elif dxt == 1:
            t[:, 3] &= 15
        t565[:] = t.reshape(-1)
        metric, refine = int(rng.integers(0, 8)), int(rng.integers(0, 3))
        nr_sel = int(rng.choice([-1, 0, 3]))
        nr_call = int(rng.choice([0, 2])) if nr_sel >= 0 else nr_sel
        w, h = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        fn = s2.encode_block_func(dxt, metric, nr_sel, refine)
        out = np.zeros(16, np.uint8)
        pyoracle.srand(it + 1)
        fn(out, t565, 8, w, h, nr_call)
        # the oracle's per-block entry point with the selection mode of nr_sel
        nr_eff = nr_call if (nr_sel >= 0 or metric == 7) else -1
        if nr_sel >= 0 and nr_call < 0:
            nr_eff = nr_call
        pyoracle.srand(it + 1)
        want, _ = oracle.encode_block(t565, 8, w, h, dxt, metric, nr_eff if nr_sel >= 0 or metric == 7 else -1,
                                      refine, prev_a1=-1)
        bs = 8 if dxt == 0 else 16
        if dxt == 2 and w * h == 1 and (nr_sel >= 0 or metric == 7) and nr_call <= 0:
            continue  # depends on the previous call's leftover
        assert np.array_equal(out[:bs], want), (it, dxt, metric, nr_sel, nr_call, refine, w, h)


def test_device_api_matches_host_api(lib):
    torch = pytest.importorskip("torch")
    img = workloads.plain_rgba(3, 300, 200)
    for fmt in (0x83F1, 0x83F3):
        o = s2.options(1, 3, 0, 2)
        want = gpu_compress(4, 300, 200, img.reshape(-1), fmt, 1, 3, 0, 2)
        d_src = torch.from_numpy(img.reshape(-1).copy()).cuda()
        d_dst = torch.zeros(len(want), dtype=torch.uint8, device="cuda")
        s2.gpu_compress(4, 300, 200, d_src, fmt, d_dst, opt=o)
        s2.gpu_synchronize()
        assert np.array_equal(d_dst.cpu().numpy(), want)
        # on a user stream
        st = torch.cuda.Stream()
        d_dst.zero_()
        s2.gpu_compress(4, 300, 200, d_src, fmt, d_dst, opt=o, stream=st.cuda_stream)
        s2.gpu_synchronize(st.cuda_stream)
        assert np.array_equal(d_dst.cpu().numpy(), want)


def test_plain_1024_quick(lib, oracle):
    """1024x1024 RGBA -> DXT1, WAVG, quick selection, ALWAYS, SIMPLE dither."""
    img = workloads.plain_rgba(1).reshape(-1)
    a = gpu_compress(4, 1024, 1024, img, 0x83F1, 1, 5, -1, 1)
    b = oracle.compress(4, 1024, 1024, img, 0x83F1, 1, 5, -1, 1)
    assert np.array_equal(a, b)


def test_value_noise_4096_exhaustive(lib, oracle):
    """4096x4096 RGBA -> DXT5, SRGB_MIXED, all-16 search, LOOP: full image."""
    img = workloads.value_noise_rgba(2).reshape(-1)
    a = gpu_compress(4, 4096, 4096, img, 0x83F3, 1, 3, 0, 2)
    b = oracle.compress(4, 4096, 4096, img, 0x83F3, 1, 3, 0, 2)
    assert np.array_equal(a, b)


def test_normal_map_random_candidates(lib, oracle):
    """A 512x512 RGB normal map -> DXT1, NORMALMAP, 64 random candidates, LOOP
    (rand() replayed in block order)."""
    img = workloads.normal_map(4, 512, 512).reshape(-1)
    a = gpu_compress(3, 512, 512, img, 0x83F1, 1, 7, 64, 2, seed=1234)
    b = oracle.compress(3, 512, 512, img, 0x83F1, 1, 7, 64, 2, seed=1234)
    assert np.array_equal(a, b)


def test_normal_map_full_2048(lib, oracle):
    """One whole 2048x2048 normal map of the 64-map workload's recipe -> DXT1,
    NORMALMAP, 64 random candidates, LOOP, SIMPLE dither: every block against
    the oracle, with libc's rand() stream consumed over the whole image
    (50 M words, generated on the GPU from the stream's position)."""
    img = workloads.normal_map(4, 2048, 2048).reshape(-1)
    a = gpu_compress(3, 2048, 2048, img, 0x83F1, 1, 7, 64, 2, seed=4321)
    after_gpu = pyoracle.libc_rand()
    b = oracle.compress(3, 2048, 2048, img, 0x83F1, 1, 7, 64, 2, seed=4321)
    assert np.array_equal(a, b)
    assert pyoracle.libc_rand() == after_gpu  # both left the stream at the same place


def test_batch_resident_rand_words_vs_oracle(lib, oracle):
    """The batched graph launch fed caller-resident random-candidate words
    (the form the batched benchmarks time): uneven mip chains with 1x1, 2x2
    and 3xN levels, mixed formats and component counts, against the oracle
    given the same words."""
    torch = pytest.importorskip("torch")
    tex = workloads.mip_textures(41, count=8, lo=3, hi=90)
    opt = s2.options(1, s2.WAVG, 16, 1)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    images, host = [], []
    for t in tex:
        for lvl in t["levels"]:
            h, w = lvl.shape[:2]
            words = s2.rand_words(w, h, t["fmt"], opt)
            rw = torch.randint(0, 2**31 - 1, (max(1, words),), dtype=torch.int32, device="cuda", generator=gen)
            n = s2.compressed_size(w, h, t["fmt"])
            images.append({"src": torch.from_numpy(lvl.reshape(-1).copy()).cuda(), "width": w, "height": h,
                           "srccomps": t["srccomps"], "format": t["fmt"], "rand": rw,
                           "dst": torch.full((n,), 0xA5, dtype=torch.uint8, device="cuda")})
            host.append((t["srccomps"], t["fmt"], lvl.reshape(-1), words))
    b = s2.Batch(images, opt)
    b.run()
    s2.gpu_synchronize()
    b.close()
    for im, (sc, fmt, px, words) in zip(images, host):
        w, h = im["width"], im["height"]
        want = oracle.compress(sc, w, h, px, fmt, 1, s2.WAVG, 16, 1,
                               rand_words=im["rand"].cpu().numpy().view(np.uint32)[:words])
        assert np.array_equal(im["dst"].cpu().numpy(), want), (w, h, hex(fmt), sc)


def test_tool_call_sequence(lib, oracle):
    """tx_compress_dxtn called level by level, as the reference's s2tc_compress
    calls it, gives the levels of the oracle's DDS file, including the last
    1x1 DXT5 level that reads the previous call's leftover alpha endpoint."""
    for k, (w, h) in enumerate([(2, 2), (5, 3), (37, 23), (64, 16)]):
        img = workloads.value_noise_rgba(40 + k, w, h)
        for dither, metric, nr, refine in ((1, 3, 0, 2), (0, 5, 0, 0), (2, 7, -1, 1)):
            s2.set_env(dither, metric, nr, refine)
            body, lw, lh, pix = b"", w, h, img.reshape(-1)
            while True:
                body += s2.tx_compress_dxtn(4, lw, lh, pix, 0x83F3).tobytes()
                if lw == 1 and lh == 1:
                    break
                pix, lw, lh = oracle.mip_reduce(pix, lw, lh)
            want = oracle.dds(img, w, h, 0x83F3, dither, metric, nr, refine)[128:]
            assert body == want, (w, h, dither, metric, nr, refine)


def test_mip_chains(lib, oracle):
    """Uneven mip chains (1x1, 2x2, 3xN edge levels), mixed formats, RGB and
    RGBA, WAVG with 64 random candidates."""
    tex = workloads.mip_textures(3, count=12, lo=4, hi=200)
    seed = 50
    for t in tex:
        for lvl in t["levels"]:
            h, w = lvl.shape[:2]
            seed += 1
            a = gpu_compress(t["srccomps"], w, h, lvl.reshape(-1), t["fmt"], 1, 5, 64, 1, seed=seed)
            b = oracle.compress(t["srccomps"], w, h, lvl.reshape(-1), t["fmt"], 1, 5, 64, 1, seed=seed)
            assert np.array_equal(a, b), (w, h, t["fmt"], t["srccomps"])


def _batch_vs_single(torch, textures, opt, seed, stream=None):
    """Encode every level of every texture as one batch and one by one through
    tx_compress_dxtn (same rand() stream order); return both outputs."""
    images, refs = [], []
    for t in textures:
        for lvl in t["levels"]:
            h, w = lvl.shape[:2]
            n = s2.compressed_size(w, h, t["fmt"])
            images.append({"src": torch.from_numpy(lvl.reshape(-1).copy()).cuda(), "width": w, "height": h,
                           "srccomps": t["srccomps"], "format": t["fmt"],
                           "dst": torch.full((n,), 0xA5, dtype=torch.uint8, device="cuda")})
    b = s2.Batch(images, opt)
    pyoracle.srand(seed)
    b.run(stream)
    s2.gpu_synchronize(stream)
    got = [im["dst"].cpu().numpy() for im in images]
    s2.set_env(opt.dither, opt.metric, opt.nrandom, opt.refine)
    pyoracle.srand(seed)
    for t in textures:
        for lvl in t["levels"]:
            h, w = lvl.shape[:2]
            refs.append(s2.tx_compress_dxtn(t["srccomps"], w, h, lvl.reshape(-1), t["fmt"]))
    b.close()
    return got, refs


@pytest.mark.parametrize("dither", [0, 1, 2])
def test_batch_mip_chains(lib, dither):
    """One graph launch for uneven mip chains (down to 1x1, with 2x2 and 3xN
    edge levels), mixed formats and component counts, against one
    tx_compress_dxtn call per level."""
    torch = pytest.importorskip("torch")
    tex = workloads.mip_textures(31 + dither, count=9, lo=3, hi=150)
    for opt in (s2.options(dither, s2.WAVG, 8, 1), s2.options(dither, s2.SRGB_MIXED, 0, 2),
                s2.options(dither, s2.W0AVG, -1, 0)):
        got, refs = _batch_vs_single(torch, tex, opt, 77)
        shapes = [(lvl.shape[1], lvl.shape[0], t["fmt"]) for t in tex for lvl in t["levels"]]
        for (w, h, fmt), g, r in zip(shapes, got, refs):
            if cases.is_unpinned_corner(w, h, fmt, opt.metric, opt.nrandom):
                continue  # tx_compress_dxtn carries the previous call's alpha endpoint there
            assert np.array_equal(g, r)


def test_batch_repeated_runs(lib):
    """A plan runs again with new pixel contents and gives fresh results."""
    torch = pytest.importorskip("torch")
    tex = workloads.mip_textures(5, count=4, lo=8, hi=64)
    images = []
    for t in tex:
        lvl = t["levels"][0]
        h, w = lvl.shape[:2]
        images.append({"src": torch.from_numpy(lvl.reshape(-1).copy()).cuda(), "width": w, "height": h,
                       "srccomps": t["srccomps"], "format": t["fmt"],
                       "dst": torch.zeros(s2.compressed_size(w, h, t["fmt"]), dtype=torch.uint8, device="cuda")})
    opt = s2.options(1, s2.SRGB, 0, 2)
    b = s2.Batch(images, opt)
    s2.set_env(1, s2.SRGB, 0, 2)
    for rnd in range(3):
        for im in images:
            im["src"].copy_(torch.randint(0, 256, im["src"].shape, dtype=torch.uint8))
        b.run()
        s2.gpu_synchronize()
        for im in images:
            want = s2.tx_compress_dxtn(im["srccomps"], im["width"], im["height"], im["src"].cpu().numpy(),
                                       im["format"])
            assert np.array_equal(im["dst"].cpu().numpy(), want)
    assert b.kernels >= 2
    b.close()


@pytest.mark.parametrize("metric", range(8))
def test_random_candidates_repeated_values(lib, oracle, metric):
    """Blocks with few distinct colours and alphas: the random candidates
    repeat, and the warp kernel searches the distinct ones only."""
    rng = np.random.default_rng(100 + metric)
    for fmt in (0x83F1, 0x83F2, 0x83F3):
        for kind in (2, 3, 1):
            w, h = int(rng.integers(4, 21)), int(rng.integers(4, 21))
            img = cases.image(rng, w, h, 4, kind)
            for nr, refine in ((64, 1), (9, 2)):
                a = gpu_compress(4, w, h, img, fmt, 0, metric, nr, refine, 5)
                b = oracle.compress(4, w, h, img, fmt, 0, metric, nr, refine, seed=5)
                assert np.array_equal(a, b), (hex(fmt), kind, nr)


def test_gpu_encode_blocks(lib, oracle):
    """The batched per-block entry point on texel words equals the encoder
    half of tx_compress_dxtn (dither NONE makes the texel words known)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    for dxt, fmt, abits in ((0, 0x83F1, 1), (1, 0x83F2, 4), (2, 0x83F3, 8)):
        for metric, nr, refine in ((5, -1, 1), (3, 0, 2), (7, 16, 2), (2, 0, 0), (1, 40, 1)):
            for w, h in ((1, 1), (int(rng.integers(2, 60)), int(rng.integers(2, 60)))):
                img = cases.image(rng, w, h, 4)
                t565 = oracle.rgb565_image(img, w, h, 4, abits, 0)
                d_t = torch.from_numpy(t565).cuda()
                d_out = torch.zeros(s2.compressed_size(w, h, fmt), dtype=torch.uint8, device="cuda")
                pyoracle.srand(5)
                s2.gpu_encode_blocks(d_t, w, h, dxt, metric, nr, refine, d_out)
                s2.gpu_synchronize(None)
                want = oracle.compress(4, w, h, img, fmt, 0, metric, nr, refine, seed=5)
                assert np.array_equal(d_out.cpu().numpy(), want), (dxt, metric, nr, refine, w, h)


def test_device_rand_stream_continues(lib, oracle):
    """Large random-candidate calls take libc's rand() words on the GPU: the
    bytes equal the oracle's (which calls rand() itself) and the process's
    rand() stream continues exactly after the words consumed."""
    img = workloads.plain_rgba(8, 384, 256).reshape(-1)
    for fmt, nr in ((0x83F1, 64), (0x83F3, 9)):
        words = s2.rand_words(384, 256, fmt, s2.options(1, 5, nr, 1))
        assert words >= 16384
        a = gpu_compress(4, 384, 256, img, fmt, 1, 5, nr, 1, seed=31)
        after = pyoracle.libc_rand()
        b = oracle.compress(4, 384, 256, img, fmt, 1, 5, nr, 1, seed=31)
        assert np.array_equal(a, b), hex(fmt)
        pyoracle.srand(31)
        for _ in range(words):
            pyoracle.libc_rand()
        assert after == pyoracle.libc_rand()


def test_launch_layouts_same_bytes(lib, oracle):
    """Every launch layout the autotuner may pick encodes the same bytes, and
    the autotuner itself leaves libc's rand() stream alone."""
    rng = np.random.default_rng(5)
    w, h = 200, 120
    img = cases.image(rng, w, h, 4, 1)
    for fmt, (metric, nr, refine) in ((0x83F3, (5, 24, 1)), (0x83F1, (3, -1, 2)), (0x83F2, (7, 0, 2))):
        want = oracle.compress(4, w, h, img, fmt, 1, metric, nr, refine, seed=3)
        opt = s2.options(1, metric, nr, refine)
        layouts = ([(128, wp, cps) for wp in (1, 2, 4) for cps in (1, 8, 64)] if nr > 0
                   else [(t, 4, 64) for t in (32, 64, 96, 128)])
        for layout in layouts:
            s2.set_layout(opt, fmt, *layout)
            a = gpu_compress(4, w, h, img, fmt, 1, metric, nr, refine, seed=3)
            assert np.array_equal(a, want), (hex(fmt), layout)
        pyoracle.srand(9)
        ms = s2.autotune(opt, fmt, 512, 256)
        assert ms > 0
        x = pyoracle.libc_rand()
        pyoracle.srand(9)
        assert x == pyoracle.libc_rand()
        a = gpu_compress(4, w, h, img, fmt, 1, metric, nr, refine, seed=3)
        assert np.array_equal(a, want), hex(fmt)


def test_pipelined_host_path(lib):
    """Large tx_compress_dxtn calls upload, dither, encode and download in
    overlapping ranges: the bytes equal the device API's (one launch per
    stage), for RGB and RGBA input, padded output rows, every dither it
    covers and the device rand() stream."""
    torch = pytest.importorskip("torch")
    w, h = 2052, 2050  # 4.2 M texels, edge blocks on both sides
    for sc, fmt, dither, metric, nr, refine, stride in ((4, 0x83F3, 1, 3, 0, 2, 0), (3, 0x83F1, 0, 5, -1, 1, 0),
                                                         (4, 0x83F1, 1, 7, 8, 1, 0), (4, 0x83F2, 1, 5, -1, 1, 9000)):
        img = workloads.value_noise_rgba(90 + sc, w, h)[:, :, :sc].copy().reshape(-1)
        dest = np.zeros(((h + 3) // 4) * stride, np.uint8) if stride else None
        a = gpu_compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed=13, stride=stride, dest=dest)
        after = pyoracle.libc_rand()
        opt = s2.options(dither, metric, nr, refine)
        d_src = torch.from_numpy(img).cuda()
        bs = 8 if fmt == 0x83F1 else 16
        row = ((w + 3) // 4) * bs
        d_dst = torch.zeros(row * ((h + 3) // 4), dtype=torch.uint8, device="cuda")
        pyoracle.srand(13)
        s2.gpu_compress(sc, w, h, d_src, fmt, d_dst, opt=opt)
        s2.gpu_synchronize(None)
        assert after == pyoracle.libc_rand(), hex(fmt)
        b = d_dst.cpu().numpy()
        if stride:
            got = a.reshape(-1)[: ((h + 3) // 4) * stride].reshape(-1, stride)[:, :row].reshape(-1)
            assert np.array_equal(got, b), (sc, hex(fmt), stride)
        else:
            assert np.array_equal(a, b), (sc, hex(fmt), dither, metric, nr)


def test_pipelined_host_path_pinned(lib):
    """The pipelined tx_compress_dxtn with pinned source and destination: the
    blocks come back chunk by chunk on the download stream while later
    chunks are encoded on four streams (the doubling dither ranges of a
    2052x2050 image: 16, 32, 64 and 141 tiles; chunks of at most 33 block
    rows), packed or with padded rows (two-dimensional copies), and the DXT5
    all-texels search's carried endpoint crosses from the last chunk to the
    next call's first.  Bytes equal the device API's."""
    torch = pytest.importorskip("torch")
    w, h = 2052, 2050
    for sc, fmt, dither, metric, nr, refine, stride in ((4, 0x83F3, 1, 3, 0, 2, 0), (4, 0x83F3, 1, 5, 0, 1, 9000),
                                                         (3, 0x83F1, 1, 5, -1, 1, 0), (4, 0x83F1, 1, 5, -1, 1, 8300)):
        img = workloads.value_noise_rgba(70 + sc, w, h)[:, :, :sc].copy().reshape(-1)
        bs = 8 if fmt == 0x83F1 else 16
        row = ((w + 3) // 4) * bs
        rows = (h + 3) // 4
        h_src = torch.from_numpy(img).pin_memory()
        h_dst = torch.zeros(rows * (stride or row), dtype=torch.uint8).pin_memory()
        s2.set_env(dither, metric, nr, refine)
        opt = s2.options(dither, metric, nr, refine)
        d_src = torch.from_numpy(img).cuda()
        d_dst = torch.zeros(row * rows, dtype=torch.uint8, device="cuda")
        for _ in range(2):  # the second call reads the first one's carried endpoint
            lib.tx_compress_dxtn(sc, w, h, h_src.data_ptr(), fmt, h_dst.data_ptr(), stride)
            s2.gpu_compress(sc, w, h, d_src, fmt, d_dst, opt=opt)
            s2.gpu_synchronize(None)
            got = h_dst.numpy()
            if stride:
                got = got.reshape(rows, stride)[:, :row].reshape(-1)
            assert np.array_equal(got, d_dst.cpu().numpy()), (sc, hex(fmt), metric, stride)


# --------------------------------------------------------------- strip kernel
# The quick mode with NONE or SIMPLE dither runs as one fused kernel over
# bands of whole block rows (images up to 4160 texels wide): the scan's
# chain crosses every band boundary, and RGBA8 sources come in by tensor
# copies of 256-texel rows that start inside a band's first row.

STRIP_SHAPES = [(3, 5), (255, 1), (257, 3), (1000, 77), (1001, 70), (4160, 9), (4161, 13), (1088, 300),
                (1089, 301), (2000, 600), (64, 260), (130, 131), (4160, 1201), (1024, 1024)]


@pytest.mark.parametrize("direct", ["1", "0"])
@pytest.mark.parametrize("fmt", [0x83F1, 0x83F2, 0x83F3])
def test_strip_bands_and_edges(lib, oracle, monkeypatch, fmt, direct):
    """Widths around the band sizes, the 17- and 65-texel segments and the
    4160 limit (4161 takes the two kernels), widths and heights that are not multiples of 4, RGB and RGBA,
    NONE and SIMPLE dither, every refinement, against the oracle; with the
    kernel reading the caller's host memory where it can (direct), and
    through the staging copies (S2TC_HOST_DIRECT=0)."""
    monkeypatch.setenv("S2TC_HOST_DIRECT", direct)
    rng = np.random.default_rng(fmt)
    for k, (w, h) in enumerate(STRIP_SHAPES):
        sc = 4 if k % 2 == 0 else 3
        img = cases.image(rng, w, h, sc, kind=[0, 4, 2, 0][k % 4])
        dither, metric, refine = k % 2, [5, 3, 0, 2, 4, 6, 1][k % 7], k % 3
        a = gpu_compress(sc, w, h, img, fmt, dither, metric, -1, refine)
        b = oracle.compress(sc, w, h, img, fmt, dither, metric, -1, refine)
        assert np.array_equal(a, b), (w, h, sc, hex(fmt), dither, metric, refine)


def test_strip_device_sources(lib, oracle):
    """The device API on the fused kernel: a 16-byte aligned RGBA source (tensor
    copies), the same pixels 4 bytes further on (vector loads), an image under
    256 texels, and block rows written `dst_pitch` apart."""
    torch = pytest.importorskip("torch")
    for w, h, fmt in ((1000, 333, 0x83F1), (96, 2, 0x83F3), (2051, 19, 0x83F2)):
        img = workloads.plain_rgba(21, w, h).reshape(-1)
        want = oracle.compress(4, w, h, img, fmt, 1, s2.WAVG, -1, 1)
        n, row = s2.compressed_size(w, h, fmt), ((w + 3) // 4) * s2.block_bytes(fmt)
        for shift in (0, 4):
            buf = torch.zeros(img.size + 64, dtype=torch.uint8, device="cuda")
            buf[shift:shift + img.size] = torch.from_numpy(img.copy()).cuda()
            d_dst = torch.full((n + 64 * ((h + 3) // 4),), 0x5A, dtype=torch.uint8, device="cuda")
            pitch = row + 64
            s2.gpu_compress(4, w, h, buf.data_ptr() + shift, fmt, d_dst, dst_pitch=pitch,
                            opt=s2.options(1, s2.WAVG, -1, 1))
            s2.gpu_synchronize()
            got = d_dst.cpu().numpy().reshape(-1, pitch)[:, :row].reshape(-1)[:n]
            assert np.array_equal(got, want), (w, h, hex(fmt), shift)


@pytest.mark.parametrize("direct", ["1", "0"])
def test_strip_pipelined_host_path(lib, oracle, monkeypatch, direct):
    """tx_compress_dxtn on images of at least 4 Mi texels in quick mode: where
    the GPU reads host memory coherently, one fused launch reads the pixels
    and writes the blocks in host memory (direct); otherwise
    (S2TC_HOST_DIRECT=0 here) the image goes up in ranges of bands and each
    range is one fused launch whose look-back reaches into the ranges before
    it."""
    monkeypatch.setenv("S2TC_HOST_DIRECT", direct)
    for w, h, fmt, sc, dither in ((2048, 2051, 0x83F1, 4, 1), (8192, 515, 0x83F3, 4, 1), (3001, 1500, 0x83F2, 3, 0)):
        img = workloads.plain_rgba(22, w, h)[:, :, :sc].reshape(-1) if sc == 4 else \
            np.ascontiguousarray(workloads.plain_rgba(22, w, h)[:, :, :3]).reshape(-1)
        a = gpu_compress(sc, w, h, img, fmt, dither, s2.WAVG, -1, 1)
        b = oracle.compress(sc, w, h, img, fmt, dither, s2.WAVG, -1, 1)
        assert np.array_equal(a, b), (w, h, hex(fmt), sc, dither)
