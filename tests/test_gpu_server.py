"""The continuous-batching request loop: every result equals the one the
request gets alone through tx_compress_dxtn, whatever else is in flight."""
import numpy as np
import pytest

import cases
import pyoracle
import s2tc_gb300 as s2
from s2tc_gb300 import workloads

pytestmark = pytest.mark.gpu


def _requests(seed, count):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        w, h = int(rng.integers(1, 300)), int(rng.integers(1, 200))
        fmt = int(rng.choice([0x83F1, 0x83F3, 0x83F2, 0x83F0]))
        metric = int(rng.choice([5, 3, 7, 2]))
        opt = s2.options(int(rng.integers(0, 3)), metric, int(rng.choice([-1, 0, 4])), int(rng.integers(0, 3)))
        img = workloads.plain_rgba(int(seed * 1000 + i), w, h).reshape(-1)
        reqs.append((img, w, h, fmt, opt))
    return reqs


def test_server_matches_requests_alone(lib):
    torch = pytest.importorskip("torch")
    reqs = _requests(3, 60)
    srv = s2.Server(256 << 20)
    pyoracle.srand(9)  # random candidates draw rand() at submit time, in order
    outs, ids = [], []
    for img, w, h, fmt, opt in reqs:
        src = torch.from_numpy(img).pin_memory()
        dst = torch.zeros(s2.compressed_size(w, h, fmt), dtype=torch.uint8).pin_memory()
        outs.append(dst)
        ids.append(srv.submit(src, 4, w, h, fmt, opt, dst))
    lat = [srv.wait(i) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["done"] == len(reqs) and st["rounds"] >= 1
    assert all(x >= 0 for x in lat)
    pyoracle.srand(9)
    for (img, w, h, fmt, opt), got in zip(reqs, outs):
        s2.set_env(opt.dither, opt.metric, opt.nrandom, opt.refine)
        want = s2.tx_compress_dxtn(4, w, h, img, fmt)
        if cases.is_unpinned_corner(w, h, fmt, opt.metric, opt.nrandom):
            continue  # tx_compress_dxtn carries the previous call's alpha endpoint there
        assert np.array_equal(got.numpy(), want), (w, h, hex(fmt), opt.metric, opt.nrandom)


def test_server_random_candidates(lib):
    """Random-candidate requests large enough for the device generator: the
    words each request draws at submit time, in order, match one
    tx_compress_dxtn call per request in the same order."""
    torch = pytest.importorskip("torch")
    srv = s2.Server(1 << 30)
    reqs = []
    for k, (w, h, fmt) in enumerate([(256, 192, 0x83F1), (64, 64, 0x83F3), (300, 200, 0x83F3), (128, 512, 0x83F1)]):
        img = workloads.plain_rgba(60 + k, w, h).reshape(-1)
        dst = torch.zeros(s2.compressed_size(w, h, fmt), dtype=torch.uint8).pin_memory()
        reqs.append((img, w, h, fmt, dst))
    opt = s2.options(1, s2.WAVG, 32, 1)
    pyoracle.srand(77)
    ids = [srv.submit(torch.from_numpy(img).pin_memory(), 4, w, h, fmt, opt, dst) for img, w, h, fmt, dst in reqs]
    for i in ids:
        srv.wait(i)
    srv.close()
    s2.set_env(1, s2.WAVG, 32, 1)
    pyoracle.srand(77)
    for img, w, h, fmt, dst in reqs:
        assert np.array_equal(dst.numpy(), s2.tx_compress_dxtn(4, w, h, img, fmt)), (w, h, hex(fmt))


def test_server_budget_admission(lib):
    """A small budget admits requests as memory frees up (several rounds, the
    pool never above the budget); a request above the budget is refused."""
    torch = pytest.importorskip("torch")
    budget = 3 << 20
    srv = s2.Server(budget)
    img = workloads.plain_rgba(5, 512, 384).reshape(-1)  # ~1.7 MB of device memory per request
    src = torch.from_numpy(img).pin_memory()
    dsts = [torch.zeros(s2.compressed_size(512, 384, 0x83F1), dtype=torch.uint8).pin_memory() for _ in range(6)]
    opt = s2.options(1, s2.WAVG, -1, 1)
    ids = [srv.submit(src, 4, 512, 384, 0x83F1, opt, d) for d in dsts]
    for i in ids:
        srv.wait(i)
    st = srv.stats()
    assert st["rounds"] >= 6 and st["max_round_requests"] == 1
    assert st["pool_high_water"] <= budget
    s2.set_env(1, s2.WAVG, -1, 1)
    want = s2.tx_compress_dxtn(4, 512, 384, img, 0x83F1)
    assert all(np.array_equal(d.numpy(), want) for d in dsts)
    big = workloads.plain_rgba(6, 1024, 1024).reshape(-1)
    out = np.zeros(s2.compressed_size(1024, 1024, 0x83F1), np.uint8)
    with pytest.raises(s2.S2tcError):
        srv.submit(big, 4, 1024, 1024, 0x83F1, opt, out)
    srv.close()


def test_server_threads_and_rounds(lib):
    """Requests submitted from two threads under a budget that holds about
    five at a time run in several rounds and all match tx_compress_dxtn."""
    import threading
    torch = pytest.importorskip("torch")
    srv = s2.Server(40 << 20)
    opt = s2.options(1, s2.SRGB_MIXED, 0, 2)
    w, h = 1024, 768
    bufs = []
    for k in range(16):
        img = workloads.value_noise_rgba(k, w, h).reshape(-1)
        bufs.append((img, torch.from_numpy(img).pin_memory(),
                     torch.zeros(s2.compressed_size(w, h, 0x83F3), dtype=torch.uint8).pin_memory()))
    ids = [[], []]

    def client(t):
        for img, src, dst in bufs[t::2]:
            ids[t].append(srv.submit(src, 4, w, h, 0x83F3, opt, dst))

    th = [threading.Thread(target=client, args=(t,)) for t in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i in ids[0] + ids[1]:
        srv.wait(i)
    st = srv.stats()
    srv.close()
    assert st["done"] == 16 and st["rounds"] >= 4 and st["pool_high_water"] <= 40 << 20
    s2.set_env(1, s2.SRGB_MIXED, 0, 2)
    for img, src, dst in bufs:
        assert np.array_equal(dst.numpy(), s2.tx_compress_dxtn(4, w, h, img, 0x83F3))


def test_server_device_resident_requests(lib):
    """Device-resident requests (no copies, blocks written in place, padded
    rows) mixed with host requests give tx_compress_dxtn's bytes."""
    torch = pytest.importorskip("torch")
    srv = s2.Server(256 << 20)
    opt = s2.options(1, s2.SRGB_MIXED, 0, 2)
    jobs = []
    for k, (w, h, fmt) in enumerate([(100, 60, 0x83F3), (257, 129, 0x83F1), (64, 64, 0x83F2), (33, 5, 0x83F3)]):
        img = workloads.value_noise_rgba(70 + k, w, h).reshape(-1)
        row = ((w + 3) // 4) * (8 if fmt == 0x83F1 else 16)
        pitch = row + 32
        d_src = torch.from_numpy(img).cuda()
        d_dst = torch.zeros(pitch * ((h + 3) // 4), dtype=torch.uint8, device="cuda")
        h_dst = torch.zeros(s2.compressed_size(w, h, fmt), dtype=torch.uint8).pin_memory()
        a = srv.submit_device(d_src, 4, w, h, fmt, opt, d_dst, pitch)
        b = srv.submit(torch.from_numpy(img).pin_memory(), 4, w, h, fmt, opt, h_dst)
        jobs.append((img, w, h, fmt, row, pitch, d_dst, h_dst, a, b))
    for j in jobs:
        srv.wait(j[8])
        srv.wait(j[9])
    srv.close()
    s2.set_env(1, s2.SRGB_MIXED, 0, 2)
    for img, w, h, fmt, row, pitch, d_dst, h_dst, _, _ in jobs:
        want = s2.tx_compress_dxtn(4, w, h, img, fmt)
        got = d_dst.cpu().numpy().reshape(-1, pitch)[:, :row].reshape(-1)
        assert np.array_equal(got, want), (w, h, hex(fmt))
        assert np.array_equal(h_dst.numpy(), want), (w, h, hex(fmt))
