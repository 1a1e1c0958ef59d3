"""Host-side checks of the C ABI that need no GPU: the library loads and
exports every symbol its header declares, the environment knobs parse like
the reference's, the texel decoders match the oracle, and invalid formats are
rejected before any device work."""
import ctypes
import os
import re
from pathlib import Path

import numpy as np
import pytest

import s2tc_gb300 as s2

HEADER = Path(__file__).resolve().parents[1] / "include" / "s2tc_gb300.h"


def _declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = set()
    for m in re.finditer(r"^[A-Za-z_][\w \t\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
        if not text[m.start():].startswith("typedef"):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol(lib):
    declared = _declared_functions()
    assert {"tx_compress_dxtn", "rgb565_image", "s2tc_encode_block_func"} <= declared
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(s2.EXPORTED_SYMBOLS)


def test_env_parsing(lib, capfd, monkeypatch):
    for k in ("S2TC_DITHER_MODE", "S2TC_COLORDIST_MODE", "S2TC_RANDOM_COLORS", "S2TC_REFINE_COLORS"):
        monkeypatch.delenv(k, raising=False)
    o = s2.options_from_env()
    assert (o.dither, o.metric, o.nrandom, o.refine) == (1, 5, -1, 1)
    monkeypatch.setenv("S2TC_DITHER_MODE", "floydsteinberg")
    monkeypatch.setenv("S2TC_COLORDIST_MODE", "srgb_Mixed")
    monkeypatch.setenv("S2TC_RANDOM_COLORS", "64abc")
    monkeypatch.setenv("S2TC_REFINE_COLORS", "Loop")
    o = s2.options_from_env()
    assert (o.dither, o.metric, o.nrandom, o.refine) == (2, 3, 64, 2)
    for i, name in enumerate(s2.COLORDIST_NAMES):
        monkeypatch.setenv("S2TC_COLORDIST_MODE", name.lower())
        assert s2.options_from_env().metric == i
    monkeypatch.setenv("S2TC_DITHER_MODE", "bogus")
    monkeypatch.setenv("S2TC_COLORDIST_MODE", "HSV")
    monkeypatch.setenv("S2TC_REFINE_COLORS", "SOMETIMES")
    monkeypatch.setenv("S2TC_RANDOM_COLORS", "x")
    capfd.readouterr()
    o = s2.options_from_env()
    assert (o.dither, o.metric, o.nrandom, o.refine) == (1, 5, 0, 1)
    err = capfd.readouterr().err
    assert "Invalid dither mode: bogus" in err
    assert "Invalid color dist mode: HSV" in err
    assert "Invalid refinement mode: SOMETIMES" in err


def test_bad_format_writes_nothing(lib, capfd):
    dest = np.full(64, 0x5A, np.uint8)
    src = np.zeros(8 * 8 * 4, np.uint8)
    capfd.readouterr()
    lib.tx_compress_dxtn(4, 8, 8, src.ctypes.data, 0x1234, dest.ctypes.data, 0)
    assert "libdxtn: Bad dstFormat 4660 in tx_compress_dxtn" in capfd.readouterr().err
    assert (dest == 0x5A).all()


def test_rand_words(lib):
    o = s2.options(nrandom=64)
    assert s2.rand_words(9, 5, 0x83F3, o) == 3 * 2 * 64 * 4
    assert s2.rand_words(9, 5, 0x83F1, o) == 3 * 2 * 64 * 3
    assert s2.rand_words(9, 5, 0x83F1, s2.options(nrandom=0)) == 0
    assert s2.rand_words(9, 5, 0x83F1, s2.options(nrandom=-1, metric=s2.NORMALMAP)) == 0
    assert s2.rand_words(9, 5, 0x1234, o) == 0


def test_fetch_matches_oracle(lib, oracle):
    rng = np.random.default_rng(3)
    for fmt in s2.FORMATS:
        dxt = s2.format_dxt(fmt)
        w, h = 12, 8
        data = rng.integers(0, 256, s2.compressed_size(w, h, fmt), dtype=np.uint8)
        # make some blocks use the c1 >= c0 and a1 >= a0 forms
        bs = s2.block_bytes(fmt)
        data[bs - 7::2 * bs] = 0
        for j in range(h):
            for i in range(w):
                got = s2.fetch_texel(fmt, w, data, i, j)
                want = oracle.fetch(dxt, 1 if fmt != 0x83F0 else 0, w, data, i, j)
                if fmt == 0x83F0:
                    want[3] = 255
                assert np.array_equal(got, want), (hex(fmt), i, j)


def test_fetch_matches_reference(lib, reference):
    rng = np.random.default_rng(4)
    names = ("fetch_2d_texel_rgb_dxt1", "fetch_2d_texel_rgba_dxt1", "fetch_2d_texel_rgba_dxt3",
             "fetch_2d_texel_rgba_dxt5")
    for fmt, name in zip(s2.FORMATS, names):
        rf = getattr(reference.lib, "ref_" + name)
        rf.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        data = rng.integers(0, 256, s2.compressed_size(16, 8, fmt), dtype=np.uint8)
        for j in range(8):
            for i in range(16):
                t = np.zeros(4, np.uint8)
                rf(16, data.ctypes.data, i, j, t.ctypes.data)
                got = s2.fetch_texel(fmt, 16, data, i, j)
                n = 3 if fmt == 0x83F0 else 4
                assert np.array_equal(got[:n], t[:n]), (name, i, j)


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_without_gpu_fails_loudly(lib, capfd):
    """No CPU fallback: without a device the call reports and writes nothing."""
    if _has_gpu():
        pytest.skip("a GPU is present")
    dest = np.full(32, 0x5A, np.uint8)
    src = np.zeros(8 * 8 * 4, np.uint8)
    capfd.readouterr()
    lib.tx_compress_dxtn(4, 8, 8, src.ctypes.data, 0x83F1, dest.ctypes.data, 0)
    assert "s2tc_gb300:" in capfd.readouterr().err
    assert (dest == 0x5A).all()
    assert s2.last_error()
