"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU checkers.

* ``Oracle``    -- the C restatement oracle/s2tc_oracle.c (libs2tc_oracle.so),
  built on every machine by ``make -C oracle``.
* ``Reference`` -- the reference's own encoder compiled from its sources
  (oracle/_ref/libs2tc_ref.so, symbols prefixed ``ref_``); only present where
  the reference sources were available at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs use this
module, and only as the checker / CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libs2tc_oracle.so"
REF_SO = HERE / "_ref" / "libs2tc_ref.so"
REF_WRAPV_SO = HERE / "_ref" / "libs2tc_ref_wrapv.so"

_libc = ctypes.CDLL(None)
_libc.srand.argtypes = [ctypes.c_uint]
_libc.rand.restype = ctypes.c_int

DITHER_NAMES = ("NONE", "SIMPLE", "FLOYDSTEINBERG")
COLORDIST_NAMES = ("RGB", "YUV", "SRGB", "SRGB_MIXED", "AVG", "WAVG", "W0AVG", "NORMALMAP")
REFINE_NAMES = ("NEVER", "ALWAYS", "LOOP")


def srand(seed: int) -> None:
    """Seed libc's rand() stream (shared by every library in the process)."""
    _libc.srand(seed)


def libc_rand() -> int:
    return _libc.rand()


def _vp(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def _block_bytes(fmt: int) -> int:
    return 8 if fmt in (0x83F0, 0x83F1) else 16


def out_size(w: int, h: int, fmt: int) -> int:
    return ((w + 3) // 4) * ((h + 3) // 4) * _block_bytes(fmt)


def ensure_built() -> None:
    if not ORACLE_SO.exists():
        subprocess.run(["make", "-C", str(HERE), "oracle"], check=True, capture_output=True)


class Oracle:
    """The C restatement of the encode path."""

    def __init__(self, path: os.PathLike | None = None):
        ensure_built()
        lib = ctypes.CDLL(str(path or ORACLE_SO))
        i, u, vp = ctypes.c_int, ctypes.c_uint, ctypes.c_void_p
        lib.s2tc_oracle_compress.argtypes = [i, i, i, vp, u, vp, i, i, i, i, i]
        lib.s2tc_oracle_compress.restype = i
        lib.s2tc_oracle_rgb565_image.argtypes = [vp, vp, i, i, i, i, i]
        lib.s2tc_oracle_encode_block_ex.argtypes = [vp, vp, i, i, i, i, i, i, i, i]
        lib.s2tc_oracle_encode_block_ex.restype = i
        lib.s2tc_oracle_color_dist.argtypes = [i] * 7
        lib.s2tc_oracle_color_dist.restype = ctypes.c_int32
        lib.s2tc_oracle_fetch.argtypes = [i, i, i, vp, i, i, vp]
        lg = ctypes.c_long
        lib.s2tc_oracle_mip_reduce.argtypes = [vp, vp, ctypes.POINTER(i), ctypes.POINTER(i)]
        lib.s2tc_oracle_dds_size.argtypes = [i, i, u]
        lib.s2tc_oracle_dds_size.restype = lg
        lib.s2tc_oracle_dds.argtypes = [vp, i, i, u, i, i, i, i, vp]
        lib.s2tc_oracle_dds.restype = lg
        lib.s2tc_oracle_decompress.argtypes = [vp, vp]
        lib.s2tc_oracle_decompress.restype = lg
        lib.s2tc_oracle_from_s3tc_block.argtypes = [i, vp]
        lib.s2tc_oracle_from_s3tc.argtypes = [vp, lg, vp]
        lib.s2tc_oracle_from_s3tc.restype = lg
        lib.s2tc_oracle_set_rand_words.argtypes = [vp, lg]
        lib.s2tc_oracle_rand_words_used.restype = lg
        self.lib = lib

    def compress(self, srccomps, w, h, src, fmt, dither, metric, nrandom, refine,
                 dst_row_stride=0, dest=None, seed=None, rand_words=None) -> np.ndarray:
        """tx_compress_dxtn with explicit knobs.  `rand_words`: the random
        candidates' words in the reference's call order, instead of libc's
        rand() (the call must take exactly that many, or ValueError)."""
        src = np.ascontiguousarray(src, dtype=np.uint8)
        if dest is None:
            dest = np.zeros(out_size(w, h, fmt), np.uint8)
        if seed is not None:
            srand(seed)
        words = None
        if rand_words is not None:
            words = np.ascontiguousarray(rand_words, dtype=np.uint32)
            self.lib.s2tc_oracle_set_rand_words(_vp(words), words.size)
        try:
            self.lib.s2tc_oracle_compress(srccomps, w, h, _vp(src), fmt, _vp(dest), dst_row_stride,
                                          dither, metric, nrandom, refine)
            used = self.lib.s2tc_oracle_rand_words_used() if words is not None else 0
        finally:
            if words is not None:
                self.lib.s2tc_oracle_set_rand_words(None, 0)
        if words is not None and used != words.size:
            raise ValueError(f"the call took {used} random words, {words.size} were given")
        return dest

    def rgb565_image(self, src, w, h, srccomps, alphabits, dither) -> np.ndarray:
        src = np.ascontiguousarray(src, dtype=np.uint8)
        out = np.zeros(w * h * 4, np.uint8)
        self.lib.s2tc_oracle_rgb565_image(_vp(out), _vp(src), w, h, srccomps, alphabits, dither)
        return out

    def encode_block(self, t565, iw, w, h, dxt, metric, nrandom, refine, prev_a1=-1, offset=0):
        """Encode the block whose first texel is texel `offset` of `t565`;
        returns (bytes, leftover alpha)."""
        out = np.zeros(16, np.uint8)
        ptr = ctypes.c_void_p(t565.ctypes.data + 4 * offset)
        left = self.lib.s2tc_oracle_encode_block_ex(_vp(out), ptr, iw, w, h, dxt, metric, nrandom, refine, prev_a1)
        return out[: 8 if dxt == 0 else 16], left

    def color_dist(self, metric, a, b) -> int:
        return self.lib.s2tc_oracle_color_dist(metric, *a, *b)

    def fetch(self, dxt, rgba_dxt1, stride, data, i, j) -> np.ndarray:
        t = np.zeros(4, np.uint8)
        self.lib.s2tc_oracle_fetch(dxt, rgba_dxt1, stride, _vp(data), i, j, _vp(t))
        return t


    # ---- the reference's command-line tools, in memory

    def mip_reduce(self, rgba, w, h):
        """One Image_MipReduce32 step towards 1x1: (pixels, w, h)."""
        src = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(-1)
        out = np.zeros(max(1, (w // 2 or 1) * (h // 2 or 1)) * 4, np.uint8)
        cw, ch = ctypes.c_int(w), ctypes.c_int(h)
        self.lib.s2tc_oracle_mip_reduce(_vp(src), _vp(out), ctypes.byref(cw), ctypes.byref(ch))
        return out[: cw.value * ch.value * 4], cw.value, ch.value

    def dds_size(self, w, h, fmt) -> int:
        return self.lib.s2tc_oracle_dds_size(w, h, fmt)

    def dds(self, rgba, w, h, fmt, dither, metric, nrandom, refine, seed=None) -> bytes:
        """s2tc_compress's DDS output for an RGBA8 image."""
        src = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(-1)
        out = np.zeros(self.dds_size(w, h, fmt), np.uint8)
        if seed is not None:
            srand(seed)
        n = self.lib.s2tc_oracle_dds(_vp(src), w, h, fmt, dither, metric, nrandom, refine, _vp(out))
        assert n == out.size, (n, out.size)
        return out.tobytes()

    def decompress(self, dds: bytes) -> bytes:
        """s2tc_decompress's TGA output for a DXT1/3/5 DDS file."""
        src = np.frombuffer(dds, np.uint8).copy()
        w, h = int.from_bytes(dds[16:20], "little"), int.from_bytes(dds[12:16], "little")
        out = np.zeros(18 + 4 * w * h, np.uint8)
        n = self.lib.s2tc_oracle_decompress(_vp(src), _vp(out))
        if n < 0:
            raise ValueError("unsupported FourCC")
        return out[:n].tobytes()

    def from_s3tc(self, dds: bytes) -> bytes:
        """s2tc_from_s3tc's output for an S3TC DDS file."""
        src = np.frombuffer(dds, np.uint8).copy()
        out = np.zeros(max(128, len(dds)), np.uint8)
        n = self.lib.s2tc_oracle_from_s3tc(_vp(src), len(dds), _vp(out))
        if n < 0:
            raise ValueError("unsupported file")
        return out[:n].tobytes()

    def from_s3tc_blocks(self, blocks: np.ndarray, dxt: int) -> np.ndarray:
        out = np.ascontiguousarray(blocks, dtype=np.uint8).copy()
        bs = 8 if dxt == 0 else 16
        for k in range(out.size // bs):
            self.lib.s2tc_oracle_from_s3tc_block(dxt, ctypes.c_void_p(out.ctypes.data + k * bs))
        return out


class ReferenceTools:
    """The reference's s2tc_compress, s2tc_decompress and s2tc_from_s3tc
    programs compiled from its own sources (`make -C oracle ref`)."""

    def __init__(self, bindir: os.PathLike | None = None):
        self.bindir = Path(bindir or REF_SO.parent)

    def available(self) -> bool:
        return all((self.bindir / t).exists() for t in ("s2tc_compress", "s2tc_decompress", "s2tc_from_s3tc"))

    def _run(self, tool, args, data: bytes, env=None) -> bytes:
        import subprocess
        r = subprocess.run([str(self.bindir / tool), *args], input=data, capture_output=True, env=env, check=True)
        return r.stdout

    def compress(self, tga: bytes, fourcc: str, dither, metric, nrandom, refine) -> bytes:
        env = dict(os.environ, S2TC_DITHER_MODE=DITHER_NAMES[dither], S2TC_COLORDIST_MODE=COLORDIST_NAMES[metric],
                   S2TC_RANDOM_COLORS=str(nrandom), S2TC_REFINE_COLORS=REFINE_NAMES[refine])
        return self._run("s2tc_compress", ["-t", fourcc], tga, env)

    def decompress(self, dds: bytes) -> bytes:
        return self._run("s2tc_decompress", [], dds)

    def from_s3tc(self, dds: bytes) -> bytes:
        return self._run("s2tc_from_s3tc", [], dds)


class Reference:
    """The reference encoder compiled from its own sources (knobs via env)."""

    def __init__(self, path: os.PathLike | None = None):
        p = Path(path or REF_SO)
        if not p.exists():
            raise FileNotFoundError(p)
        lib = ctypes.CDLL(str(p))
        i, u, vp = ctypes.c_int, ctypes.c_uint, ctypes.c_void_p
        lib.ref_tx_compress_dxtn.argtypes = [i, i, i, vp, u, vp, i]
        lib.ref_rgb565_image.argtypes = [vp, vp, i, i, i, i, i]
        lib.ref_s2tc_encode_block_func.argtypes = [i, i, i, i]
        lib.ref_s2tc_encode_block_func.restype = vp
        self.lib = lib

    @staticmethod
    def available(path: os.PathLike | None = None) -> bool:
        return Path(path or REF_SO).exists()

    def compress(self, srccomps, w, h, src, fmt, dither, metric, nrandom, refine,
                 dst_row_stride=0, dest=None, seed=None) -> np.ndarray:
        src = np.ascontiguousarray(src, dtype=np.uint8)
        os.environ["S2TC_DITHER_MODE"] = DITHER_NAMES[dither]
        os.environ["S2TC_COLORDIST_MODE"] = COLORDIST_NAMES[metric]
        os.environ["S2TC_RANDOM_COLORS"] = str(nrandom)
        os.environ["S2TC_REFINE_COLORS"] = REFINE_NAMES[refine]
        if dest is None:
            dest = np.zeros(out_size(w, h, fmt), np.uint8)
        if seed is not None:
            srand(seed)
        self.lib.ref_tx_compress_dxtn(srccomps, w, h, _vp(src), fmt, _vp(dest), dst_row_stride)
        return dest

    def rgb565_image(self, src, w, h, srccomps, alphabits, dither) -> np.ndarray:
        src = np.ascontiguousarray(src, dtype=np.uint8)
        out = np.zeros(w * h * 4, np.uint8)
        self.lib.ref_rgb565_image(_vp(out), _vp(src), w, h, srccomps, alphabits, dither)
        return out
