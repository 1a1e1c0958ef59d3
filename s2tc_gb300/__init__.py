"""GB300 S2TC encoder: Python view of the C ABI in ``include/s2tc_gb300.h``.

The compute path is ``libs2tc_gb300.so`` (hand-written CUDA for sm_103a behind a
C ABI).  This module only loads it and converts numpy / torch buffers to
pointers; it has no encoding code of its own, so there is nothing to fall back
to: if the library cannot be loaded, importing ``lib`` raises.

Names and argument meaning follow the reference's API (divVerent/s2tc:
``tx_compress_dxtn`` in txc_dxtn.h:47-49, ``rgb565_image`` and
``s2tc_encode_block_func`` in s2tc_algorithm.h:38, 65-66).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libs2tc_gb300.so"

# GL_EXT_texture_compression_s3tc formats
GL_COMPRESSED_RGB_S3TC_DXT1_EXT = 0x83F0
GL_COMPRESSED_RGBA_S3TC_DXT1_EXT = 0x83F1
GL_COMPRESSED_RGBA_S3TC_DXT3_EXT = 0x83F2
GL_COMPRESSED_RGBA_S3TC_DXT5_EXT = 0x83F3
FORMATS = (GL_COMPRESSED_RGB_S3TC_DXT1_EXT, GL_COMPRESSED_RGBA_S3TC_DXT1_EXT,
           GL_COMPRESSED_RGBA_S3TC_DXT3_EXT, GL_COMPRESSED_RGBA_S3TC_DXT5_EXT)

# Enums with the reference's values (s2tc_algorithm.h:31-63)
DITHER_NONE, DITHER_SIMPLE, DITHER_FLOYDSTEINBERG = 0, 1, 2
DXT1, DXT3, DXT5 = 0, 1, 2
REFINE_NEVER, REFINE_ALWAYS, REFINE_LOOP = 0, 1, 2
RGB, YUV, SRGB, SRGB_MIXED, AVG, WAVG, W0AVG, NORMALMAP = range(8)

DITHER_NAMES = ("NONE", "SIMPLE", "FLOYDSTEINBERG")
COLORDIST_NAMES = ("RGB", "YUV", "SRGB", "SRGB_MIXED", "AVG", "WAVG", "W0AVG", "NORMALMAP")
REFINE_NAMES = ("NEVER", "ALWAYS", "LOOP")

S2TC_OK = 0


class S2tcError(RuntimeError):
    pass


class Image(ctypes.Structure):
    """``s2tc_image``: one image of a batch (device pointers)."""
    _fields_ = [("src", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("srccomps", ctypes.c_int), ("format", ctypes.c_uint), ("dst", ctypes.c_void_p),
                ("dst_pitch", ctypes.c_longlong), ("rand", ctypes.c_void_p)]


class Options(ctypes.Structure):
    """``s2tc_options``: the S2TC_* knobs as a struct."""
    _fields_ = [("dither", ctypes.c_int), ("metric", ctypes.c_int),
                ("nrandom", ctypes.c_int), ("refine", ctypes.c_int)]


def format_dxt(fmt: int) -> int:
    return {GL_COMPRESSED_RGB_S3TC_DXT1_EXT: DXT1, GL_COMPRESSED_RGBA_S3TC_DXT1_EXT: DXT1,
            GL_COMPRESSED_RGBA_S3TC_DXT3_EXT: DXT3, GL_COMPRESSED_RGBA_S3TC_DXT5_EXT: DXT5}[fmt]


def block_bytes(fmt: int) -> int:
    return 8 if format_dxt(fmt) == DXT1 else 16


def compressed_size(width: int, height: int, fmt: int) -> int:
    return ((width + 3) // 4) * ((height + 3) // 4) * block_bytes(fmt)


_lib = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load ``libs2tc_gb300.so`` (building is ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise S2tcError(f"{p} is missing: build it with s2tc_gb300/build.py")
    lib = ctypes.CDLL(str(p))
    c_int, c_uint, vp, c_ll = ctypes.c_int, ctypes.c_uint, ctypes.c_void_p, ctypes.c_longlong
    lib.tx_compress_dxtn.argtypes = [c_int, c_int, c_int, vp, c_uint, vp, c_int]
    lib.tx_compress_dxtn.restype = None
    lib.rgb565_image.argtypes = [vp, vp, c_int, c_int, c_int, c_int, c_int]
    lib.rgb565_image.restype = None
    lib.s2tc_encode_block_func.argtypes = [c_int, c_int, c_int, c_int]
    lib.s2tc_encode_block_func.restype = vp
    for name in ("fetch_2d_texel_rgb_dxt1", "fetch_2d_texel_rgba_dxt1",
                 "fetch_2d_texel_rgba_dxt3", "fetch_2d_texel_rgba_dxt5"):
        f = getattr(lib, name)
        f.argtypes = [c_int, vp, c_int, c_int, vp]
        f.restype = None
    lib.s2tc_options_from_env.argtypes = [ctypes.POINTER(Options)]
    lib.s2tc_options_from_env.restype = None
    lib.s2tc_gpu_compress.argtypes = [c_int, c_int, c_int, vp, c_uint, vp, c_ll,
                                      ctypes.POINTER(Options), vp, vp]
    lib.s2tc_gpu_compress.restype = c_int
    lib.s2tc_gpu_compress_noalloc.argtypes = [c_int, c_int, c_int, vp, c_uint, vp, c_ll,
                                              ctypes.POINTER(Options), vp, vp]
    lib.s2tc_gpu_compress_noalloc.restype = c_int
    lib.s2tc_gpu_synchronize.argtypes = [vp]
    lib.s2tc_gpu_synchronize.restype = c_int
    lib.s2tc_rand_words.argtypes = [c_int, c_int, c_uint, ctypes.POINTER(Options)]
    lib.s2tc_rand_words.restype = c_ll
    lib.s2tc_gpu_set_timing.argtypes = [c_int]
    lib.s2tc_gpu_set_timing.restype = c_int
    lib.s2tc_gpu_stage_ms.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(c_ll)]
    lib.s2tc_gpu_stage_ms.restype = c_int
    lib.s2tc_gpu_kernel_launches.argtypes = []
    lib.s2tc_gpu_kernel_launches.restype = c_ll
    lib.s2tc_test_dither_hold.argtypes = [c_ll, c_int]
    lib.s2tc_test_dither_hold.restype = c_int
    lib.s2tc_gpu_compress_each.argtypes = [ctypes.POINTER(Image), c_int, ctypes.POINTER(Options), vp]
    lib.s2tc_gpu_compress_each.restype = c_int
    lib.s2tc_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Image), c_int,
                                      ctypes.POINTER(Options)]
    lib.s2tc_batch_create.restype = c_int
    lib.s2tc_batch_run.argtypes = [vp, vp]
    lib.s2tc_batch_run.restype = c_int
    lib.s2tc_batch_kernels.argtypes = [vp]
    lib.s2tc_batch_kernels.restype = c_int
    lib.s2tc_batch_destroy.argtypes = [vp]
    lib.s2tc_batch_destroy.restype = None
    lib.s2tc_server_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), c_ll]
    lib.s2tc_server_create.restype = c_int
    lib.s2tc_server_submit.argtypes = [vp, vp, c_int, c_int, c_int, c_uint, ctypes.POINTER(Options), vp, c_ll,
                                       ctypes.POINTER(c_ll)]
    lib.s2tc_server_submit.restype = c_int
    lib.s2tc_server_submit_device.argtypes = [vp, vp, c_int, c_int, c_int, c_uint, ctypes.POINTER(Options), vp,
                                              c_ll, ctypes.POINTER(c_ll)]
    lib.s2tc_server_submit_device.restype = c_int
    lib.s2tc_server_wait.argtypes = [vp, c_ll, ctypes.POINTER(ctypes.c_double)]
    lib.s2tc_server_wait.restype = c_int
    lib.s2tc_server_stats.argtypes = [vp, ctypes.POINTER(c_ll), ctypes.POINTER(c_ll), ctypes.POINTER(c_int),
                                      ctypes.POINTER(c_int), ctypes.POINTER(c_ll)]
    lib.s2tc_server_stats.restype = c_int
    lib.s2tc_server_destroy.argtypes = [vp]
    lib.s2tc_server_destroy.restype = None
    lib.s2tc_gpu_encode_blocks.argtypes = [vp, c_int, c_int, c_int, c_int, c_int, c_int, vp, c_ll, vp, vp]
    lib.s2tc_gpu_encode_blocks.restype = c_int
    lib.s2tc_autotune.argtypes = [ctypes.POINTER(Options), c_uint, c_int, c_int, ctypes.POINTER(ctypes.c_float)]
    lib.s2tc_autotune.restype = c_int
    lib.s2tc_encode_layout_set.argtypes = [ctypes.POINTER(Options), c_uint, c_int, c_int, c_int]
    lib.s2tc_encode_layout_set.restype = c_int
    lib.s2tc_encode_layout_get.argtypes = [ctypes.POINTER(Options), c_uint, ctypes.POINTER(c_int),
                                           ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    lib.s2tc_encode_layout_get.restype = c_int
    lib.s2tc_dds_size.argtypes = [c_int, c_int, c_uint]
    lib.s2tc_dds_size.restype = c_ll
    lib.s2tc_compress_dds.argtypes = [vp, c_int, c_int, c_uint, ctypes.POINTER(Options), vp, c_ll,
                                      ctypes.POINTER(c_ll)]
    lib.s2tc_compress_dds.restype = c_int
    lib.s2tc_gpu_decode.argtypes = [vp, c_uint, c_int, c_int, vp, c_ll, c_int, vp]
    lib.s2tc_gpu_decode.restype = c_int
    lib.s2tc_decompress_dds.argtypes = [vp, c_ll, vp, c_ll, ctypes.POINTER(c_ll)]
    lib.s2tc_decompress_dds.restype = c_int
    lib.s2tc_gpu_from_s3tc.argtypes = [vp, vp, c_ll, c_uint, vp]
    lib.s2tc_gpu_from_s3tc.restype = c_int
    lib.s2tc_from_s3tc_dds.argtypes = [vp, c_ll, vp, c_ll, ctypes.POINTER(c_ll)]
    lib.s2tc_from_s3tc_dds.restype = c_int
    lib.s2tc_last_error.argtypes = []
    lib.s2tc_last_error.restype = ctypes.c_char_p
    if path is None:
        _lib = lib
    return lib


# Every exported symbol of the C ABI (include/s2tc_gb300.h).
EXPORTED_SYMBOLS = (
    "tx_compress_dxtn", "fetch_2d_texel_rgb_dxt1", "fetch_2d_texel_rgba_dxt1",
    "fetch_2d_texel_rgba_dxt3", "fetch_2d_texel_rgba_dxt5", "rgb565_image",
    "s2tc_encode_block_func", "s2tc_options_from_env", "s2tc_gpu_compress",
    "s2tc_gpu_synchronize", "s2tc_rand_words", "s2tc_gpu_set_timing", "s2tc_gpu_stage_ms",
    "s2tc_gpu_kernel_launches", "s2tc_test_dither_hold", "s2tc_gpu_compress_noalloc", "s2tc_batch_create", "s2tc_batch_run", "s2tc_gpu_compress_each",
    "s2tc_batch_kernels", "s2tc_batch_destroy", "s2tc_server_create", "s2tc_server_submit", "s2tc_server_submit_device",
    "s2tc_server_wait", "s2tc_server_stats", "s2tc_server_destroy",
    "s2tc_gpu_encode_blocks", "s2tc_autotune", "s2tc_encode_layout_set", "s2tc_encode_layout_get", "s2tc_dds_size", "s2tc_compress_dds", "s2tc_gpu_decode", "s2tc_decompress_dds",
    "s2tc_gpu_from_s3tc", "s2tc_from_s3tc_dds",
    "s2tc_last_error",
)


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(type(a))


def last_error() -> str:
    return load().s2tc_last_error().decode()


def options(dither=DITHER_SIMPLE, metric=WAVG, nrandom=-1, refine=REFINE_ALWAYS) -> Options:
    return Options(int(dither), int(metric), int(nrandom), int(refine))


def options_from_env() -> Options:
    o = Options()
    load().s2tc_options_from_env(ctypes.byref(o))
    return o


def set_env(dither=None, metric=None, nrandom=None, refine=None) -> None:
    """Set the S2TC_* environment knobs that tx_compress_dxtn reads (None
    removes a knob)."""
    for key, val, names in (("S2TC_DITHER_MODE", dither, DITHER_NAMES),
                            ("S2TC_COLORDIST_MODE", metric, COLORDIST_NAMES),
                            ("S2TC_RANDOM_COLORS", nrandom, None),
                            ("S2TC_REFINE_COLORS", refine, REFINE_NAMES)):
        if val is None:
            os.environ.pop(key, None)
        elif isinstance(val, str):
            os.environ[key] = val
        else:
            os.environ[key] = str(val) if names is None else names[int(val)]


def tx_compress_dxtn(srccomps: int, width: int, height: int, src, destformat: int,
                     dstRowStride: int = 0, dest: np.ndarray | None = None) -> np.ndarray:
    """Compress host pixels through the reference-compatible C entry point.

    ``src`` is a packed uint8 array (``width*height*srccomps`` bytes).  Returns
    the destination buffer (allocated packed unless ``dest`` is given)."""
    src = np.ascontiguousarray(src, dtype=np.uint8)
    if dest is None:
        dest = np.zeros(compressed_size(width, height, destformat) if destformat in FORMATS else 0, np.uint8)
    load().tx_compress_dxtn(srccomps, width, height, _ptr(src), destformat, _ptr(dest), dstRowStride)
    return dest


def rgb565_image(rgba, w: int, h: int, srccomps: int, alphabits: int, dither: int) -> np.ndarray:
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    out = np.zeros(w * h * 4, np.uint8)
    load().rgb565_image(_ptr(out), _ptr(rgba), w, h, srccomps, alphabits, dither)
    return out


_BLOCKFN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                            ctypes.c_int, ctypes.c_int)


def encode_block_func(dxt: int, cd: int, nrandom: int, refine: int):
    """``s2tc_encode_block_func``: returns f(out, rgba565, iw, w, h, nrandom)
    taking numpy arrays (``rgba565`` may be an offset view of a texel image)."""
    addr = load().s2tc_encode_block_func(dxt, cd, nrandom, refine)
    fn = _BLOCKFN(addr)

    def call(out: np.ndarray, rgba: np.ndarray, iw: int, w: int, h: int, nr: int) -> None:
        fn(_ptr(out), _ptr(rgba), iw, w, h, nr)

    return call


def fetch_texel(destformat: int, stride: int, data: np.ndarray, i: int, j: int) -> np.ndarray:
    lib = load()
    f = {GL_COMPRESSED_RGB_S3TC_DXT1_EXT: lib.fetch_2d_texel_rgb_dxt1,
         GL_COMPRESSED_RGBA_S3TC_DXT1_EXT: lib.fetch_2d_texel_rgba_dxt1,
         GL_COMPRESSED_RGBA_S3TC_DXT3_EXT: lib.fetch_2d_texel_rgba_dxt3,
         GL_COMPRESSED_RGBA_S3TC_DXT5_EXT: lib.fetch_2d_texel_rgba_dxt5}[destformat]
    t = np.zeros(4, np.uint8)
    f(stride, _ptr(data), i, j, _ptr(t))
    return t


def rand_words(width: int, height: int, destformat: int, opt: Options) -> int:
    return int(load().s2tc_rand_words(width, height, destformat, ctypes.byref(opt)))


def gpu_compress(srccomps: int, width: int, height: int, d_src, destformat: int, d_dst,
                 dst_pitch: int | None = None, opt: Options | None = None, d_rand=None,
                 stream: int | None = None) -> None:
    """Compress an image resident in device memory (torch CUDA tensors or raw
    device pointers) on ``stream`` (a raw cudaStream_t value; None = the
    library's stream)."""
    if dst_pitch is None:
        dst_pitch = ((width + 3) // 4) * block_bytes(destformat)
    opt = opt if opt is not None else options_from_env()
    src_p = d_src if isinstance(d_src, int) else _ptr(d_src)
    dst_p = d_dst if isinstance(d_dst, int) else _ptr(d_dst)
    rnd_p = None if d_rand is None else (d_rand if isinstance(d_rand, int) else _ptr(d_rand))
    st = load().s2tc_gpu_compress(srccomps, width, height, src_p, destformat, dst_p, dst_pitch,
                                  ctypes.byref(opt), rnd_p, stream)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_compress failed ({st}): {last_error()}")


def set_timing(enable: bool) -> None:
    st = load().s2tc_gpu_set_timing(1 if enable else 0)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_set_timing failed ({st}): {last_error()}")


def stage_ms() -> tuple[float, float, int]:
    """(dither_ms, encode_ms, calls): summed stage durations of the
    compressions since set_timing(True), from CUDA events recorded on their
    stream."""
    a, b, n = ctypes.c_float(), ctypes.c_float(), ctypes.c_longlong()
    st = load().s2tc_gpu_stage_ms(ctypes.byref(a), ctypes.byref(b), ctypes.byref(n))
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_stage_ms failed ({st}): {last_error()}")
    return a.value, b.value, n.value


def hold_dither_tile(hold_tile: int = -1, spin_limit: int = 0) -> None:
    """The timeout-path test hook (s2tc_test_dither_hold); (-1, 0) restores
    normal operation."""
    load().s2tc_test_dither_hold(int(hold_tile), int(spin_limit))


def kernel_launches() -> int:
    return int(load().s2tc_gpu_kernel_launches())


def gpu_compress_noalloc(srccomps: int, width: int, height: int, d_src, destformat: int, d_dst,
                         dst_pitch: int | None = None, opt: Options | None = None, d_rand=None,
                         stream: int | None = None) -> int:
    """``s2tc_gpu_compress_noalloc``: like gpu_compress, but the library
    allocates nothing (scratch in a fixed device array, images up to 4 Mi
    texels; returns when done).  For callers that cannot allocate device
    memory.  Returns the status code."""
    if dst_pitch is None:
        dst_pitch = ((width + 3) // 4) * block_bytes(destformat)
    opt = opt if opt is not None else options_from_env()
    src_p = d_src if isinstance(d_src, int) else _ptr(d_src)
    dst_p = d_dst if isinstance(d_dst, int) else _ptr(d_dst)
    rnd_p = None if d_rand is None else (d_rand if isinstance(d_rand, int) else _ptr(d_rand))
    return int(load().s2tc_gpu_compress_noalloc(srccomps, width, height, src_p, destformat, dst_p, dst_pitch,
                                                ctypes.byref(opt), rnd_p, stream))


def image_array(images):
    """ctypes array of ``Image`` from dicts (see ``Batch``)."""
    arr = (Image * max(1, len(images)))()
    for i, im in enumerate(images):
        w, h, fmt = int(im["width"]), int(im["height"]), int(im["format"])
        pitch = im.get("dst_pitch") or ((w + 3) // 4) * block_bytes(fmt)
        rnd = im.get("rand")
        arr[i] = Image(_addr(im["src"]), w, h, int(im["srccomps"]), fmt, _addr(im["dst"]), int(pitch),
                       None if rnd is None else _addr(rnd))
    return arr


def gpu_compress_each(images, opt: Options, stream: int | None = None, arr=None) -> None:
    """``s2tc_gpu_compress_each``: one image at a time, each with its own
    launches (pass a prebuilt ``image_array`` as ``arr`` to skip conversion)."""
    arr = arr if arr is not None else image_array(images)
    st = load().s2tc_gpu_compress_each(arr, len(images), ctypes.byref(opt), stream)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_compress_each failed ({st}): {last_error()}")


class Batch:
    """A planned batch (``s2tc_batch_create``): images of uneven sizes and
    mixed formats encoded by one CUDA-graph launch per ``run``.

    ``images`` is a list of dicts with keys src, width, height, srccomps,
    format, dst and optionally dst_pitch and rand (device tensors or raw
    pointers)."""

    def __init__(self, images, opt: Options):
        arr = image_array(images)
        self._keep = list(images)
        self._opt = opt
        h = ctypes.c_void_p()
        st = load().s2tc_batch_create(ctypes.byref(h), arr, len(images), ctypes.byref(opt))
        if st != S2TC_OK:
            raise S2tcError(f"s2tc_batch_create failed ({st}): {last_error()}")
        self.handle = h

    @property
    def kernels(self) -> int:
        return int(load().s2tc_batch_kernels(self.handle))

    def run(self, stream: int | None = None) -> None:
        st = load().s2tc_batch_run(self.handle, stream)
        if st != S2TC_OK:
            raise S2tcError(f"s2tc_batch_run failed ({st}): {last_error()}")

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().s2tc_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """``s2tc_server_*``: a continuous-batching request loop under a device
    memory budget.  ``submit`` takes host buffers (numpy arrays or torch CPU
    tensors; pinned ones let copies overlap) and returns an id; ``wait``
    returns the latency in milliseconds."""

    def __init__(self, budget_bytes: int):
        h = ctypes.c_void_p()
        st = load().s2tc_server_create(ctypes.byref(h), int(budget_bytes))
        if st != S2TC_OK:
            raise S2tcError(f"s2tc_server_create failed ({st}): {last_error()}")
        self.handle = h
        self._keep = {}

    def submit(self, src, srccomps: int, width: int, height: int, fmt: int, opt: Options, dst,
               dst_pitch: int = 0) -> int:
        rid = ctypes.c_longlong()
        st = load().s2tc_server_submit(self.handle, _addr(src), srccomps, width, height, fmt, ctypes.byref(opt),
                                       _addr(dst), dst_pitch, ctypes.byref(rid))
        if st != S2TC_OK:
            raise S2tcError(f"s2tc_server_submit failed ({st})")
        self._keep[rid.value] = (src, dst)
        return rid.value

    def submit_device(self, d_src, srccomps: int, width: int, height: int, fmt: int, opt: Options, d_dst,
                      dst_pitch: int = 0) -> int:
        rid = ctypes.c_longlong()
        st = load().s2tc_server_submit_device(self.handle, _addr(d_src), srccomps, width, height, fmt,
                                              ctypes.byref(opt), _addr(d_dst), dst_pitch, ctypes.byref(rid))
        if st != S2TC_OK:
            raise S2tcError(f"s2tc_server_submit_device failed ({st})")
        self._keep[rid.value] = (d_src, d_dst)
        return rid.value

    def wait(self, rid: int) -> float:
        lat = ctypes.c_double()
        st = load().s2tc_server_wait(self.handle, rid, ctypes.byref(lat))
        self._keep.pop(rid, None)
        if st != S2TC_OK:
            raise S2tcError(f"request {rid} failed ({st})")
        return lat.value

    def stats(self) -> dict:
        r, d, hw = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        mi, mr = ctypes.c_int(), ctypes.c_int()
        load().s2tc_server_stats(self.handle, ctypes.byref(r), ctypes.byref(d), ctypes.byref(mi), ctypes.byref(mr),
                                 ctypes.byref(hw))
        return {"rounds": r.value, "done": d.value, "max_inflight_rounds": mi.value,
                "max_round_requests": mr.value, "pool_high_water": hw.value}

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().s2tc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gpu_encode_blocks(d_t565, width: int, height: int, dxt: int, colordist: int, nrandom: int, refine: int, d_dst,
                      dst_pitch: int = 0, d_rand=None, stream: int | None = None) -> None:
    """``s2tc_gpu_encode_blocks``: the per-block encoder over a texel-word image."""
    if dst_pitch == 0:
        dst_pitch = ((width + 3) // 4) * (8 if dxt == 0 else 16)
    st = load().s2tc_gpu_encode_blocks(_addr(d_t565), width, height, dxt, colordist, nrandom, refine, _addr(d_dst),
                                       dst_pitch, None if d_rand is None else _addr(d_rand), stream)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_encode_blocks failed ({st}): {last_error()}")


def autotune(opt: Options, fmt: int, width: int = 1024, height: int = 1024) -> float:
    """``s2tc_autotune``: keeps the fastest launch layout for this mode;
    returns its encoder time in ms."""
    ms = ctypes.c_float()
    st = load().s2tc_autotune(ctypes.byref(opt), fmt, width, height, ctypes.byref(ms))
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_autotune failed ({st}): {last_error()}")
    return ms.value


def set_layout(opt: Options, fmt: int, threads: int = 128, rand_warps: int = 4, rand_ctas_per_sm: int = 64) -> None:
    st = load().s2tc_encode_layout_set(ctypes.byref(opt), fmt, threads, rand_warps, rand_ctas_per_sm)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_encode_layout_set failed ({st}): {last_error()}")


def get_layout(opt: Options, fmt: int) -> dict:
    t, w, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    load().s2tc_encode_layout_get(ctypes.byref(opt), fmt, ctypes.byref(t), ctypes.byref(w), ctypes.byref(c))
    return {"threads": t.value, "rand_warps": w.value, "rand_ctas_per_sm": c.value}


# ------------------------------------------------------- the reference's tools

def dds_size(width: int, height: int, fmt: int) -> int:
    return int(load().s2tc_dds_size(width, height, fmt))


def compress_dds(rgba, width: int, height: int, fmt: int, opt: Options | None = None) -> bytes:
    """``s2tc_compress_dds``: the DDS file s2tc_compress writes for an RGBA8
    image (every mip level to 1x1).  ``opt`` None reads the S2TC_* env."""
    src = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(-1)
    n = dds_size(width, height, fmt)
    if n < 0:
        raise S2tcError("bad format or size")
    out = np.zeros(n, np.uint8)
    written = ctypes.c_longlong()
    st = load().s2tc_compress_dds(_ptr(src), width, height, fmt, ctypes.byref(opt) if opt is not None else None,
                                  _ptr(out), n, ctypes.byref(written))
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_compress_dds failed ({st}): {last_error()}")
    return out[: written.value].tobytes()


def gpu_decode(d_blocks, fmt: int, width: int, height: int, d_out, dst_pitch: int = 0, bgra: bool = False,
               stream: int | None = None) -> None:
    st = load().s2tc_gpu_decode(_addr(d_blocks), fmt, width, height, _addr(d_out), dst_pitch, int(bgra), stream)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_decode failed ({st})")


def decompress_dds(dds: bytes) -> bytes:
    """``s2tc_decompress_dds``: the TGA s2tc_decompress writes."""
    src = np.frombuffer(dds, np.uint8).copy()
    w = int.from_bytes(dds[16:20], "little") if len(dds) >= 20 else 0
    h = int.from_bytes(dds[12:16], "little") if len(dds) >= 16 else 0
    out = np.zeros(18 + 4 * max(0, w) * max(0, h), np.uint8)
    written = ctypes.c_longlong()
    st = load().s2tc_decompress_dds(_ptr(src), src.size, _ptr(out), out.size, ctypes.byref(written))
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_decompress_dds failed ({st})")
    return out[: written.value].tobytes()


def gpu_from_s3tc(d_src, d_dst, nblocks: int, fmt: int, stream: int | None = None) -> None:
    st = load().s2tc_gpu_from_s3tc(_addr(d_src), _addr(d_dst), nblocks, fmt, stream)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_from_s3tc failed ({st})")


def from_s3tc_dds(dds: bytes) -> bytes:
    """``s2tc_from_s3tc_dds``: the file s2tc_from_s3tc writes."""
    src = np.frombuffer(dds, np.uint8).copy()
    out = np.zeros(max(128, src.size), np.uint8)
    written = ctypes.c_longlong()
    st = load().s2tc_from_s3tc_dds(_ptr(src), src.size, _ptr(out), out.size, ctypes.byref(written))
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_from_s3tc_dds failed ({st})")
    return out[: written.value].tobytes()


def _addr(x) -> int:
    return x if isinstance(x, int) else _ptr(x)


def gpu_synchronize(stream: int | None = None) -> None:
    st = load().s2tc_gpu_synchronize(stream)
    if st != S2TC_OK:
        raise S2tcError(f"s2tc_gpu_synchronize failed ({st}): {last_error()}")
