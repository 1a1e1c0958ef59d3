"""Arithmetic restated for the GPU kernels, checked exhaustively on the CPU.

The kernels take the reference's rounded mean ((s << 1) + n) / (n << 1)
(s2tc_algorithm.cpp:542-551) in float (s2tc_gb300/csrc/s2tc_device.cuh,
`rmean`): floor(fma(float(2s + n), rcp_rn(float(2n)), 2^-6)).  Here the same
operations are emulated with exact float32 rounding (the product of a 13-bit
integer and a float32 and the added 2^-6 are exact in float64, so one
float64 -> float32 conversion is the fused multiply-add's single rounding) and
compared with the integer division over the whole domain the kernels use it
on: 1 <= n <= 16 texels, 0 <= s <= 16 * 255."""
import numpy as np


def test_rmean_float_form_is_exact():
    n = np.arange(1, 17, dtype=np.int64)[:, None]
    s = np.arange(0, 16 * 255 + 1, dtype=np.int64)[None, :]
    x = 2 * s + n
    want = x // (2 * n)
    rcp = (np.float32(1.0) / (2 * n).astype(np.float32)).astype(np.float32)  # correctly rounded
    fma = (x.astype(np.float64) * rcp.astype(np.float64) + 2.0 ** -6).astype(np.float32)
    got = np.floor(fma).astype(np.int64)
    assert np.array_equal(got, want)
