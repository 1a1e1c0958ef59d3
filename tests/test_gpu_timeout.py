"""The timeout path of the SIMPLE dither's bounded waits.

Every wait in the dither scan (a tile's look-back at the tiles before it) is
bounded; when one gives up, the kernel sets an error flag and finishes, and
the call reports S2TC_ERR_TIMEOUT instead of hanging.  These tests make one
wait run out on purpose through the library's test hook
(s2tc_test_dither_hold): one tile never publishes its scan state and the
look-back limit is cut to 1024 polls, so the tiles behind it give up within a
millisecond or so.  Nothing faults or spins without a limit.  After the hook
is cleared, the next call must give the oracle's bytes again."""
import numpy as np
import pytest

import pyoracle
import s2tc_gb300 as s2
from s2tc_gb300 import workloads

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # S2TC_ERR_TIMEOUT


def test_device_call_reports_timeout_then_recovers(lib, oracle):
    torch = pytest.importorskip("torch")
    w, h, fmt = 512, 512, 0x83F1  # 16 dither tiles
    img = workloads.plain_rgba(9, w, h).reshape(-1)
    opt = s2.options(1, s2.WAVG, -1, 1)
    d_src = torch.from_numpy(img.copy()).cuda()
    d_dst = torch.zeros(s2.compressed_size(w, h, fmt), dtype=torch.uint8, device="cuda")
    s2.gpu_synchronize()  # no stale flag from earlier tests
    try:
        s2.hold_dither_tile(5, 1024)
        s2.gpu_compress(4, w, h, d_src, fmt, d_dst, opt=opt)
        st = lib.s2tc_gpu_synchronize(None)
    finally:
        s2.hold_dither_tile(-1, 0)
    assert st == TIMEOUT
    assert "bounded wait" in s2.last_error()
    # the flag was consumed by that report; the next call is exact again
    s2.gpu_compress(4, w, h, d_src, fmt, d_dst, opt=opt)
    s2.gpu_synchronize()
    want = oracle.compress(4, w, h, img, fmt, 1, s2.WAVG, -1, 1)
    assert np.array_equal(d_dst.cpu().numpy(), want)


@pytest.mark.parametrize("nrandom,w,hold", [(-1, 4096, 300), (0, 2048, 30)])
def test_pipelined_host_call_reports_timeout_then_recovers(lib, oracle, nrandom, w, hold):
    """tx_compress_dxtn on the large-image paths.  The quick mode (nrandom -1,
    4096x2048) runs the fused strip kernel over 512 bands of one block row:
    in one launch that reads host memory where the GPU reads it coherently,
    else in two ranges of 256 as the image goes up; the all-texel search
    (nrandom 0, 2048x2048) runs the dither over 253 tiles of 16640 texels in
    ranges of 16, 32, 64 and 141 as the image goes up.  The held band or tile
    sits in the second half or range, so waits across a range boundary give
    up too."""
    h, fmt = 2048, 0x83F1
    img = workloads.plain_rgba(10, w, h).reshape(-1)
    s2.set_env(1, s2.WAVG, nrandom, 1)
    try:
        s2.hold_dither_tile(hold, 1024)
        s2.tx_compress_dxtn(4, w, h, img, fmt)
        err = s2.last_error()
    finally:
        s2.hold_dither_tile(-1, 0)
    assert "bounded wait" in err
    pyoracle.srand(1)
    got = s2.tx_compress_dxtn(4, w, h, img, fmt)
    want = oracle.compress(4, w, h, img, fmt, 1, s2.WAVG, nrandom, 1)
    assert np.array_equal(got, want)
