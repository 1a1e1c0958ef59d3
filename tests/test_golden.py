"""The oracle against the committed golden vectors (made by the reference
encoder compiled from its sources; tests/golden/make_golden.py)."""
import numpy as np

from golden import golden


def test_encode_golden(oracle):
    n = 0
    for c in golden.encode_cases():
        out = oracle.compress(c["sc"], c["w"], c["h"], c["src"], c["fmt"], c["dither"], c["metric"],
                              c["nrandom"], c["refine"], dst_row_stride=c["stride"], seed=c["seed"])
        assert np.array_equal(out, c["out"]), {k: v for k, v in c.items() if k not in ("src", "out")}
        n += 1
    assert n > 500


def test_dither_golden(oracle):
    for c in golden.dither_cases():
        out = oracle.rgb565_image(c["src"], c["w"], c["h"], c["sc"], c["alphabits"], c["dither"])
        assert np.array_equal(out, c["out"]), {k: v for k, v in c.items() if k not in ("src", "out")}


def test_explicit_rand_words_equal_libc_stream(oracle):
    """The oracle fed the random candidates' words from an array gives the
    bytes it gives when it calls libc's rand() itself, given the same words
    (the form the batched GPU bench outputs are checked in)."""
    import cases
    import pyoracle
    rng = np.random.default_rng(5)
    for i in range(60):
        w, h = int(rng.integers(1, 21)), int(rng.integers(1, 21))
        sc = int(rng.choice([3, 4]))
        fmt = int(rng.choice(cases.FORMATS))
        nr = int(rng.choice([1, 5, 64]))
        metric, refine, dither = int(rng.integers(0, 8)), int(rng.integers(0, 3)), int(rng.integers(0, 3))
        img = cases.image(rng, w, h, sc)
        nwords = ((w + 3) // 4) * ((h + 3) // 4) * nr * (4 if fmt == 0x83F3 else 3)
        pyoracle.srand(900 + i)
        words = np.array([pyoracle.libc_rand() for _ in range(nwords)], np.uint32)
        want = oracle.compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed=900 + i)
        got = oracle.compress(sc, w, h, img, fmt, dither, metric, nr, refine, rand_words=words)
        assert np.array_equal(got, want), (w, h, sc, hex(fmt), nr, metric, refine)
    import pytest
    with pytest.raises(ValueError):
        oracle.compress(4, 8, 8, np.zeros(256, np.uint8), 0x83F1, 1, 5, 4, 1, rand_words=np.zeros(3, np.uint32))
