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
