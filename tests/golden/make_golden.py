"""Generate tests/golden/s2tc_golden.npz from the reference encoder compiled
from its own sources (oracle/Makefile target `ref`).

    make -C oracle ref && python tests/golden/make_golden.py

Each case stores its parameters, the input pixels and the reference's output
bytes; rand() is seeded with the stored seed right before the reference call.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1] / "oracle"))

import cases  # noqa: E402
import pyoracle  # noqa: E402

OUT = HERE / "s2tc_golden.npz"


def main() -> None:
    ref = pyoracle.Reference()
    params, ins, outs = [], [], []

    def add(w, h, sc, fmt, dither, metric, nr, refine, img, seed, stride=0):
        if cases.is_unpinned_corner(w, h, fmt, metric, nr):
            return
        out = ref.compress(sc, w, h, img, fmt, dither, metric, nr, refine, seed=seed)
        params.append((w, h, sc, fmt, dither, metric, nr, refine, seed, stride))
        ins.append(np.asarray(img, np.uint8))
        outs.append(out)

    # every mode combination on small random images
    rng = np.random.default_rng(2024)
    for fmt in cases.FORMATS:
        for metric in range(8):
            for refine in range(3):
                for nr in (-1, 0, 3):
                    w, h = int(rng.integers(1, 13)), int(rng.integers(1, 13))
                    sc = int(rng.choice([3, 4]))
                    add(w, h, sc, fmt, int(rng.integers(0, 3)), metric, nr, refine,
                        cases.image(rng, w, h, sc), int(rng.integers(1, 1 << 30)))
    # random sweep
    for c in cases.random_cases(7, 300):
        add(*c)
    # a few larger images per format and selection mode
    for fmt in cases.FORMATS:
        for metric, nr, refine in ((5, -1, 1), (3, 0, 2), (7, 2, 2), (2, 0, 0)):
            w, h = int(rng.integers(30, 70)), int(rng.integers(30, 70))
            add(w, h, 4, fmt, int(rng.integers(0, 3)), metric, nr, refine, cases.image(rng, w, h, 4, 0),
                int(rng.integers(1, 1 << 30)))

    # dither goldens (rgb565_image)
    d_params, d_in, d_out = [], [], []
    for dither in range(3):
        for sc in (3, 4):
            for ab in (1, 4, 8):
                for _ in range(4):
                    w, h = int(rng.integers(1, 40)), int(rng.integers(1, 40))
                    img = cases.image(rng, w, h, sc)
                    d_params.append((w, h, sc, ab, dither))
                    d_in.append(img)
                    d_out.append(ref.rgb565_image(img, w, h, sc, ab, dither))

    def pack(arrs):
        off = np.cumsum([0] + [len(a) for a in arrs]).astype(np.int64)
        return off, (np.concatenate(arrs) if arrs else np.zeros(0, np.uint8))

    in_off, in_data = pack(ins)
    out_off, out_data = pack(outs)
    d_in_off, d_in_data = pack(d_in)
    d_out_off, d_out_data = pack(d_out)
    np.savez_compressed(OUT, params=np.array(params, np.int64), in_off=in_off, in_data=in_data,
                        out_off=out_off, out_data=out_data, d_params=np.array(d_params, np.int64),
                        d_in_off=d_in_off, d_in_data=d_in_data, d_out_off=d_out_off, d_out_data=d_out_data)
    print(f"{OUT}: {len(params)} encode cases, {len(d_params)} dither cases, {OUT.stat().st_size} bytes")


if __name__ == "__main__":
    main()
