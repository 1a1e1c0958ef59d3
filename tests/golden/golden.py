"""Reader for tests/golden/s2tc_golden.npz (see make_golden.py)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

PATH = Path(__file__).resolve().parent / "s2tc_golden.npz"


def encode_cases():
    z = np.load(PATH)
    p, io, idata, oo, odata = z["params"], z["in_off"], z["in_data"], z["out_off"], z["out_data"]
    for k in range(len(p)):
        w, h, sc, fmt, dither, metric, nr, refine, seed, stride = (int(v) for v in p[k])
        yield dict(w=w, h=h, sc=sc, fmt=fmt, dither=dither, metric=metric, nrandom=nr, refine=refine,
                   seed=seed, stride=stride, src=idata[io[k]:io[k + 1]], out=odata[oo[k]:oo[k + 1]])


def dither_cases():
    z = np.load(PATH)
    p, io, idata, oo, odata = z["d_params"], z["d_in_off"], z["d_in_data"], z["d_out_off"], z["d_out_data"]
    for k in range(len(p)):
        w, h, sc, ab, dither = (int(v) for v in p[k])
        yield dict(w=w, h=h, sc=sc, alphabits=ab, dither=dither, src=idata[io[k]:io[k + 1]],
                   out=odata[oo[k]:oo[k + 1]])
