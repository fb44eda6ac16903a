"""Band records of this repository's GPU methods on the orientation fixture's patterns.

Run from the repository root on a machine with a CUDA GPU and the built library:

    python tests/golden/make_gpu_records.py [out.npz]     # default tests/golden/orient_80x80_gpu.npz

Reads ``tests/golden/orient_80x80.npz`` (made by ``make_orientation_golden.py``), detects its
patterns with the plan this host builds (the product's own Radon table) and stores, per
method, every band-record field the indexer reads.  ``tests/test_orientation_agreement.py`` indexes these with the reference's
triplet voting.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))

FIELDS = ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")
METHODS = ("fused", "plain", "plain64", "fused16")


def main():
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import synthetic as syn
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "orient_80x80_gpu.npz")
    fx = np.load(os.path.join(HERE, "orient_80x80.npz"))
    p = json.loads(str(fx["params"]))
    bd = pg.BandDetect(**p)
    bd.band_detect_setup(patDim=(80, 80), patternmask=syn.circular_mask(80, 80))
    rec = {}
    for m in METHODS:
        r = bd.find_bands(fx["patterns"], method=m)
        for f in FIELDS:
            rec[m + "_" + f] = r[f]
    np.savez_compressed(out, **rec)
    print(out)


if __name__ == "__main__":
    main()
