"""Golden vectors for NLPAR's lambda optimisation: the reference's ``NLPAR.opt_lambda_cpu``.

Run from the repository root on a machine that has the reference source tree:

    python tests/golden/make_nlpar_lambda_golden.py      # writes tests/golden/nlparlam_*.npz

A seeded Voronoi scan (the NLPAR configuration's generator, smaller grid) is served to the
reference's ``NLPAR`` through an in-memory stand-in for its pattern-file object (the
``read_header`` / ``read_data`` calls ``calcsigma_cpu`` makes, nlpar_cpu.py:224-260), and
``opt_lambda_cpu`` (nlpar_cpu.py:94-155: ``sigma_numba`` with nn = 1 and its normalised
neighbour distances, then a bounded Nelder-Mead per target weight) runs unchanged.  Stored:
the patterns, the mask, sigma, the normalised distances d2 and counts n2 [nrows, ncols, 9],
and the three lambda values.
"""
from __future__ import annotations

import json
import os
import sys
import time
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.dirname(os.path.abspath(__file__))

from oracle import refshim  # noqa: E402
from pyebsdindex_gb300 import synthetic as syn  # noqa: E402

CASES = {
    # name: (nrows, ncols, h, w, dthresh, saturation_protect, saturate, seed)
    "nlparlam_16x20_40": (16, 20, 40, 40, 0.0, True, False, 41),
    "nlparlam_12x14_32_dt": (12, 14, 32, 32, 0.4, False, True, 42),
}


class MemoryPatterns:
    """The pattern-file calls NLPAR's sigma estimate makes, served from an array."""

    def __init__(self, pats):
        self.pats = pats
        self.nRows, self.nCols, self.patternH, self.patternW = pats.shape
        self.datamin = float(pats.min())

    def read_header(self):
        return None

    def read_data(self, patStartCount=None, convertToFloat=False, returnArrayOnly=False, **kw):
        (c0, r0), (nc, nr) = patStartCount
        d = self.pats[r0:r0 + nr, c0:c0 + nc].reshape(-1, self.patternH, self.patternW)
        return (d.astype(np.float32) if convertToFloat else d), None


def make_case(ref, name, nrows, ncols, h, w, dthresh, satp, saturate, seed):
    pats, _ = syn.voronoi_scan(nrows, ncols, ngrains=max(3, nrows * ncols // 12), h=h, w=w, seed=seed)
    if saturate:
        pats[::5, h // 2, :] = 255
    grid = pats.reshape(nrows, ncols, h, w)
    N = ref.nlpar_cpu.NLPAR(lam=0.7, searchradius=3, dthresh=dthresh, saturation_protect=satp,
                            nrows=nrows, ncols=ncols)
    mem = MemoryPatterns(grid)
    N.getinfileobj = lambda: mem
    seen = {}
    real = N.calcsigma_cpu

    def capture(**kw):
        out = real(**kw)
        seen["sigma"], seen["d2"], seen["n2"] = out
        return out

    N.calcsigma_cpu = capture
    t0 = time.time()
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        lam = N.opt_lambda_cpu(target_weights=(0.5, 0.34, 0.25), autoupdate=True, verbose=0)
    rec = dict(data=pats.reshape(nrows * ncols, h * w).astype(np.float32), mask=N.mask, sigma=seen["sigma"],
               d2=seen["d2"], n2=seen["n2"], lam=np.asarray(lam, np.float64), lam_opt=np.float64(N.lam),
               params=json.dumps(dict(nrows=nrows, ncols=ncols, h=h, w=w, dthresh=dthresh,
                                      saturation_protect=satp, target_weights=[0.5, 0.34, 0.25])))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(f"{name}: lambda {np.asarray(lam)} in {time.time() - t0:.1f}s")


def main():
    ref = refshim.load()
    for name, args in CASES.items():
        make_case(ref, name, *args)


if __name__ == "__main__":
    main()
