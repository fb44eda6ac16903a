"""Golden NLPAR file runs: the reference's ``NLPAR.calcnlpar_cpu`` on small UP1 scans.

Run from the repository root on a machine that has the reference source tree:

    python tests/golden/make_nlpar_file_golden.py   # writes tests/golden/nlparfile/*

Each case writes a seeded scan of synthetic patterns with the reference's ``UPFile`` writer, runs
the reference's ``NLPAR(file).calcnlpar_cpu`` (nlpar_cpu.py:283-540, imported through
``oracle/refshim.py``) into an output file, and keeps the input file, the output file and the
parameters (``<name>.json``) -- one case in one scan tile, one in several.
"""
from __future__ import annotations

import json
import os
import sys
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nlparfile")

from oracle import refshim  # noqa: E402
from pyebsdindex_gb300 import synthetic as syn  # noqa: E402

CASES = {
    # name: (nrows, ncols, pattern size, search radius, lambda, chunksize bytes, seed)
    "onetile_9x11_16": (9, 11, 16, 2, 0.9, 0, 7),
    "tiles_10x12_16": (10, 12, 16, 2, 0.8, 60_000, 8),
}


def main():
    ref = refshim.load()
    rp = refshim.pattern_module()
    os.makedirs(OUT, exist_ok=True)
    for name, (nrows, ncols, h, sr, lam, chunk, seed) in CASES.items():
        pats = syn.make_patterns(nrows * ncols, h, h, seed=seed, noise_frac=0.1)[0]
        src = os.path.join(OUT, name + "_in.up1")
        dst = os.path.join(OUT, name + "_out.up1")
        for p in (src, dst):
            if os.path.exists(p):
                os.remove(p)
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            f = rp.UPFile(src)
            f.version, f.patternW, f.patternH = 3, h, h
            f.nCols, f.nRows, f.nPatterns, f.xStep, f.yStep = ncols, nrows, nrows * ncols, 1.0, 1.0
            f.extraPatterns, f.hexflag, f.filedatatype = 0, 0, np.uint8
            f.write_data(newpatterns=pats, patStartCount=[0, -1], writeHead=True)
            nl = ref.nlpar_cpu.NLPAR(src, lam=lam, searchradius=sr)
            nl.calcnlpar_cpu(chunksize=chunk, fileout=dst, verbose=0)
        with open(os.path.join(OUT, name + ".json"), "w") as fh:
            json.dump({"nrows": nrows, "ncols": ncols, "h": h, "searchradius": sr, "lam": lam, "chunksize": chunk},
                      fh)
        np.save(os.path.join(OUT, name + "_sigma.npy"), np.asarray(nl.sigma, np.float32))
        print(name, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
