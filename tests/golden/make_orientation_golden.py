"""Golden vectors for the downstream check: orientations indexed from band records.

Run from the repository root on a machine that has the reference source tree:

    python tests/golden/make_orientation_golden.py          # writes tests/golden/orient_80x80.npz

200 seeded synthetic 80x80 uint8 patterns (the batched configuration's generator: FCC bands,
PC (0.46, 0.70, 0.64), Poisson noise at 200 counts, circular mask, 10% noise-only) go through
the reference's own CPU ``BandDetect.find_bands`` (band_detect.py:411-526, imported through
``oracle/refshim.py``, run in spawned worker processes) and then through the reference's
``EBSDIndexer.index_pats`` (_ebsd_index_single.py:466) with that band-detect plan returning
those records, so triplet voting (tripletvote.py) turns them into orientations.  Stored:
the patterns, the reference's records and its quaternion / fit / nmatch per pattern.

``tests/golden/make_gpu_records.py`` then runs this repository's GPU band detection on the
same patterns (on a GPU machine), and ``tests/test_orientation_agreement.py`` indexes those
records with the reference's voting and compares the orientations.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "orient_80x80.npz")
PARAMS = dict(nTheta=180, nRho=120, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=9)
PC = (0.46, 0.70, 0.64)
N, SEED = 200, 7000


def make_indexer(ref):
    from pyebsdindex_gb300 import synthetic as syn
    idx = ref.ebsd_index_single.EBSDIndexer(PC=PC, patDim=(80, 80), **PARAMS)
    idx.bandDetectPlan.band_detect_setup(patDim=(80, 80), patternmask=syn.circular_mask(80, 80))
    return idx


def index_records(ref, idx, pats, records):
    """Reference index_pats with its band-detect plan returning ``records``."""
    bd = idx.bandDetectPlan
    saved = bd.find_bands
    bd.find_bands = lambda *a, **k: records.copy()
    try:
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            data = idx.index_pats(pats)[0]
    finally:
        bd.find_bands = saved
    return data[-1]


def _worker(args):
    lo, hi = args
    from oracle import refshim
    from pyebsdindex_gb300 import synthetic as syn
    ref = refshim.load()
    idx = make_indexer(ref)
    pats = syn.make_patterns(N, 80, 80, seed=SEED, noise_frac=0.1)[0][lo:hi]
    return lo, refshim.find_bands(idx.bandDetectPlan, pats)


def main():
    from oracle import refshim
    from pyebsdindex_gb300 import synthetic as syn
    ref = refshim.load()
    pats, quats, noise = syn.make_patterns(N, 80, 80, seed=SEED, noise_frac=0.1)
    t0 = time.time()
    nproc = min(8, os.cpu_count() or 1)
    bounds = [(i * N // nproc, (i + 1) * N // nproc) for i in range(nproc)]
    with mp.get_context("spawn").Pool(nproc) as pool:
        parts = pool.map(_worker, bounds)
    parts.sort(key=lambda x: x[0])
    recs = np.concatenate([r for _, r in parts])
    idx = make_indexer(ref)
    res = index_records(ref, idx, pats, recs)
    rec = {"patterns": pats, "noise_only": noise, "true_quat": quats,
           "params": np.array(json.dumps(PARAMS)), "pc": np.asarray(PC),
           "ref_quat": res["quat"], "ref_fit": res["fit"], "ref_nmatch": res["nmatch"],
           "ref_phase": res["phase"]}
    for f in ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
        rec["ref_" + f] = recs[f]
    np.savez_compressed(OUT, **rec)
    print(f"{OUT}: {N} patterns in {time.time() - t0:.1f}s; indexed (nmatch >= 3): "
          f"{int((res['nmatch'] >= 3).sum())}")


if __name__ == "__main__":
    main()
