"""NLPAR lambda optimisation, CPU side: the oracle (oracle/nlpar_oracle.py) against the
reference's own opt_lambda_cpu outputs (tests/golden/nlparlam_*.npz, made by
tests/golden/make_nlpar_lambda_golden.py), and the scan tiling restated in the package
(nlpar.scan_tiles) against the oracle's and the reference's NLPAR._calcchunks."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from oracle import nlpar_oracle as no

CASES = ("nlparlam_16x20_40", "nlparlam_12x14_32_dt")


def load(name):
    d = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    return d, json.loads(str(d["params"]))


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_sigma_distances_and_lambda(name):
    d, p = load(name)
    ind = np.asarray(d["mask"].flatten().nonzero()[0], np.int64)
    sig, d2, n2 = no.calcsigma_chunked(d["data"], p["nrows"], p["ncols"], p["h"], p["w"], ind,
                                       p["saturation_protect"], 2e9)
    assert sig.tobytes() == d["sigma"].tobytes()
    assert n2.tobytes() == d["n2"].tobytes()
    assert d2.tobytes() == d["d2"].tobytes()
    # the reference's uint64 window arithmetic: row 0 and column 0 of every tile have no window
    assert np.all(n2[0] == 0) and np.all(n2[:, 0] == 0) and np.all(sig[0] == np.float32(1e12))
    lam = no.opt_lambda(d2, sig.size, p["target_weights"], p["dthresh"])
    assert np.array_equal(lam, d["lam"])


def test_scan_tiles_match_the_oracle():
    from pyebsdindex_gb300.nlpar import scan_tiles
    rng = np.random.default_rng(0)
    for _ in range(2000):
        nr, nc = int(rng.integers(2, 500)), int(rng.integers(2, 500))
        h = int(rng.integers(16, 160))
        tb = float(rng.choice([1e5, 1e6, 1e7, 2e9, 8e9]))
        a = no.calcchunks([h, h], nc, nr, tb, 1, 1)
        b = scan_tiles([h, h], nc, nr, tb, 1, 1)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (nr, nc, h, tb)


def test_scan_tiles_match_the_reference():
    from oracle import refshim
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    ref = refshim.load()
    N = ref.nlpar_cpu.NLPAR()
    rng = np.random.default_rng(1)
    for _ in range(500):
        nr, nc = int(rng.integers(2, 500)), int(rng.integers(2, 500))
        h = int(rng.integers(16, 160))
        tb = float(rng.choice([1e5, 1e6, 1e7, 2e9]))
        want = N._calcchunks([h, h], nc, nr, target_bytes=tb, col_overlap=1, row_overlap=1)
        cols, rows = no.calcchunks([h, h], nc, nr, tb, 1, 1)
        assert np.array_equal(cols, want[2]) and np.array_equal(rows, want[3]), (nr, nc, h, tb)
