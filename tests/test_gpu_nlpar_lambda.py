"""NLPAR lambda optimisation on the device (ebsd_nlpar_sigma_tile, ebsd_nlpar_lambda_metric,
NLPAR.opt_lambda_array) against the reference's own opt_lambda_cpu outputs
(tests/golden/nlparlam_*.npz) and the oracle.  sigma, the normalised distances and counts are
float32 in the reference's operation order and must be bit-identical; the objective is
float64 with CUDA's exp (numpy's is its own SIMD exp) and a fixed-order block sum: within
1e-12 relative of the oracle; the lambda values within 1e-6 relative of the reference's."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from oracle import nlpar_oracle as no

pytestmark = pytest.mark.gpu
CASES = ("nlparlam_16x20_40", "nlparlam_12x14_32_dt")


def load(name):
    d = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    return d, json.loads(str(d["params"]))


def make(p):
    from pyebsdindex_gb300 import NLPAR
    return NLPAR(lam=0.7, searchradius=3, dthresh=p["dthresh"], saturation_protect=p["saturation_protect"])


@pytest.mark.parametrize("name", CASES)
def test_tile_sigma_and_distances_bit_exact(cuda, name):
    d, p = load(name)
    nl = make(p)
    pats = d["data"].reshape(p["nrows"] * p["ncols"], p["h"], p["w"])
    sig, d2, n2 = nl.calcsigma_tiles_array(pats, p["nrows"], p["ncols"], target_bytes=2e9)
    assert sig.tobytes() == d["sigma"].tobytes()
    assert n2.tobytes() == d["n2"].tobytes()
    assert d2.tobytes() == d["d2"].tobytes()


def test_many_tiles_match_the_oracle(cuda):
    d, p = load("nlparlam_16x20_40")
    nl = make(p)
    pats = d["data"].reshape(p["nrows"] * p["ncols"], p["h"], p["w"])
    ind = np.asarray(d["mask"].flatten().nonzero()[0], np.int64)
    tb = 2.5e5  # about a dozen tiles
    cols, rows = no.calcchunks([p["w"], p["h"]], p["ncols"], p["nrows"], tb, 1, 1)
    assert len(cols) * len(rows) > 6
    want = no.calcsigma_chunked(d["data"], p["nrows"], p["ncols"], p["h"], p["w"], ind, p["saturation_protect"], tb)
    got = nl.calcsigma_tiles_array(pats, p["nrows"], p["ncols"], target_bytes=tb)
    for g, w in zip(got, want):
        assert g.tobytes() == w.tobytes()


@pytest.mark.parametrize("stride", [1, 2, 3])
def test_objective_matches_oracle(cuda, stride):
    import ctypes as C
    import torch
    from pyebsdindex_gb300 import _lib
    from pyebsdindex_gb300.nlpar import _bind
    d, p = load("nlparlam_12x14_32_dt")
    lib = _bind()
    d2 = torch.from_numpy(d["d2"]).cuda()
    work = torch.empty(256, dtype=torch.float64, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    for lam, tw in ((0.3, 0.5), (1.0, 0.34), (4.7, 0.25), (9.9, 0.5)):
        _lib.check(lib.ebsd_nlpar_lambda_metric(d2.data_ptr(), p["nrows"], p["ncols"], stride,
                                                float(np.float32(p["dthresh"])), lam, tw, work.data_ptr(),
                                                out.data_ptr(), C.c_void_p(0)))
        want = no.lambda_metric(np.array([lam]), d["d2"][0::stride, 0::stride, :], tw, np.float32(p["dthresh"]))
        assert abs(out.item() - want) <= 1e-12 * abs(want)


@pytest.mark.parametrize("name", CASES)
def test_opt_lambda_matches_reference(cuda, name):
    d, p = load(name)
    nl = make(p)
    pats = d["data"].reshape(p["nrows"] * p["ncols"], p["h"], p["w"])
    lam = nl.opt_lambda_array(pats, p["nrows"], p["ncols"], target_weights=p["target_weights"], target_bytes=2e9)
    np.testing.assert_allclose(lam, d["lam"], rtol=1e-6)
    assert abs(nl.lam - d["lam_opt"]) <= 1e-6 * d["lam_opt"]
