"""The NLPAR oracle reproduces the reference's sigma_numba / nlpar_nb golden vectors exactly."""
import numpy as np
import pytest

from conftest import load_golden, nlpar_golden_names
from oracle import nlpar_oracle as no


@pytest.mark.parametrize("name", nlpar_golden_names())
def test_nlpar_oracle_matches_reference(name):
    c = load_golden(name)
    p = c["params"]
    mask = no.automask(p["h"], p["w"])
    assert np.array_equal(mask, c["mask"])
    ind = np.nonzero(mask.ravel())[0]
    sig = no.sigma(c["data"], p["nrows"], p["ncols"], ind, p["saturation_protect"])
    assert np.array_equal(sig, c["sigma"])
    out = no.nlpar(c["data"], p["lam"], p["sr"], p["dthresh"], c["sigma"], p["nrows"], p["ncols"], ind,
                   p["saturation_protect"])
    assert np.array_equal(out, c["out"])


def test_nlpar_oracle_matches_reference_on_non_integer_and_large_data():
    """nlpar_nb sums a pair's squared differences in float64 (np.float32 ** np.int32 promotes);
    the oracle does too, so it stays bit-identical to the reference (run through
    oracle/refshim.py) where float32 sums would round: square roots of patterns (stem_scale),
    fractional values, and uint16-range counts whose pair sums pass 2^24.  The reference's
    sigma is passed to both: the shim's sigma_numba squares float32 scalars with numpy's scalar
    power, which for squares above 2^24 can differ in the last bit from the x * x numba
    compiles (and the oracle and the device use)."""
    import warnings
    from oracle import refshim
    from pyebsdindex_gb300 import synthetic as syn
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    N = refshim.load().nlpar_cpu.NLPAR
    pats = syn.make_patterns(7 * 9, 16, 16, seed=19, noise_frac=0.1)[0].astype(np.float32)
    rng = np.random.default_rng(4)
    ind = np.asarray(no.automask(16, 16).ravel().nonzero()[0], np.int64)
    for d in (np.sqrt(pats - pats.min()), pats + rng.random(pats.shape),
              pats * 200 + rng.integers(0, 3000, pats.shape)):
        d = np.ascontiguousarray(d, dtype=np.float32).reshape(63, -1)
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            rsig = N.sigma_numba(d, 1, 7, 9, np.array([0, 7], np.int64), np.array([0, 9], np.int64), ind, True)[0]
            want = N.nlpar_nb(d, np.float32(0.8), 2, np.float32(0.1), rsig, 7, 9, indices_in=ind,
                              saturation_protect=True)
        got = no.nlpar(d, 0.8, 2, 0.1, rsig, 7, 9, ind, True)
        assert got.tobytes() == want.tobytes()
