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
