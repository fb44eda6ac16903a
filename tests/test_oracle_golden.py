"""The oracle (CPU restatement) reproduces the reference's golden vectors exactly."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import band_oracle as bo

FIELDS = ["max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid",
          "band_match_index", "id", "pqmax", "bandfit"]


def oracle_plan(case):
    p = case["params"]
    pats = case["patterns"]
    return bo.Plan(pats.shape[-2:], p["nTheta"], p["nRho"], p["tSigma"], p["rSigma"], p["rhoMaskFrac"],
                   p["nBands"], mask=case.get("mask"), background=case.get("background"))


@pytest.mark.parametrize("name", golden_names())
def test_oracle_plan_matches_reference(name):
    case = load_golden(name)
    plan = oracle_plan(case)
    nPx = int(np.prod(case["patterns"].shape[-2:]))
    assert np.array_equal(np.minimum(plan.lut, nPx + 1), case["lut"].astype(np.int64))
    assert np.array_equal(plan.rdnmask, case["rdnmask"].astype(bool))
    assert np.array_equal(plan.kernel, case["kernel"])
    assert np.array_equal(plan.theta, case["theta"]) and np.array_equal(plan.rho, case["rho"])
    assert np.array_equal(plan.padding, case["padding"]) and np.array_equal(plan.peakPad, case["peakPad"])
    assert np.array_equal(plan.count, case["count"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_bands_match_reference_exactly(name):
    case = load_golden(name)
    plan = oracle_plan(case)
    out = bo.find_bands(plan, case["patterns"], chunksize=case["params"].get("chunksize", 512))
    for f in FIELDS:
        assert np.array_equal(out[f], case["out_" + f]), f


def test_oracle_fp64_close_to_reference():
    """The FP64 / direct-convolution oracle agrees with the FFT float32 reference to far
    below the 1e-3 Radon-pixel sub-pixel tolerance."""
    from bandcmp import compare
    case = load_golden("c1_80_u8")
    plan = oracle_plan(case)
    out = bo.find_bands(plan, case["patterns"], conv="direct", dtype=np.float64)
    ref = {f: case["out_" + f] for f in ["max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta",
                                         "rho", "valid"]}
    c = compare(out, ref)
    assert c["frac"] == 1.0
    assert c["aveloc"] < 1e-4


@pytest.mark.parametrize("name", golden_names())
def test_c_port_matches_reference(name):
    """The C/OpenMP restatement (the timed CPU baseline) agrees with the reference: same
    integer peaks, sub-pixel within 1e-3 Radon pixels (it convolves directly, not by FFT)."""
    from bandcmp import compare
    from oracle import cport
    case = load_golden(name)
    plan = oracle_plan(case)
    out = cport.find_bands(plan, case["patterns"], threads=2)
    ref = {f: case["out_" + f] for f in ["max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta",
                                         "rho", "valid"]}
    c = compare(out, ref, skip=case["degenerate"])
    assert c["frac"] == 1.0, c
    assert c["aveloc"] <= 1e-3, c
    assert c["rel"]["max"] <= 1e-4, c
