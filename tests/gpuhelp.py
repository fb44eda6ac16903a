"""Helpers shared by the GPU parity tests."""
import numpy as np

import pyebsdindex_gb300 as pg

RECORD_FIELDS = ["max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"]


def plan_from_golden(case, use_golden_lut=True):
    """Product BandDetect configured like the golden case; the reference's LUT is installed so
    that the host's float32 sin/cos (which differ between CPU back ends) cannot perturb it."""
    p = case["params"]
    bd = pg.BandDetect(nTheta=p["nTheta"], nRho=p["nRho"], tSigma=p["tSigma"], rSigma=p["rSigma"],
                       rhoMaskFrac=p["rhoMaskFrac"], nBands=p["nBands"])
    bd.band_detect_setup(patDim=case["patterns"].shape[-2:], patternmask=case.get("mask"))
    if use_golden_lut:
        bd.radonPlan.indexPlan = case["lut"].astype(np.int64)
    if "background" in case:
        bd.backgroundsub = case["background"]
    return bd


def golden_records(case):
    return {f: case["out_" + f] for f in RECORD_FIELDS}
