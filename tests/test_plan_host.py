"""Host-side plan construction (LUT, masks, kernel, background fit) equals the reference's."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
import pyebsdindex_gb300 as pg
from pyebsdindex_gb300.band_detect import record_dtype


def product_plan(case):
    p = case["params"]
    bd = pg.BandDetect(nTheta=p["nTheta"], nRho=p["nRho"], tSigma=p["tSigma"], rSigma=p["rSigma"],
                       rhoMaskFrac=p["rhoMaskFrac"], nBands=p["nBands"])
    bd.band_detect_setup(patDim=case["patterns"].shape[-2:], patternmask=case.get("mask"))
    return bd


@pytest.mark.parametrize("name", golden_names())
def test_plan_matches_reference(name):
    case = load_golden(name)
    bd = product_plan(case)
    nPx = int(np.prod(case["patterns"].shape[-2:]))
    assert np.array_equal(np.minimum(bd.radonPlan.indexPlan, nPx + 1), case["lut"].astype(np.int64))
    assert np.array_equal(bd.rdnmask, case["rdnmask"].astype(bool))
    assert np.array_equal(bd.kernel[0], case["kernel"])
    assert np.array_equal(bd.radonPlan.theta, case["theta"])
    assert np.array_equal(bd.radonPlan.rho, case["rho"])
    assert np.array_equal(bd.padding, case["padding"])
    assert np.array_equal(bd.peakPad, case["peakPad"])
    assert np.float32(bd.rhoMax) == case["rhoMax"]


def test_background_fit_matches_reference():
    case = load_golden("u16_bg_60")
    bd = product_plan(case)
    with np.errstate(all="ignore"):
        bd.collect_background(patsIn=case["patterns"])
    np.testing.assert_allclose(bd.backgroundsub, case["background"], rtol=1e-9, atol=1e-9)


def test_record_dtype():
    dt = record_dtype(10)
    assert dt.itemsize == 209
    assert dt.names == ('id', 'max', 'normmax', 'maxloc', 'avemax', 'aveloc', 'pqmax', 'width', 'theta',
                        'rho', 'valid', 'band_match_index', 'bandfit')
    bd = pg.BandDetect(patDim=(60, 60), nPhases=3)
    assert bd.dataType == record_dtype(3)


def test_setup_shape_change_keeps_reference_behaviour():
    """Like the reference (radon_fast.py:189-190), re-running setup for a smaller pattern keeps
    the previous size's default maskindex and raises; a fresh plan for the new size works."""
    bd = pg.BandDetect(patDim=(60, 60), nRho=90, tSigma=1.0, rSigma=1.0)
    assert bd.radonPlan.indexPlan.shape == (90, 180, 60)
    with pytest.raises(Exception, match="max of index array"):
        bd.band_detect_setup(patDim=(40, 50))
    bd2 = pg.BandDetect(patDim=(40, 50), nRho=90, tSigma=1.0, rSigma=1.0)
    assert bd2.radonPlan.indexPlan.shape == (90, 180, 50)
    assert bd2.rhoMax == np.float32(20.0)


def test_maskindex_out_of_range_raises():
    bd = pg.BandDetect()
    with pytest.raises(Exception):
        bd.band_detect_setup(patDim=(10, 10), patternmaskindex=np.full((10, 10), 100))
