"""GPU NLPAR against the reference's golden vectors (sigma_numba / nlpar_nb).

The device kernels keep the reference's float32 accumulation order; the exponential is CUDA's
expf instead of numpy's float32 exp, so weights may differ in the last bit.  Tolerances:
sigma bit-identical, averaged patterns within 1e-5 relative of the pattern scale.
"""
import numpy as np
import pytest

from conftest import load_golden, nlpar_golden_names
import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import synthetic as syn
from oracle import nlpar_oracle as no

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", nlpar_golden_names())
def test_nlpar_matches_reference(cuda, name):
    c = load_golden(name)
    p = c["params"]
    nl = pg.NLPAR(lam=p["lam"], searchradius=p["sr"], dthresh=p["dthresh"],
                  saturation_protect=p["saturation_protect"])
    data = c["data"].reshape(p["nrows"] * p["ncols"], p["h"], p["w"])
    sig = nl.calcsigma_array(data, p["nrows"], p["ncols"])
    assert np.array_equal(sig, c["sigma"]), np.abs(sig - c["sigma"]).max()
    out = nl.calcnlpar_array(data, p["nrows"], p["ncols"], sigma=c["sigma"])
    ref = c["out"].reshape(out.shape)
    scale = np.abs(ref).max()
    assert np.abs(out - ref).max() <= 1e-5 * scale, np.abs(out - ref).max()


def test_nlpar_torch_device_roundtrip(cuda):
    import torch
    pats, _ = syn.voronoi_scan(12, 14, ngrains=10, h=40, w=40, seed=11)
    nl = pg.NLPAR(lam=0.7, searchradius=3)
    host = nl.calcnlpar_array(pats, 12, 14, reset_sigma=True)
    nl2 = pg.NLPAR(lam=0.7, searchradius=3)
    dev = nl2.calcnlpar_array(torch.from_numpy(pats).to(cuda), 12, 14, reset_sigma=True)
    assert isinstance(dev, torch.Tensor) and dev.is_cuda
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    # oracle on the same input
    mask = no.automask(40, 40)
    ind = np.nonzero(mask.ravel())[0]
    data = pats.reshape(12 * 14, -1).astype(np.float32)
    sig = no.sigma(data, 12, 14, ind)
    ref = no.nlpar(data, 0.7, 3, 0.0, sig, 12, 14, ind).reshape(host.shape)
    assert np.abs(host - ref).max() <= 1e-5 * np.abs(ref).max()


def test_nlpar_then_band_detection_stays_on_device(cuda):
    """NLPAR output feeds find_bands directly (float32 device tensor, no host round trip)."""
    import torch
    pats, _ = syn.voronoi_scan(10, 12, ngrains=8, h=60, w=60, seed=12)
    nl = pg.NLPAR(lam=0.7, searchradius=2)
    smooth = nl.calcnlpar_array(torch.from_numpy(pats).to(cuda), 10, 12)
    bd = pg.BandDetect(nTheta=180, nRho=90, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=8)
    bd.band_detect_setup(patDim=(60, 60), patternmask=syn.circular_mask(60, 60))
    a = bd.find_bands(smooth, method="fused")
    b = bd.find_bands(smooth.cpu().numpy(), method="plain")
    assert (a["valid"] == 1).mean() > 0.5
    assert np.array_equal(a["maxloc"][a["valid"] == 1], b["maxloc"][a["valid"] == 1]) or \
        (a["maxloc"] == b["maxloc"]).mean() > 0.99


def test_nlpar_rejects_oversized_window(cuda):
    pats, _ = syn.voronoi_scan(4, 4, ngrains=3, h=20, w=20, seed=1)
    nl = pg.NLPAR(lam=0.7, searchradius=3)
    with pytest.raises(RuntimeError, match="invalid argument"):
        nl.calcnlpar_array(pats, 4, 4)


@pytest.mark.parametrize("out_dtype", [np.uint8, np.uint16])
def test_nlpar_integer_output_is_the_reference_writers_conversion(cuda, out_dtype):
    """The averaging kernel's integer output equals the float32 average clipped to the type's
    range and truncated, as the reference's pattern writer stores NLPAR output (pat_flt2int
    'clip', ebsd_pattern.py:118-182) -- bit for bit, and band detection reads it directly."""
    import pyebsdindex_gb300 as pg
    pats, _ = syn.voronoi_scan(12, 14, ngrains=6, h=40, w=40, seed=8, peak_range=(60.0, 250.0))
    nl = pg.NLPAR(lam=0.7, searchradius=3)
    f = nl.calcnlpar_array(pats, 12, 14)
    g = nl.calcnlpar_array(pats, 12, 14, out_dtype=out_dtype)
    hi = np.iinfo(out_dtype).max
    assert g.dtype == out_dtype
    assert np.array_equal(g, np.clip(f, 0, hi).astype(out_dtype))
    if out_dtype is np.uint8:
        bd = pg.BandDetect(nTheta=180, nRho=60, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=8)
        bd.band_detect_setup(patDim=(40, 40), patternmask=syn.circular_mask(40, 40))
        a = bd.find_bands(g, method="fused")
        b = bd.find_bands(np.clip(f, 0, 255).astype(np.uint8), method="fused")
        for k in ("max", "maxloc", "aveloc", "valid"):
            assert a[k].tobytes() == b[k].tobytes(), k
