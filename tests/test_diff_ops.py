"""Sparse operators of the differentiable path equal the band-detection arithmetic (CPU):
R x is the Radon ray mean (radon_fast.py:281-310), M r is the padded LoG response
(band_detect.py:573-606) on the interior, and the transposes are exact transposes."""
import numpy as np

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import diff, synthetic as syn
from oracle import band_oracle as bo


def _dense(rowptr, col, val, shape):
    d = np.zeros(shape)
    rows = np.repeat(np.arange(shape[0]), np.diff(rowptr))
    np.add.at(d, (rows, col), val.astype(np.float64))
    return d


def _setup(h=40, w=48, nRho=60, nTheta=90):
    bd = pg.BandDetect(nTheta=nTheta, nRho=nRho, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=6)
    bd.band_detect_setup(patDim=(h, w), patternmask=syn.circular_mask(h, w))
    plan = bo.Plan((h, w), nTheta, nRho, 1.0, 1.0, 0.1, 6, mask=syn.circular_mask(h, w))
    return bd, plan


def test_radon_operator_is_the_ray_mean():
    bd, plan = _setup()
    R = _dense(*diff.radon_csr(bd))
    pats = syn.make_patterns(3, 40, 48, seed=3)[0].astype(np.float64)
    ref = bo.radon_gather(plan, pats, dtype=np.float64)
    p0, p1 = plan.padding
    inner = ref[p0:p0 + plan.nRho, p1:p1 + plan.nTheta, :].reshape(-1, 3)
    got = R @ pats.reshape(3, -1).T
    nonempty = plan.count.reshape(-1) > 0
    # 1/count is held as float32 in the operator: relative 6e-8
    np.testing.assert_allclose(got[nonempty], inner[nonempty], rtol=1e-7, atol=1e-9)
    assert np.all(got[~nonempty] == 0)


def test_log_operator_is_padded_convolution():
    bd, plan = _setup()
    M = _dense(*diff.log_csr(bd))
    rng = np.random.default_rng(0)
    r = rng.normal(size=(plan.nRho, plan.nTheta))
    p0, p1 = plan.padding
    full = np.zeros((plan.nRho + 2 * p0, plan.nTheta + 2 * p1, 1))
    full[p0:p0 + plan.nRho, p1:p1 + plan.nTheta, 0] = r
    conv = bo.conv_direct(bo.radon_pad(plan, full), plan.kernel, dtype=np.float64)
    ref = conv[p0:p0 + plan.nRho, p1:p1 + plan.nTheta, 0].reshape(-1)
    # taps folded onto the same source cell are summed then held as float32
    np.testing.assert_allclose(M @ r.reshape(-1), ref, rtol=1e-6, atol=1e-6)


def test_transpose_is_exact():
    bd, _ = _setup()
    for csr in (diff.radon_csr(bd), diff.log_csr(bd)):
        A = _dense(*csr)
        AT = _dense(*diff.transpose_csr(*csr))
        assert np.array_equal(AT, A.T)
