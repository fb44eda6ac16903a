"""Without a CUDA device every product entry point raises: there is no CPU fallback (the
reference's OpenCL path fell back to the CPU on any exception, band_detect_cl.py:195-197)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, gpu_available

pytestmark = pytest.mark.skipif(gpu_available(), reason="checks the no-device behaviour")


def test_detection_entry_points_raise(built_lib, tmp_path):
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import synthetic as syn
    from pyebsdindex_gb300.ebsd_pattern import write_up
    bd = pg.BandDetect(nTheta=60, nRho=30, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=4)
    bd.band_detect_setup(patDim=(20, 20), patternmask=syn.circular_mask(20, 20))
    pats = np.zeros((3, 20, 20), np.uint8)
    with pytest.raises(RuntimeError):
        bd.find_bands(pats)
    path = os.path.join(tmp_path, "s.up1")
    write_up(path, pats)
    with pytest.raises(RuntimeError):
        bd.find_bands_file(path)


def test_nlpar_entry_points_raise(built_lib):
    import pyebsdindex_gb300 as pg
    nl = pg.NLPAR(lam=0.7, searchradius=1)
    data = np.random.default_rng(0).integers(0, 255, (12, 16, 16)).astype(np.float32)
    for call in (lambda: nl.calcsigma_array(data, 3, 4), lambda: nl.calcnlpar_array(data, 3, 4),
                 lambda: nl.opt_lambda_array(data, 3, 4, target_bytes=2e9)):
        with pytest.raises((RuntimeError, AssertionError)):
            call()


def test_nlpar_file_interface_raises(built_lib, tmp_path):
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300.ebsd_pattern import write_ebsp
    path = os.path.join(tmp_path, "s.ebsp")
    write_ebsp(path, np.random.default_rng(1).integers(0, 255, (12, 16, 16)).astype(np.uint8), nCols=4, nRows=3)
    for call in (lambda: pg.NLPAR(path, searchradius=1).calcnlpar(fileout=os.path.join(tmp_path, "o.ebsp"), verbose=0),
                 lambda: pg.NLPAR(path).opt_lambda(verbose=0), lambda: pg.NLPAR(path).calcsigma(verbose=0)):
        with pytest.raises((RuntimeError, AssertionError)):
            call()


def test_vote_entry_points_raise(built_lib):
    from oracle import vote_oracle as vo
    from pyebsdindex_gb300 import tripletvote as tv
    lib, params, ins, _ = vo.load_case(os.path.join(GOLDEN_DIR, "vote_fcc_syn4.npz"))
    bi = tv.BandIndexer(lib=lib, angTol=params["angTol"], nband_earlyexit=params["nband_earlyexit"])
    with pytest.raises((RuntimeError, AssertionError)):
        bi.bandindex(ins["norms"], band_intensity=ins["inten"])
