"""BandDetect.find_bands_file (ebsd_find_bands_file: a reader thread fills pinned chunk buffers
from a UP1 / UP2, Oxford .ebsp or ThermoFisher .pat file while two streams copy and detect)
must give the records find_bands gives for the same patterns in memory, bit for bit, whatever
the chunking."""
import os

import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import synthetic as syn
from pyebsdindex_gb300.ebsd_pattern import write_ebsp, write_tfpat, write_up

pytestmark = pytest.mark.gpu
FIELDS = ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")


def plan(h=80, nRho=120):
    bd = pg.BandDetect(nTheta=180, nRho=nRho, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=9)
    bd.band_detect_setup(patDim=(h, h), patternmask=syn.circular_mask(h, h))
    return bd


@pytest.mark.parametrize("method,chunk", [("fused", 0), ("fused", 700), ("plain", 500)])
def test_file_stream_equals_in_memory(cuda, tmp_path, method, chunk):
    pats = syn.make_patterns(2900, 80, 80, seed=51, noise_frac=0.1)[0]
    path = os.path.join(tmp_path, "scan.up1")
    write_up(path, pats, nCols=58, nRows=50)
    bd = plan()
    want = bd.find_bands(pats, method=method)
    got = bd.find_bands_file(path, method=method, chunk=chunk)
    for f in FIELDS:
        assert got[f].tobytes() == want[f].tobytes(), f
    part = bd.find_bands_file(path, patStart=1234, nPat=777, method=method, chunk=chunk)
    for f in FIELDS:
        assert part[f].tobytes() == want[f][1234:2011].tobytes(), f
    tail = bd.find_bands_file(path, patStart=2890, nPat=100, method=method)  # clamped to the file
    assert tail.shape[0] == 10


@pytest.mark.parametrize("kind", ["ebsp-u8", "ebsp-u16-v5", "tfpat"])
def test_record_files_stream_equal_in_memory(cuda, tmp_path, kind):
    """EBSP and TFPAT records (a header and footer around each pattern) gathered into the
    pinned chunks; an EBSP pattern that is not stored is detected as a zero pattern."""
    pats = syn.make_patterns(1300, 80, 80, seed=55, noise_frac=0.1)[0]
    if kind == "ebsp-u8":
        path = os.path.join(tmp_path, "scan.ebsp")
        write_ebsp(path, pats, nCols=50, nRows=26, version=4)
        with open(path, "r+b") as f:  # pattern 700 not stored
            f.seek(9 + 8 * 700)
            f.write(np.uint64(0).tobytes())
        pats[700] = 0
    elif kind == "ebsp-u16-v5":
        pats = pats.astype(np.uint16) * 16
        path = os.path.join(tmp_path, "scan.ebsp")
        write_ebsp(path, pats, nCols=50, nRows=26, version=5)
    else:
        pats = pats.astype(np.uint16) * 16
        path = os.path.join(tmp_path, "scan.pat")
        write_tfpat(path, pats, nCols=50, nRows=26, bitdepth=12, background=np.zeros((80, 80)))
    bd = plan()
    want = bd.find_bands(pats)
    got = bd.find_bands_file(path, chunk=300)
    for f in FIELDS:
        assert got[f].tobytes() == want[f].tobytes(), (kind, f)
    part = bd.find_bands_file(path, patStart=650, nPat=400, chunk=128)
    for f in FIELDS:
        assert part[f].tobytes() == want[f][650:1050].tobytes(), (kind, f)


def test_uint16_file(cuda, tmp_path):
    pats = (syn.make_patterns(600, 60, 60, seed=52, noise_frac=0.1)[0].astype(np.uint16) * 16)
    path = os.path.join(tmp_path, "scan.up2")
    write_up(path, pats, version=1)
    bd = plan(60, 90)
    want = bd.find_bands(pats)
    got = bd.find_bands_file(path, chunk=256)
    for f in FIELDS:
        assert got[f].tobytes() == want[f].tobytes(), f


def test_file_sets_up_the_plan_for_its_size(cuda, tmp_path):
    pats = syn.make_patterns(50, 60, 60, seed=53, noise_frac=0.1)[0]
    path = os.path.join(tmp_path, "s.up1")
    write_up(path, pats)
    bd = pg.BandDetect(nTheta=180, nRho=90, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=8)
    got = bd.find_bands_file(path)
    assert got.shape == (50, 8)
    assert np.array_equal(got["max"], bd.find_bands(pats)["max"])
    with pytest.raises(RuntimeError, match="pattern file"):
        bd.find_bands_file(os.path.join(tmp_path, "missing.up1"))


@pytest.mark.parametrize("method", ["fused", "plain"])
def test_pinned_input_in_place_or_copied(cuda, method):
    """Pinned host input read in place by the kernels (the default on a coherent CPU-GPU link)
    or staged by copies gives the same records as device input."""
    import torch
    from pyebsdindex_gb300 import _lib
    pats = syn.make_patterns(1500, 80, 80, seed=54, noise_frac=0.1)[0]
    bd = plan()
    want = bd.find_bands(torch.from_numpy(pats).cuda(), method=method)
    pinned = torch.from_numpy(pats).pin_memory().numpy()
    dp = bd._device_plan()
    for mode in (-1, 0, 1):
        dp.set_host_input(mode)
        got = dp.find_bands_host_records(pinned, method, bd.dataType, chunk=400)
        for f in FIELDS:
            assert got[f].tobytes() == want[f].tobytes(), (mode, f)
    dp.set_host_input(-1)
    with pytest.raises(RuntimeError, match="invalid argument"):
        dp.set_host_input(2)
