"""NLPAR's file interface on the device (pyebsdindex_gb300/nlpar.py: calcnlpar, opt_lambda,
calcsigma on pattern files).  One tile: the output file holds exactly calcnlpar_array of the
file's scan, clipped to the file's type.  Several tiles: sigma bit-identical to the oracle run
through the same tiling, the averaged patterns within one count (CUDA's expf against numpy's
float32 exp, then truncation to uint8).  opt_lambda / calcsigma on a file give what the array
forms give on the file's scan."""
import os

import numpy as np
import pytest

from oracle import nlpar_oracle as no
from pyebsdindex_gb300 import synthetic as syn
from pyebsdindex_gb300.ebsd_pattern import get_pattern_file_obj, pat_flt2int, write_up
from pyebsdindex_gb300.nlpar import NLPAR

pytestmark = pytest.mark.gpu


def voronoi_file(tmp_path, nrows, ncols, h, seed):
    pats, _ = syn.voronoi_scan(nrows, ncols, ngrains=max(3, nrows * ncols // 10), h=h, w=h, seed=seed)
    path = os.path.join(tmp_path, "scan.up1")
    write_up(path, pats.reshape(nrows * ncols, h, h), nCols=ncols, nRows=nrows)
    return path


def read_all(path):
    return get_pattern_file_obj(path).read_data(patStartCount=[0, -1], returnArrayOnly=True)[0]


def test_one_tile_equals_the_array_form(cuda, tmp_path):
    src = voronoi_file(tmp_path, 12, 15, 32, 61)
    out = NLPAR(src, lam=0.8, searchradius=2).calcnlpar(fileout=os.path.join(tmp_path, "o.up1"), verbose=0)
    data = read_all(src).astype(np.float32)
    want = NLPAR(lam=0.8, searchradius=2).calcnlpar_array(data, 12, 15)
    assert read_all(out).tobytes() == pat_flt2int(want, typeout=np.uint8).tobytes()


@pytest.mark.parametrize("diff_offset", [0.0, 0.3])
def test_tiles_follow_the_oracle(cuda, tmp_path, monkeypatch, diff_offset):
    """Several tiles, with and without a diff_offset (the centre-weight additions)."""
    src = voronoi_file(tmp_path, 11, 13, 24, 62)
    nl = NLPAR(src, lam=0.8, searchradius=2)
    got = nl.calcnlpar(chunksize=80_000, fileout=os.path.join(tmp_path, "g.up1"), verbose=0, diff_offset=diff_offset)
    sig_dev = nl.sigma.copy()

    def tile_sigma(self, data, nrows, ncols, saturation_protect):
        ind = np.asarray(np.asarray(self.mask).ravel().nonzero()[0], np.int64)
        return no.sigma(data.reshape(nrows * ncols, -1), nrows, ncols, ind, saturation_protect)

    def tile_nlpar(self, data, nrows, ncols, lam, sr, dthresh, saturation_protect, sigma, centre_offset=None):
        ind = np.asarray(np.asarray(self.mask).ravel().nonzero()[0], np.int64)
        return no.nlpar(data.reshape(nrows * ncols, -1), lam, sr, dthresh, sigma, nrows, ncols, ind,
                        saturation_protect, centre_offset=centre_offset).reshape(data.shape)

    monkeypatch.setattr(NLPAR, "_tile_sigma", tile_sigma)
    monkeypatch.setattr(NLPAR, "_tile_nlpar", tile_nlpar)
    ref = NLPAR(src, lam=0.8, searchradius=2)
    want = ref.calcnlpar(chunksize=80_000, fileout=os.path.join(tmp_path, "w.up1"), verbose=0,
                         diff_offset=diff_offset)
    assert sig_dev.tobytes() == ref.sigma.tobytes()
    a, b = read_all(got).astype(np.int16), read_all(want).astype(np.int16)
    assert np.abs(a - b).max() <= 1
    assert (a == b).mean() > 0.995


def test_lambda_and_sigma_on_a_file(cuda, tmp_path):
    src = voronoi_file(tmp_path, 14, 16, 32, 63)
    data = read_all(src).astype(np.float32)
    a = NLPAR(src)
    lam_file = a.opt_lambda(verbose=0)
    lam_arr = NLPAR().opt_lambda_array(data, 14, 16)
    assert np.array_equal(lam_file, lam_arr)
    sig_f, d2_f, n2_f = NLPAR(src).calcsigma(verbose=0)
    sig_a, d2_a, n2_a = NLPAR().calcsigma_tiles_array(data, 14, 16)
    assert sig_f.tobytes() == sig_a.tobytes() and d2_f.tobytes() == d2_a.tobytes() and n2_f.tobytes() == n2_a.tobytes()
    out = NLPAR(src, searchradius=1).auto_nlpar(fileout=os.path.join(tmp_path, "auto.up1"), verbose=0)
    assert read_all(out).shape == (14 * 16, 32, 32)


NLPARFILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nlparfile")


@pytest.mark.parametrize("name", ["onetile_9x11_16", "tiles_10x12_16"])
def test_calcnlpar_against_reference_run(cuda, tmp_path, name):
    """The device path on the committed reference runs of calcnlpar_cpu (tests/golden/nlparfile/):
    merged sigma bit-identical, output patterns within one count of the reference's file."""
    import json
    import shutil
    p = json.load(open(os.path.join(NLPARFILE, name + ".json")))
    src = os.path.join(tmp_path, "in.up1")
    shutil.copyfile(os.path.join(NLPARFILE, name + "_in.up1"), src)
    nl = NLPAR(src, lam=p["lam"], searchradius=p["searchradius"])
    out = nl.calcnlpar(chunksize=p["chunksize"], fileout=os.path.join(tmp_path, "out.up1"), verbose=0)
    assert nl.sigma.tobytes() == np.load(os.path.join(NLPARFILE, name + "_sigma.npy")).tobytes()
    a = read_all(out).astype(np.int16)
    b = read_all(os.path.join(NLPARFILE, name + "_out.up1")).astype(np.int16)
    assert np.abs(a - b).max() <= 1
    assert (a == b).mean() > 0.995
