"""NLPAR's file interface (NLPAR.setfile / calcnlpar / opt_lambda / calcsigma / auto_nlpar,
pyebsdindex_gb300/nlpar.py) -- the host side: scan tiles with halos, sigma merged tile by tile,
tile interiors clipped and written into the output file -- against the reference's own
calcnlpar_cpu (nlpar_cpu.py:283-540, imported through oracle/refshim.py) on UP1, EBSP and TFPAT
files, byte for byte.

The per-tile device computations (``NLPAR._tile_sigma`` = calcsigma_array and
``NLPAR._tile_nlpar`` = calcnlpar_array, checked against the reference on the GPU in
tests/test_gpu_nlpar.py) are replaced here by the oracle's restatements of sigma_numba and
nlpar_nb, so that what these CPU tests check is the host logic around them; the device path
through the same interface is tests/test_gpu_nlpar_file.py."""
import os
import warnings

import numpy as np
import pytest

from oracle import nlpar_oracle as no
from oracle import refshim
from pyebsdindex_gb300 import synthetic as syn


@pytest.fixture(scope="module")
def ref():
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    ns = refshim.load()
    refshim.pattern_module()
    return ns


@pytest.fixture
def oracle_tiles(monkeypatch):
    """NLPAR's two per-tile device calls answered by the oracle."""
    from pyebsdindex_gb300.nlpar import NLPAR

    def tile_sigma(self, data, nrows, ncols, saturation_protect):
        ind = np.asarray(np.asarray(self.mask).ravel().nonzero()[0], np.int64)
        return no.sigma(data.reshape(nrows * ncols, -1), nrows, ncols, ind, saturation_protect)

    def tile_nlpar(self, data, nrows, ncols, lam, sr, dthresh, saturation_protect, sigma, centre_offset=None):
        ind = np.asarray(np.asarray(self.mask).ravel().nonzero()[0], np.int64)
        out = no.nlpar(data.reshape(nrows * ncols, -1), lam, sr, dthresh, sigma, nrows, ncols, ind,
                       saturation_protect, centre_offset=centre_offset)
        return out.reshape(data.shape)

    monkeypatch.setattr(NLPAR, "_tile_sigma", tile_sigma)
    monkeypatch.setattr(NLPAR, "_tile_nlpar", tile_nlpar)


def scan(nrows, ncols, h, seed, dtype=np.uint8):
    pats = syn.make_patterns(nrows * ncols, h, h, seed=seed, noise_frac=0.1)[0]
    return pats if dtype == np.uint8 else pats.astype(np.uint16) * 8


def write(kind, path_dir, pats, nrows, ncols):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    if kind == "up1":
        path = os.path.join(path_dir, "scan.up1")
        ep.write_up(path, pats, nCols=ncols, nRows=nrows)
    elif kind == "ebsp":
        path = os.path.join(path_dir, "scan.ebsp")
        ep.write_ebsp(path, pats, nCols=ncols, nRows=nrows, xStep=0.5, yStep=0.5, version=4)
    else:
        path = os.path.join(path_dir, "scan.pat")
        ep.write_tfpat(path, pats, nCols=ncols, nRows=nrows, bitdepth=12)
    return path


# (file kind, nrows, ncols, pattern size, searchradius, chunksize bytes: small ones force several tiles)
CASES = [("up1", 9, 11, 16, 2, 0), ("up1", 9, 11, 16, 2, 60_000), ("ebsp", 8, 10, 16, 1, 50_000),
         ("tfpat", 10, 8, 14, 2, 45_000)]


@pytest.mark.parametrize("kind,nrows,ncols,h,sr,chunk", CASES)
def test_calcnlpar_file_matches_reference(tmp_path, ref, oracle_tiles, built_lib, kind, nrows, ncols, h, sr, chunk):
    from pyebsdindex_gb300.nlpar import NLPAR
    pats = scan(nrows, ncols, h, 7, np.uint8 if kind != "tfpat" else np.uint16)
    src = write(kind, str(tmp_path), pats, nrows, ncols)
    mine_out = os.path.join(tmp_path, "mine" + os.path.splitext(src)[1])
    theirs_out = os.path.join(tmp_path, "theirs" + os.path.splitext(src)[1])
    nl = NLPAR(src, lam=0.9, searchradius=sr)
    got = nl.calcnlpar(chunksize=chunk, fileout=mine_out, verbose=0)
    rn = ref.nlpar_cpu.NLPAR(src, lam=0.9, searchradius=sr)
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        want = rn.calcnlpar_cpu(chunksize=chunk, fileout=theirs_out, verbose=0)
    assert os.path.samefile(got, mine_out) and os.path.samefile(want, theirs_out)
    assert open(mine_out, "rb").read() == open(theirs_out, "rb").read()
    assert nl.sigma.tobytes() == np.asarray(rn.sigma, np.float32).tobytes()
    if chunk:
        from pyebsdindex_gb300.nlpar import scan_tiles
        c, r = scan_tiles([h, h], ncols, nrows, chunk, sr, sr)
        assert len(c) * len(r) > 1  # the case runs several tiles


def test_default_output_name_and_sigma_reuse(tmp_path, ref, oracle_tiles, built_lib):
    """Without fileout the output is <stem>_NLPAR_l{lam:.2f}sr{sr}<ext> beside the input; a
    sigma already set (here a constant) is used as is, as the reference does."""
    from pyebsdindex_gb300.nlpar import NLPAR
    pats = scan(6, 7, 16, 11)
    src = write("up1", str(tmp_path), pats, 6, 7)
    nl = NLPAR(src, lam=1.25, searchradius=1)
    nl.sigma = np.float32(3.0)
    got = nl.calcnlpar(verbose=0)
    assert os.path.basename(got) == "scan_NLPAR_l1.25sr1.up1"
    rn = ref.nlpar_cpu.NLPAR(src, lam=1.25, searchradius=1)
    rn.sigma = np.array([3.0], np.float32)
    theirs = os.path.join(tmp_path, "t.up1")
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        rn.calcnlpar_cpu(fileout=theirs, verbose=0)
    assert open(got, "rb").read() == open(theirs, "rb").read()
    assert np.all(nl.sigma == 3.0)
    with pytest.raises(ValueError, match="exactly the same"):
        NLPAR(src).calcnlpar(fileout=src, verbose=0)


def test_file_writers_match_reference_write_data(tmp_path, ref, built_lib):
    """write_data on a copy_file(empty_data) output, a slab of float patterns, as the
    reference's write_data lays it down (clip to the file's type)."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    rp = refshim.pattern_module()
    pats = scan(5, 6, 12, 13)
    rng = np.random.default_rng(3)
    newp = rng.uniform(-20, 300, size=(6, 12, 12)).astype(np.float32)
    for kind in ("up1", "ebsp", "tfpat"):
        src = write(kind, str(tmp_path), pats if kind != "tfpat" else pats.astype(np.uint16), 5, 6)
        ext = os.path.splitext(src)[1]
        a, b = os.path.join(tmp_path, "a" + ext), os.path.join(tmp_path, "b" + ext)
        mine = ep.get_pattern_file_obj(src)
        mine.copy_file(a, empty_data=True)
        theirs = rp.get_pattern_file_obj(src)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            theirs.copy_file(b, empty_data=True)
        fa, fb = ep.get_pattern_file_obj(a), rp.get_pattern_file_obj(b)
        fa.write_data(newpatterns=newp, patStartCount=[[1, 2], [3, 2]], flt2int='clip', scalevalue=1.0)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            fb.write_data(newpatterns=newp, patStartCount=[[1, 2], [3, 2]], flt2int='clip', scalevalue=1.0)
        assert open(a, "rb").read() == open(b, "rb").read(), kind


def test_pat_flt2int_matches_reference(ref, built_lib):
    from pyebsdindex_gb300.ebsd_pattern import pat_flt2int
    rp = refshim.pattern_module()
    rng = np.random.default_rng(5)
    x = rng.uniform(-50, 70000, size=(3, 7, 9)).astype(np.float32)
    for kw in (dict(typeout=np.uint8), dict(typeout=np.uint16), dict(), dict(typeout=np.uint8, maxScale=100),
               dict(typeout=np.uint16, method='fullscale'), dict(typeout=np.uint8, method='scale', scalevalue=0.9),
               dict(typeout=np.float32)):
        a, b = pat_flt2int(x, **kw), rp.pat_flt2int(x, **kw)
        assert a.dtype == b.dtype and a.tobytes() == b.tobytes(), kw


@pytest.fixture
def oracle_scans(monkeypatch):
    """NLPAR's whole-scan device calls (calcsigma_tiles_array, opt_lambda_array) answered by
    the oracle's restatement of calcsigma_cpu / opt_lambda_cpu."""
    from pyebsdindex_gb300.nlpar import NLPAR

    def tiles(self, data, nrows, ncols, saturation_protect=None, target_bytes=None):
        h, w = data.shape[-2:]
        if self.mask is None:
            self.mask = self.makeautomask(h, w) if self.automask is True else np.ones((h, w), np.uint8)
        ind = np.asarray(np.asarray(self.mask).ravel().nonzero()[0], np.int64)
        return no.calcsigma_chunked(data.reshape(nrows * ncols, -1), nrows, ncols, h, w, ind,
                                    saturation_protect, target_bytes)

    def lam(self, data, nrows, ncols, target_weights=(0.5, 0.34, 0.25), autoupdate=True, dthresh=None,
            saturation_protect=None, target_bytes=None, verbose=0):
        if dthresh is not None:
            self.dthresh = dthresh
        sig, d2, _ = tiles(self, data, nrows, ncols, saturation_protect, target_bytes)
        vals = no.opt_lambda(d2, sig.size, target_weights, float(np.float32(self.dthresh)))
        if autoupdate:
            self.lam = np.median(vals)
        if self.sigma is None:
            self.sigma = sig
        return vals

    monkeypatch.setattr(NLPAR, "calcsigma_tiles_array", tiles)
    monkeypatch.setattr(NLPAR, "opt_lambda_array", lam)


def test_opt_lambda_and_calcsigma_files_match_reference(tmp_path, ref, oracle_scans, oracle_tiles, built_lib):
    """opt_lambda / calcsigma on a file read the scan the reference reads (its shape from the
    file), and auto_nlpar then averages with the chosen lambda and the lambda path's sigma."""
    from pyebsdindex_gb300.nlpar import NLPAR
    pats, _ = syn.voronoi_scan(8, 10, ngrains=7, h=24, w=24, seed=17)
    src = write("up1", str(tmp_path), pats, 8, 10)
    nl = NLPAR(src, searchradius=2)
    rn = ref.nlpar_cpu.NLPAR(src, searchradius=2)
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        want_sig = rn.calcsigma_cpu(chunksize=30_000, verbose=0)
        want_lam = rn.opt_lambda_cpu(verbose=0, chunksize=30_000)
    got_sig = nl.calcsigma(chunksize=30_000, verbose=0)
    for a, b in zip(got_sig, want_sig):
        assert np.asarray(a).tobytes() == np.asarray(b).tobytes()
    got_lam = nl.opt_lambda(verbose=0, chunksize=30_000)
    assert np.array_equal(got_lam, want_lam) and nl.lam == rn.lam
    assert nl.sigma.tobytes() == np.asarray(rn.sigma).tobytes()
    mine, theirs = os.path.join(tmp_path, "m.up1"), os.path.join(tmp_path, "t.up1")
    nl.calcnlpar(fileout=mine, verbose=0)
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        rn.calcnlpar_cpu(fileout=theirs, verbose=0)
    assert open(mine, "rb").read() == open(theirs, "rb").read()


@pytest.mark.parametrize("opts", [dict(stem_scale=True), dict(rescale=True), dict(dthresh=0.3, saturation_protect=False)])
def test_calcnlpar_options_match_reference(tmp_path, ref, oracle_tiles, built_lib, opts):
    """stem_scale (square root above the file's minimum, squared back), rescale (each output
    pattern stretched to the file type's range) and a distance threshold without saturation
    protection, as calcnlpar_cpu applies them."""
    from pyebsdindex_gb300.nlpar import NLPAR
    pats = scan(7, 9, 16, 19)
    src = write("up1", str(tmp_path), pats, 7, 9)
    mine, theirs = os.path.join(tmp_path, "m.up1"), os.path.join(tmp_path, "t.up1")
    NLPAR(src, lam=0.8, searchradius=2).calcnlpar(fileout=mine, chunksize=40_000, verbose=0, **opts)
    rn = ref.nlpar_cpu.NLPAR(src, lam=0.8, searchradius=2)
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        rn.calcnlpar_cpu(fileout=theirs, chunksize=40_000, verbose=0, **opts)
    assert open(mine, "rb").read() == open(theirs, "rb").read()


def test_diff_offset_matches_reference(tmp_path, ref, oracle_tiles, built_lib):
    """A non-zero diff_offset: the centre-weight additions nlpar_nb accumulates over its serial
    visit order (per tile, over the computed block), in one tile and in several."""
    from pyebsdindex_gb300.nlpar import NLPAR
    pats = scan(9, 11, 16, 29)
    src = write("up1", str(tmp_path), pats, 9, 11)
    for chunk in (0, 60_000):
        mine, theirs = os.path.join(tmp_path, "m.up1"), os.path.join(tmp_path, "t.up1")
        NLPAR(src, lam=0.8, searchradius=2).calcnlpar(fileout=mine, chunksize=chunk, diff_offset=0.3, verbose=0)
        rn = ref.nlpar_cpu.NLPAR(src, lam=0.8, searchradius=2)
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            rn.calcnlpar_cpu(fileout=theirs, chunksize=chunk, diff_offset=np.float32(0.3), verbose=0)
        assert open(mine, "rb").read() == open(theirs, "rb").read(), chunk


def test_diff_offsets_equal_the_oracles():
    """The product's vectorised centre-weight additions equal the oracle's step-by-step
    restatement of nlpar_nb's loops (itself checked against the reference above)."""
    from pyebsdindex_gb300.nlpar import _diff_offsets
    for nrows, ncols, sr, block in ((7, 9, 2, (0, 0, 9, 7)), (12, 10, 3, (3, 2, 5, 8)), (6, 6, 1, (1, 1, 4, 4))):
        a = _diff_offsets(nrows, ncols, sr, np.float32(0.37), block)
        b = no.diff_offsets(nrows, ncols, sr, np.float32(0.37), block)
        assert a.tobytes() == b.tobytes()


def test_backsub_matches_reference(tmp_path, ref, oracle_tiles, built_lib):
    """The fitted background (a Gaussian on a plane over the tile's mean pattern) as the
    reference's NLPAR.backsub computes it, alone and inside calcnlpar."""
    from pyebsdindex_gb300.nlpar import NLPAR
    pats = scan(7, 9, 20, 23)
    data = pats.astype(np.float32)
    mine = NLPAR(searchradius=1)
    mine.mask = mine.makeautomask(20, 20)
    theirs = ref.nlpar_cpu.NLPAR(searchradius=1)
    theirs.mask = theirs.makeautomask(20, 20)
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        want = theirs.backsub(data.copy())
    assert mine.backsub(data.copy()).tobytes() == want.tobytes()
    src = write("up1", str(tmp_path), pats, 7, 9)
    a, b = os.path.join(tmp_path, "a.up1"), os.path.join(tmp_path, "b.up1")
    NLPAR(src, lam=0.8, searchradius=1).calcnlpar(fileout=a, backsub=True, chunksize=50_000, verbose=0)
    rn = ref.nlpar_cpu.NLPAR(src, lam=0.8, searchradius=1)
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        rn.calcnlpar_cpu(fileout=b, backsub=True, chunksize=50_000, verbose=0)
    assert open(a, "rb").read() == open(b, "rb").read()


NLPARFILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nlparfile")


@pytest.mark.parametrize("name", ["onetile_9x11_16", "tiles_10x12_16"])
def test_calcnlpar_matches_committed_reference_run(tmp_path, oracle_tiles, built_lib, name):
    """The host logic on the committed reference runs (tests/golden/nlparfile/, made by
    tests/golden/make_nlpar_file_golden.py): output file and merged sigma identical, with no
    reference tree needed."""
    import json
    import shutil
    from pyebsdindex_gb300.nlpar import NLPAR
    p = json.load(open(os.path.join(NLPARFILE, name + ".json")))
    src = os.path.join(tmp_path, "in.up1")
    shutil.copyfile(os.path.join(NLPARFILE, name + "_in.up1"), src)
    out = os.path.join(tmp_path, "out.up1")
    nl = NLPAR(src, lam=p["lam"], searchradius=p["searchradius"])
    nl.calcnlpar(chunksize=p["chunksize"], fileout=out, verbose=0)
    assert open(out, "rb").read() == open(os.path.join(NLPARFILE, name + "_out.up1"), "rb").read()
    assert nl.sigma.tobytes() == np.load(os.path.join(NLPARFILE, name + "_sigma.npy")).tobytes()
