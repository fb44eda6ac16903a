"""EDAX UP1 / UP2 pattern files read by libebsdgpu (pyebsdindex_gb300/ebsd_pattern.py) against
the reference's own UPFile (ebsd_pattern.py:435-570, imported through oracle/refshim.py):
header attributes, runs and slabs of patterns, scan positions.  The reads are host code and
need no GPU."""
import os

import numpy as np
import pytest

from oracle import refshim


@pytest.fixture(scope="module")
def ref():
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    return refshim.load()


def make_file(tmp_path, name, n, h, w, dtype, version, ncols=None, nrows=None, step=(1.5, 2.25)):
    from pyebsdindex_gb300.ebsd_pattern import write_up
    import zlib
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    hi = 256 if dtype == np.uint8 else 4096
    pats = rng.integers(0, hi, size=(n, h, w)).astype(dtype)
    path = os.path.join(tmp_path, name)
    write_up(path, pats, nCols=ncols, nRows=nrows, version=version, xStep=step[0], yStep=step[1])
    return path, pats


CASES = [("a.up1", 60, 20, 24, np.uint8, 3, 10, 6), ("b.up2", 35, 16, 18, np.uint16, 3, 7, 5),
         ("c.up1", 23, 12, 12, np.uint8, 1, None, None), ("d.up2", 9, 10, 14, np.uint16, 1, None, None)]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_reader_matches_reference(tmp_path, ref, built_lib, case):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    name, n, h, w, dt, ver, nc, nr = case
    path, pats = make_file(tmp_path, name, n, h, w, dt, ver, nc, nr)
    mine = ep.get_pattern_file_obj(path)
    import importlib
    rp = importlib.import_module("pyebsdindex.ebsd_pattern")
    theirs = rp.get_pattern_file_obj(path)
    theirs.read_header()
    for a in ("version", "patternW", "patternH", "filePos", "nPatterns", "nCols", "nRows", "xStep", "yStep",
              "hexflag", "extraPatterns", "filedatatype"):
        assert np.all(np.asarray(getattr(mine, a)) == np.asarray(getattr(theirs, a))), a
        assert np.asarray(getattr(mine, a)).dtype == np.asarray(getattr(theirs, a)).dtype, a
    reads = [dict(patStartCount=[0, -1]), dict(patStartCount=[3, 5]), dict(patStartCount=[n - 2, 10]),
             dict(patStartCount=[4, 0]), dict(patStartCount=[1, 7], convertToFloat=True)]
    if ver == 3:
        reads += [dict(patStartCount=[[2, 1], [4, 3]]), dict(patStartCount=[[0, 0], [-1, -1]]),
                  dict(patStartCount=[[nc - 3, nr - 2], [10, 10]], convertToFloat=True)]
    for kw in reads:
        a, axy = mine.read_data(returnArrayOnly=True, **kw)
        b, bxy = theirs.read_data(returnArrayOnly=True, **kw)
        assert a.dtype == b.dtype and a.shape == b.shape, kw
        assert a.tobytes() == b.tobytes(), kw
        assert axy.tobytes() == bxy.tobytes(), kw
    obj = mine.read_data(patStartCount=[2, 3])
    want = theirs.read_data(patStartCount=[2, 3])
    assert np.array_equal(obj.patterns, want.patterns) and np.array_equal(obj.patStart, want.patStart)
    assert np.array_equal(obj.nPatterns, want.nPatterns)


def test_reader_round_trip_without_reference(tmp_path, built_lib):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    path, pats = make_file(tmp_path, "e.up2", 40, 32, 30, np.uint16, 3, 8, 5)
    f = ep.get_pattern_file_obj(path)
    got, xy = f.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    assert got.tobytes() == pats.tobytes()
    assert xy.shape == (40, 2)


def test_unreadable_files_raise(tmp_path, built_lib):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    with pytest.raises(NotImplementedError):
        ep.get_pattern_file_obj(os.path.join(tmp_path, "x.h5"))
    bad = os.path.join(tmp_path, "bad.up1")
    with open(bad, "wb") as fh:
        fh.write(b"\x02\x00")
    with pytest.raises(RuntimeError, match="pattern file"):
        ep.get_pattern_file_obj(bad)
    with pytest.raises(RuntimeError, match="pattern file"):
        ep.get_pattern_file_obj(os.path.join(tmp_path, "missing.up1"))


@pytest.mark.parametrize("version", [1, 3])
def test_writer_header_matches_reference_writer(tmp_path, ref, built_lib, version):
    """write_up lays out the header as the reference's UPFile.write_header (ebsd_pattern.py:573-620)."""
    import importlib
    from pyebsdindex_gb300.ebsd_pattern import write_up
    rp = importlib.import_module("pyebsdindex_gb300.ebsd_pattern")
    pats = np.arange(6 * 8 * 10, dtype=np.uint8).reshape(6, 8, 10)
    mine = os.path.join(tmp_path, "m.up1")
    write_up(mine, pats, nCols=3, nRows=2, version=version, xStep=0.5, yStep=0.25)
    refmod = importlib.import_module("pyebsdindex.ebsd_pattern")
    theirs = os.path.join(tmp_path, "t.up1")
    f = refmod.UPFile(theirs)
    f.version, f.patternW, f.patternH = version, 10, 8
    f.nCols, f.nRows, f.xStep, f.yStep = 3, 2, 0.5, 0.25
    f.extraPatterns, f.hexflag = 0, 0
    f.write_header(writeBlank=False)
    head = 16 if version == 1 else 42
    assert open(mine, "rb").read()[:head] == open(theirs, "rb").read()[:head]
    assert rp.get_pattern_file_obj(mine).read_data(patStartCount=[0, -1], returnArrayOnly=True)[0].tobytes() \
        == pats.tobytes()


def test_other_extension_with_bitdepth(tmp_path, built_lib):
    import shutil
    from pyebsdindex_gb300 import ebsd_pattern as ep
    path, pats = make_file(tmp_path, "f.up2", 12, 9, 11, np.uint16, 3, 4, 3)
    other = os.path.join(tmp_path, "scan.dat")
    shutil.copyfile(path, other)
    f = ep.UPFile(other)
    f.read_header(bitdepth=16)
    got, _ = f.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    assert got.dtype == np.uint16 and got.tobytes() == pats.tobytes()
    with pytest.raises(RuntimeError, match="invalid argument"):
        ep.UPFile(other).read_header()
