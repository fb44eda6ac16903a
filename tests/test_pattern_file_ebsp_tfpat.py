"""Oxford .ebsp and ThermoFisher .pat files read by libebsdgpu (ebsd_pf_read_header /
ebsd_pf_read, pyebsdindex_gb300/ebsd_pattern.py) against the reference's own EBSPFile and
TFPatFile (ebsd_pattern.py:709-1395, imported through oracle/refshim.py): header attributes,
runs and slabs of patterns, scan positions; the writers against the reference's writers byte
for byte.  Host code only, no GPU."""
import ctypes as C
import os
import warnings
import zlib

import numpy as np
import pytest

from oracle import refshim

EBSP_ATTRS = ("version", "patternW", "patternH", "filePos", "nPatterns", "nCols", "nRows", "xStep", "yStep",
              "filedatatype", "hasxypos")
TFPAT_ATTRS = ("version", "patternW", "patternH", "filePos", "nPatterns", "nCols", "nRows", "xStep", "yStep",
               "filedatatype", "bitdepth", "hasbackground", "isscan")


@pytest.fixture(scope="module")
def rp():
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    return refshim.pattern_module()


def patterns(name, n, h, w, dtype, hi):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    return rng.integers(0, hi, size=(n, h, w)).astype(dtype)


def same_attrs(mine, theirs, attrs):
    for a in attrs:
        m, t = getattr(mine, a), getattr(theirs, a)
        assert np.all(np.asarray(m) == np.asarray(t)), (a, m, t)
        assert np.asarray(m).dtype == np.asarray(t).dtype, (a, type(m), type(t))


def same_reads(mine, theirs, n):
    ncols, nrows = int(mine.nCols), int(mine.nRows)
    reads = [dict(patStartCount=[0, -1]), dict(patStartCount=[3, 5]), dict(patStartCount=[n - 2, 10]),
             dict(patStartCount=[4, 0]), dict(patStartCount=[1, 7], convertToFloat=True),
             dict(patStartCount=[[1, 1], [2, 2]]), dict(patStartCount=[[0, 0], [-1, -1]]),
             dict(patStartCount=[[ncols - 2, nrows - 2], [10, 10]], convertToFloat=True)]
    for kw in reads:
        a, axy = mine.read_data(returnArrayOnly=True, **kw)
        b, bxy = theirs.read_data(returnArrayOnly=True, **kw)
        assert a.dtype == b.dtype and a.shape == b.shape, kw
        assert a.tobytes() == b.tobytes(), kw
        assert axy.dtype == bxy.dtype and axy.tobytes() == bxy.tobytes(), kw


EBSP_CASES = [(v, xy, np.uint8) for v in (1, 2, 3, 4, 5) for xy in (True, False) if not (v == 1 and not xy)]
EBSP_CASES += [(3, True, np.uint16), (5, False, np.uint16)]


@pytest.mark.parametrize("version,xy,dtype", EBSP_CASES, ids=[f"v{c[0]}-{'xy' if c[1] else 'noxy'}-"
                                                               f"{np.dtype(c[2]).name}" for c in EBSP_CASES])
def test_ebsp_reader_matches_reference(tmp_path, rp, built_lib, version, xy, dtype):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    name = f"v{version}{xy}{np.dtype(dtype).name}.ebsp"
    pats = patterns(name, 35, 12, 14, dtype, 256 if dtype == np.uint8 else 4096)
    path = os.path.join(tmp_path, name)
    ep.write_ebsp(path, pats, nCols=7, nRows=5, xStep=0.5, yStep=0.75, version=version, hasxypos=xy)
    mine = ep.get_pattern_file_obj(path)
    theirs = rp.get_pattern_file_obj(path)
    same_attrs(mine, theirs, EBSP_ATTRS)
    same_reads(mine, theirs, 35)
    obj, want = mine.read_data(patStartCount=[2, 3]), theirs.read_data(patStartCount=[2, 3])
    assert np.array_equal(obj.patterns, want.patterns) and np.array_equal(obj.patStart, want.patStart)


@pytest.mark.parametrize("version", [2, 4])
def test_ebsp_pattern_not_stored(tmp_path, rp, built_lib, version):
    """A zero record position (a pattern not stored) reads as zeros, position (0, 0)."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns("ns", 24, 10, 10, np.uint8, 256)
    path = os.path.join(tmp_path, "ns.ebsp")
    ep.write_ebsp(path, pats, nCols=6, nRows=4, xStep=1.5, yStep=1.5, version=version)
    head = 9 if version >= 4 else 8
    with open(path, "r+b") as f:
        for k in (5, 17):
            f.seek(head + 8 * k)
            f.write(np.uint64(0).tobytes())
    mine = ep.get_pattern_file_obj(path)
    theirs = rp.get_pattern_file_obj(path)
    same_attrs(mine, theirs, EBSP_ATTRS)
    same_reads(mine, theirs, 24)
    got, xy = mine.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    assert not got[5].any() and not got[17].any() and not xy[5].any()
    keep = [i for i in range(24) if i not in (5, 17)]
    assert got[keep].tobytes() == pats[keep].tobytes()


@pytest.mark.parametrize("version,xy", [(1, True), (2, True), (2, False), (4, True), (4, False)])
def test_ebsp_writer_matches_reference_writer(tmp_path, rp, built_lib, version, xy):
    """write_ebsp writes the bytes EBSPFile.write_data writes for a new file (uint8 patterns:
    the reference's writer always writes 8-bit)."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns("w", 12, 9, 11, np.uint8, 256)
    mine, theirs = os.path.join(tmp_path, "m.ebsp"), os.path.join(tmp_path, "t.ebsp")
    ep.write_ebsp(mine, pats, nCols=4, nRows=3, xStep=0.5, yStep=0.75, version=version, hasxypos=xy)
    f = rp.EBSPFile(theirs)
    f.version = np.int64(version)  # numpy 2 refuses np.uint64 of a negative Python int
    f.nCols, f.nRows, f.nPatterns, f.patternW, f.patternH = 4, 3, 12, 11, 9
    f.xStep, f.yStep, f.hasxypos = 0.5, 0.75, xy
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        f.write_data(newpatterns=pats, patStartCount=[0, -1])
    assert open(mine, "rb").read() == open(theirs, "rb").read()


TFPAT_CASES = [(12, True, True, True), (16, False, True, False), (8, False, False, False)]


@pytest.mark.parametrize("bitdepth,background,isscan,sidecar", TFPAT_CASES)
def test_tfpat_reader_matches_reference(tmp_path, rp, built_lib, bitdepth, background, isscan, sidecar):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns(f"t{bitdepth}", 30, 11, 13, np.uint16, 1 << bitdepth)
    path = os.path.join(tmp_path, "scan.pat")
    back = np.arange(11 * 13, dtype=np.uint16).reshape(11, 13) if background else None
    ep.write_tfpat(path, pats, nCols=6, nRows=5, bitdepth=bitdepth, background=back, isscan=isscan)
    if sidecar:  # the step 45 bytes before the end of the .ebsd file of the same name
        with open(os.path.join(tmp_path, "scan.ebsd"), "wb") as f:
            f.write(b"\x01" * 20 + np.float64(0.35).tobytes() + b"\x02" * 37)
    mine = ep.get_pattern_file_obj(path)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        theirs = rp.get_pattern_file_obj(path)
    same_attrs(mine, theirs, TFPAT_ATTRS)
    assert (mine.xStep == 0.35) == sidecar
    if background:
        assert np.array_equal(mine.background, back) and np.array_equal(mine.background, theirs.background)
    same_reads(mine, theirs, 30)
    got, _ = mine.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    assert got.tobytes() == pats.tobytes()


@pytest.mark.parametrize("bitdepth,background", [(12, False), (16, True), (8, False)])
def test_tfpat_writer_matches_reference_writer(tmp_path, rp, built_lib, bitdepth, background):
    """write_tfpat writes the bytes TFPatFile.write_data writes for a new file (pixels clipped
    to the bit depth; the reference writes a zero background)."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns("tw", 12, 9, 11, np.uint16, 4096)
    mine, theirs = os.path.join(tmp_path, "m.pat"), os.path.join(tmp_path, "t.pat")
    ep.write_tfpat(mine, pats, nCols=4, nRows=3, bitdepth=bitdepth,
                   background=np.zeros((9, 11)) if background else None)
    f = rp.TFPatFile(theirs)
    f.version, f.nCols, f.nRows, f.nPatterns = 1, np.uint32(4), np.uint32(3), 12
    f.patternW, f.patternH, f.bitdepth, f.hasbackground = np.uint32(11), np.uint32(9), bitdepth, background
    f.filedatatype = np.uint16
    f.filePos = 25 + 11 * 9 * 2 if background else 25
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        f.write_data(newpatterns=pats, patStartCount=[0, -1])
    assert open(mine, "rb").read() == open(theirs, "rb").read()


def test_round_trips_without_reference(tmp_path, built_lib):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns("rt", 20, 16, 18, np.uint16, 4096)
    for v in (2, 5):
        path = os.path.join(tmp_path, f"r{v}.ebsp")
        ep.write_ebsp(path, pats, nCols=5, nRows=4, xStep=2.0, yStep=3.0, version=v)
        f = ep.get_pattern_file_obj(path)
        got, xy = f.read_data(patStartCount=[0, -1], returnArrayOnly=True)
        assert got.tobytes() == pats.tobytes()
        assert (int(f.nCols), int(f.nRows), float(f.xStep), float(f.yStep)) == (5, 4, 2.0, 3.0)
        assert np.array_equal(xy[6], [(1 - 2.5) * 2.0, (1 - 2.0) * 3.0])
    path = os.path.join(tmp_path, "r.pat")
    ep.write_tfpat(path, pats, nCols=5, nRows=4, bitdepth=12)
    f = ep.get_pattern_file_obj(path)
    got, xy = f.read_data(patStartCount=[[1, 2], [3, 2]], returnArrayOnly=True)
    assert got.tobytes() == pats.reshape(4, 5, 16, 18)[2:4, 1:4].tobytes()
    assert np.array_equal(xy[0], [1 - 2.5, 2 - 2.0])


def test_threaded_runs_equal_one_thread(tmp_path, built_lib):
    """Records read by several threads in runs through the bounce buffers (about 20 MB, so the
    reads split) equal a one-thread read, from any start."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns("big", 1600, 60, 100, np.uint16, 65536)
    for path, write in ((os.path.join(tmp_path, "big.ebsp"), lambda p: ep.write_ebsp(p, pats, nCols=40, nRows=40)),
                        (os.path.join(tmp_path, "big.pat"), lambda p: ep.write_tfpat(p, pats, nCols=40, nRows=40))):
        write(path)
        f = ep.get_pattern_file_obj(path)
        lib = ep._bind()
        pos = C.c_void_p(f.filePos.ctypes.data) if f.filetype == 'EBSP' else None
        for start, n, threads in ((0, 1600, 1), (0, 1600, 6), (333, 1111, 4), (1599, 1, 8)):
            out = np.zeros((n, 60, 100), np.uint16)
            aux = np.zeros((n, 16 if f.filetype == 'EBSP' else 8), np.uint8)
            rc = lib.ebsd_pf_read(str(f.filepath).encode(), C.byref(f._info), pos, start, n,
                                  C.c_void_p(out.ctypes.data), C.c_void_p(aux.ctypes.data), threads)
            assert rc == 0
            assert out.tobytes() == pats[start:start + n].tobytes(), (path, start, n, threads)
            if f.filetype == 'TFPAT':
                loc = aux.view(np.uint32)
                assert np.array_equal(loc[:, 0], np.arange(start, start + n) % 40)


def test_unsupported_and_broken_files_raise(tmp_path, built_lib):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    pats = patterns("bad", 6, 8, 8, np.uint8, 256)
    path = os.path.join(tmp_path, "c.ebsp")
    ep.write_ebsp(path, pats, version=3)
    with open(path, "r+b") as f:  # mark the first record compressed
        f.seek(8 + 8 * 6)
        f.write(np.uint32(1).tobytes())
    with pytest.raises(RuntimeError, match="format or version not read"):
        ep.get_pattern_file_obj(path)
    v0 = os.path.join(tmp_path, "v0.ebsp")
    with open(v0, "wb") as f:
        f.write(np.int64(0).tobytes() + b"\x00" * 64)
    with pytest.raises(RuntimeError, match="format or version not read"):
        ep.get_pattern_file_obj(v0)
    short = os.path.join(tmp_path, "s.pat")
    ep.write_tfpat(short, pats.astype(np.uint16), nCols=3, nRows=2)
    with open(short, "r+b") as f:
        f.truncate(25 + 2 * (8 + 128))
    f = ep.get_pattern_file_obj(short)  # the header promises 6 patterns, the file holds 2
    assert f.read_data(patStartCount=[0, 2], returnArrayOnly=True)[0].shape == (2, 8, 8)
    with pytest.raises(RuntimeError, match="pattern file"):
        f.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    with pytest.raises(ValueError, match="extension not recognized"):
        ep.get_pattern_file_obj(os.path.join(tmp_path, "x.tiff"))
    with pytest.raises(NotImplementedError):
        ep.get_pattern_file_obj(os.path.join(tmp_path, "x.h5oina"))


def test_ebsp_table_across_read_blocks(tmp_path, rp, built_lib):
    """More records than one 64 Ki-entry block of the position table, a pattern not stored
    beyond the first block: the header parse streams the table and agrees with the reference."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    n = 70_000
    pats = patterns("blocks", n, 4, 4, np.uint8, 256)
    path = os.path.join(tmp_path, "many.ebsp")
    ep.write_ebsp(path, pats, nCols=350, nRows=200, xStep=1.0, yStep=1.0, version=3)
    with open(path, "r+b") as f:
        f.seek(8 + 8 * 66_000)
        f.write(np.uint64(0).tobytes())
    mine = ep.get_pattern_file_obj(path)
    theirs = rp.get_pattern_file_obj(path)
    same_attrs(mine, theirs, EBSP_ATTRS)
    a, axy = mine.read_data(patStartCount=[65_990, 20], returnArrayOnly=True)
    b, bxy = theirs.read_data(patStartCount=[65_990, 20], returnArrayOnly=True)
    assert a.tobytes() == b.tobytes() and axy.tobytes() == bxy.tobytes()
    assert not a[10].any()


def test_ebsp_records_out_of_order(tmp_path, rp, built_lib):
    """Records stored in another order than the table (here reversed, with spacing gaps): every
    run breaks at each record and the reads still gather the right pixels and footers."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    n, h, w = 40, 6, 7
    pats = patterns("rev", n, h, w, np.uint8, 256)
    path = os.path.join(tmp_path, "rev.ebsp")
    table_end = 8 + 8 * n
    rec = 16 + h * w + 18
    pos = np.empty(n, np.uint64)
    with open(path, "wb") as f:
        f.write(np.uint64((1 << 64) - 2).tobytes())
        f.write(b"\0" * (8 * n))
        at = table_end
        for i in reversed(range(n)):
            pos[i] = at
            r, c = divmod(i, 8)
            f.write(np.array([0, h, w, h * w], np.uint32).tobytes() + pats[i].tobytes())
            f.write(b"\x01" + np.float64((c - 4.0) * 0.5).tobytes() + b"\x01" + np.float64((r - 2.5) * 0.5).tobytes())
            f.write(b"\xee" * (i % 3))  # uneven gaps between records
            at += rec + (i % 3)
        f.seek(8)
        f.write(pos.tobytes())
    mine = ep.get_pattern_file_obj(path)
    theirs = rp.get_pattern_file_obj(path)
    same_attrs(mine, theirs, EBSP_ATTRS)
    same_reads(mine, theirs, n)
    got, _ = mine.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    assert got.tobytes() == pats.tobytes()


def test_edge_cases(tmp_path, rp, built_lib):
    """A UP file holding no patterns, a one-pattern EBSP file (the reference's step guess
    indexes past its arrays there; here the y step is 0), a TFPAT file whose size is not a
    whole number of records (its count from the file size, rounded down), truncated headers."""
    from pyebsdindex_gb300 import ebsd_pattern as ep
    empty = os.path.join(tmp_path, "e.up1")
    ep.write_up(empty, np.zeros((0, 8, 8), np.uint8), nCols=0, nRows=0)
    mine, theirs = ep.get_pattern_file_obj(empty), rp.get_pattern_file_obj(empty)
    assert int(mine.nPatterns) == int(theirs.nPatterns) == 0
    a, _ = mine.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    b, _ = theirs.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    assert a.shape == b.shape == (0, 8, 8)

    one = os.path.join(tmp_path, "one.ebsp")
    ep.write_ebsp(one, patterns("one", 1, 5, 6, np.uint8, 256), version=2)
    f = ep.get_pattern_file_obj(one)
    assert int(f.nPatterns) == 1 and int(f.nCols) == 1 and int(f.nRows) == 1 and float(f.yStep) == 0.0
    with pytest.raises(IndexError):
        rp.get_pattern_file_obj(one)

    pats = patterns("frac", 9, 6, 5, np.uint16, 4096)
    odd = os.path.join(tmp_path, "odd.pat")
    ep.write_tfpat(odd, pats, nCols=3, nRows=3, isscan=False)
    with open(odd, "ab") as fh:
        fh.write(b"\x00" * 17)  # a partial record at the end
    mine, theirs = ep.get_pattern_file_obj(odd), rp.get_pattern_file_obj(odd)
    same_attrs(mine, theirs, TFPAT_ATTRS)
    assert int(mine.nPatterns) == 9

    for name, head in (("t.up1", b"\x03\x00\x00\x00\x10"), ("t.ebsp", b"\xfe\xff\xff\xff"), ("t.pat", b"\x01\x00\x00\x00\x02")):
        p = os.path.join(tmp_path, name)
        with open(p, "wb") as fh:
            fh.write(head)
        with pytest.raises(RuntimeError, match="pattern file"):
            ep.get_pattern_file_obj(p)
