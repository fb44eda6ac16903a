"""EDAX UP1 / UP2 pattern files, read by libebsdgpu's parallel positional reader.

Mirrors the reference's ``ebsd_pattern.get_pattern_file_obj`` / ``UPFile`` (ebsd_pattern.py:33-60,
:208-330, :435-570): the same header attributes (``version``, ``patternW``, ``patternH``,
``filePos``, ``nPatterns``, ``nCols``, ``nRows``, ``extraPatterns``, ``hexflag``, ``xStep``,
``yStep``, ``filedatatype``) and the same ``read_data(patStartCount, convertToFloat,
returnArrayOnly)`` for a run of patterns ``[start, count]`` or a slab ``[[col, row], [ncol,
nrow]]``, returning the patterns and their scan positions.  The bytes are read by
``ebsd_up_read`` (several positional reads in parallel); ``BandDetect.find_bands_file`` streams
a file through ``ebsd_find_bands_file`` (reads, host-to-device copies and detection overlap).

``write_up`` writes a file in the layout ``UPFile.write_header`` / ``pat_writer`` produce
(ebsd_pattern.py:573-640).  The HDF5 formats (EDAX .oh5, Oxford .h5oina, Bruker, kikuchipy,
EMsoft) and Oxford .ebsp are not read here.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _lib

__all__ = ["get_pattern_file_obj", "UPFile", "EBSDPatterns", "write_up"]


class UPInfo(C.Structure):
    _fields_ = [("version", C.c_int32), ("W", C.c_int32), ("H", C.c_int32), ("bytes_per_px", C.c_int32),
                ("file_pos", C.c_int64), ("n_patterns", C.c_int64), ("n_cols", C.c_int64), ("n_rows", C.c_int64),
                ("extra_patterns", C.c_int32), ("hexflag", C.c_int32), ("x_step", C.c_double),
                ("y_step", C.c_double), ("file_bytes", C.c_int64)]


def _bind():
    lib = _lib.load()
    if not getattr(lib, "_up_bound", False):
        lib.ebsd_up_read_header.argtypes = [C.c_char_p, C.c_int, C.POINTER(UPInfo)]
        lib.ebsd_up_read_header.restype = C.c_int
        lib.ebsd_up_read.argtypes = [C.c_char_p, C.POINTER(UPInfo), C.c_int64, C.c_int64, C.c_void_p, C.c_int]
        lib.ebsd_up_read.restype = C.c_int
        lib.ebsd_find_bands_file.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int, C.c_int64, C.c_int64,
                                             C.POINTER(_lib.Bands), C.c_int64]
        lib.ebsd_find_bands_file.restype = C.c_int
        lib._up_bound = True
    return lib


def get_pattern_file_obj(path, file_type=''):
    """The reader for ``path`` (ebsd_pattern.py:33-60); UP1 / UP2 only."""
    p = np.atleast_1d(path)[0]
    ext = str.lower(Path(str(p)).suffix)
    ftype = str.upper(file_type)
    if ext in ('.up1', '.up2') or ftype == 'UP':
        f = UPFile(p)
        f.read_header()
        return f
    raise NotImplementedError(f"pattern files of type {ext or file_type!r} are not read here (UP1 / UP2 only)")


class EBSDPatterns:
    """What ``read_data`` returns without ``returnArrayOnly`` (ebsd_pattern.py:184-206)."""

    def __init__(self):
        self.vendor = None
        self.file = None
        self.filetype = None
        self.patternW = None
        self.patternH = None
        self.nFileCols = None
        self.nFileRows = None
        self.nPatterns = None
        self.hexflag = False
        self.xStep = None
        self.yStep = None
        self.patStart = None
        self.patterns = None
        self.xyLocations = None


class UPFile:
    """EDAX UP1 / UP2 reader with the reference ``UPFile`` interface."""

    def __init__(self, path=None):
        self.filepath = Path(str(np.atleast_1d(path)[0])).expanduser().resolve() if path is not None else None
        self.vendor = 'EDAX'
        self.filetype = 'UP'
        self.version = None
        self.nCols = None
        self.nRows = None
        self.nPatterns = None
        self.patternW = None
        self.patternH = None
        self.xStep = None
        self.yStep = None
        self.xyCenter = np.array([0.0, 0.0])
        self.datamax = None
        self.datamin = None
        self.hexflag = 0
        self.filedatatype = None
        self.filePos = None
        self.extraPatterns = 0
        self._info = None

    def read_header(self, path=None, bitdepth=None):
        if path is not None:
            self.filepath = Path(str(path)).expanduser().resolve()
        info = UPInfo()
        _lib.check(_bind().ebsd_up_read_header(str(self.filepath).encode(), int(bitdepth or 0), C.byref(info)),
                   "ebsd_up_read_header")
        self._info = info
        self.filedatatype = np.uint8 if info.bytes_per_px == 1 else np.uint16
        self.version = np.uint32(info.version)
        self.patternW = np.uint32(info.W)
        self.patternH = np.uint32(info.H)
        self.filePos = np.uint32(info.file_pos)
        if info.version == 1:
            self.nPatterns = np.int64(info.n_patterns)
            if self.xStep is None:
                self.xStep = 0.0
            if self.yStep is None:
                self.yStep = 0.0
            if self.nCols is None or self.nCols == 0:
                self.nCols = np.uint64(self.nPatterns)
            if self.nRows is None:
                self.nRows = np.uint64(np.floor(self.nPatterns / self.nCols))
        else:
            self.extraPatterns = np.uint8(info.extra_patterns)
            self.nCols = np.uint64(info.n_cols)
            self.nRows = np.uint64(info.n_rows)
            self.nPatterns = np.int64(self.nCols.astype(np.uint64) * self.nRows.astype(np.uint64))
            self.hexflag = np.uint8(info.hexflag)
            self.xStep = np.float64(info.x_step)
            self.yStep = np.float64(info.y_step)
        return 0

    def pat_reader(self, patStart=0, nPatToRead=1):
        """Patterns [patStart, patStart + nPatToRead) and their scan positions
        (ebsd_pattern.py:515-537)."""
        patStart, nPatToRead = int(patStart), int(nPatToRead)
        out = np.empty((nPatToRead, int(self.patternH), int(self.patternW)), dtype=self.filedatatype)
        _lib.check(_bind().ebsd_up_read(str(self.filepath).encode(), C.byref(self._info), patStart, nPatToRead,
                                        C.c_void_p(out.ctypes.data), 0), "ebsd_up_read")
        yx = np.unravel_index(np.arange(np.int64(patStart), np.int64(patStart + nPatToRead), dtype=np.uint64),
                              (np.int64(self.nRows), np.int64(self.nCols)))
        xyloc = np.array([yx[1], yx[0]]).T.copy().astype(np.float32)
        xyloc[:, 0] -= self.nCols * 0.5
        xyloc[:, 1] -= self.nRows * 0.5
        xyloc[:, 0] *= self.xStep
        xyloc[:, 1] *= self.yStep
        return out, xyloc

    def read_data(self, path=None, convertToFloat=False, patStartCount=[0, -1], returnArrayOnly=False):
        """ebsd_pattern.py:236-329: a run [start, count] (count -1: to the end) or a slab
        [[col, row], [ncol, nrow]] (negative sizes: to the edge), clamped to the file."""
        if path is not None:
            self.filepath = Path(str(path)).expanduser().resolve()
            self.read_header()
        if self.version is None:
            self.read_header()
        typeout = np.float32 if convertToFloat else self.filedatatype
        pse = np.asarray(patStartCount, dtype=np.int64)
        if pse.ndim == 1:
            patStart = np.int64(pse[0])
            nPatToRead = np.int64(pse[-1])
            if nPatToRead == -1:
                nPatToRead = np.int64(self.nPatterns - patStart)
            if nPatToRead == 0:
                nPatToRead = 1
            if (patStart + nPatToRead) > self.nPatterns:
                nPatToRead = np.int64(self.nPatterns - patStart)
            readpats, xyloc = self.pat_reader(patStart, nPatToRead)
            patterns = readpats.astype(typeout)
        else:
            colstart, ncolread = np.int64(pse[0, 0]), np.int64(pse[1, 0])
            rowstart, nrowread = np.int64(pse[0, 1]), np.int64(pse[1, 1])
            patStart = [colstart, rowstart]
            if ncolread < 0:
                ncolread = np.int64(self.nCols - colstart)
            if nrowread < 0:
                nrowread = np.int64(self.nRows - rowstart)
            if (colstart + ncolread) > self.nCols:
                ncolread = np.int64(self.nCols - colstart)
            if (rowstart + nrowread) > self.nRows:
                nrowread = np.int64(self.nRows - rowstart)
            nrowread, ncolread = np.uint64(nrowread), np.uint64(ncolread)
            nPatToRead = [ncolread, nrowread]
            patterns = np.zeros([np.int64(ncolread * nrowread), self.patternH, self.patternW], dtype=typeout)
            xyloc = np.zeros([np.int64(ncolread * nrowread), 2], dtype=np.float32)
            for i in range(int(nrowread)):
                pstart = np.int64(np.int64(np.int64(rowstart + i) * self.nCols) + colstart)
                pt, xy = self.read_data(convertToFloat=convertToFloat, patStartCount=[pstart, ncolread],
                                        returnArrayOnly=True)
                patterns[np.int64(i * ncolread):np.int64((i + 1) * ncolread)] = pt
                xyloc[np.int64(i * ncolread):np.int64((i + 1) * ncolread)] = xy
        if returnArrayOnly:
            return patterns, xyloc
        out = EBSDPatterns()
        out.vendor, out.file, out.filetype = self.vendor, Path(self.filepath).expanduser(), self.filetype
        out.patternW, out.patternH = self.patternW, self.patternH
        out.nFileCols, out.nFileRows = np.uint64(self.nCols), np.uint64(self.nRows)
        out.nPatterns = np.array(nPatToRead)
        out.hexflag, out.xStep, out.yStep = self.hexflag, self.xStep, self.yStep
        out.patStart = np.array(patStart)
        out.patterns, out.xyLocations = patterns, xyloc
        return out


def write_up(path, patterns, nCols=None, nRows=None, version=3, xStep=1.0, yStep=1.0, hexflag=0):
    """Write patterns [n, H, W] (uint8 -> .up1, uint16 -> .up2) in the reference's UP layout
    (UPFile.write_header / pat_writer, ebsd_pattern.py:573-640): version 3 carries the scan
    shape and steps and puts the first pattern at byte 42; version 1 at byte 16."""
    pats = np.asarray(patterns)
    if pats.ndim == 2:
        pats = pats[None]
    dt = np.uint8 if str(path).lower().endswith('.up1') else np.uint16
    pats = np.ascontiguousarray(pats, dtype=dt)
    n, h, w = pats.shape
    if nCols is None:
        nCols, nRows = n, 1
    if nRows is None:
        nRows = n // nCols
    with open(os.path.expanduser(str(path)), 'wb') as f:
        np.asarray(version, dtype=np.uint32).tofile(f)
        np.asarray(w, dtype=np.uint32).tofile(f)
        np.asarray(h, dtype=np.uint32).tofile(f)
        if version == 1:
            np.asarray(16, dtype=np.uint32).tofile(f)
        else:
            np.asarray(42, dtype=np.uint32).tofile(f)
            np.asarray(0, dtype=np.uint8).tofile(f)
            np.asarray(nCols, dtype=np.uint32).tofile(f)
            np.asarray(nRows, dtype=np.uint32).tofile(f)
            np.asarray(hexflag, dtype=np.uint8).tofile(f)
            np.asarray(xStep, dtype=np.float64).tofile(f)
            np.asarray(yStep, dtype=np.float64).tofile(f)
        pats.tofile(f)
