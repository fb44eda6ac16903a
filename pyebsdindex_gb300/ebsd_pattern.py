"""EBSD pattern files -- EDAX UP1 / UP2, Oxford .ebsp, ThermoFisher .pat -- read by
libebsdgpu's parallel positional readers.

Mirrors the reference's ``ebsd_pattern.get_pattern_file_obj``, ``EBSDPatternFile``,
``UPFile``, ``EBSPFile`` and ``TFPatFile`` (ebsd_pattern.py:33-117, :208-433, :435-708,
:709-1088, :1090-1395): the same header attributes (``version``, ``patternW``, ``patternH``,
``filePos``, ``nPatterns``, ``nCols``, ``nRows``, ``xStep``, ``yStep``, ``filedatatype`` and
each format's own) and the same ``read_data(patStartCount, convertToFloat, returnArrayOnly)``
for a run of patterns ``[start, count]`` or a slab ``[[col, row], [ncol, nrow]]``, returning
the patterns and their scan positions.  The bytes are read by ``ebsd_up_read`` /
``ebsd_pf_read`` (several positional reads in parallel; the .ebsp and .pat records are read
in runs and their pixels gathered); ``BandDetect.find_bands_file`` streams any of the three
through ``ebsd_find_bands_file`` (reads, host-to-device copies and detection overlap).

``write_up``, ``write_ebsp`` and ``write_tfpat`` write files in the layouts the reference's
writers produce (ebsd_pattern.py:573-640, :960-1088, :1227-1300).  The HDF5 formats (EDAX
.oh5, Oxford .h5oina, Bruker, kikuchipy, EMsoft, DM5) are not read here.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _lib

__all__ = ["get_pattern_file_obj", "EBSDPatternFile", "UPFile", "EBSPFile", "TFPatFile", "EBSDPatterns",
           "write_up", "write_ebsp", "write_tfpat"]

EBSD_PF_EBSP = 2
EBSD_PF_TFPAT = 3


class UPInfo(C.Structure):
    _fields_ = [("version", C.c_int32), ("W", C.c_int32), ("H", C.c_int32), ("bytes_per_px", C.c_int32),
                ("file_pos", C.c_int64), ("n_patterns", C.c_int64), ("n_cols", C.c_int64), ("n_rows", C.c_int64),
                ("extra_patterns", C.c_int32), ("hexflag", C.c_int32), ("x_step", C.c_double),
                ("y_step", C.c_double), ("file_bytes", C.c_int64)]


class PFInfo(C.Structure):
    """ebsd_pf_info (include/ebsdgpu.h)."""
    _fields_ = [("format", C.c_int32), ("version", C.c_int32), ("W", C.c_int32), ("H", C.c_int32),
                ("bytes_per_px", C.c_int32), ("record_head", C.c_int32), ("n_patterns", C.c_int64),
                ("first_record", C.c_int64), ("record_bytes", C.c_int64), ("file_bytes", C.c_int64),
                ("has_xy", C.c_int32), ("xy_flag_bytes", C.c_int32), ("is_scan", C.c_int32),
                ("bitdepth", C.c_int32), ("has_background", C.c_int32), ("reserved", C.c_int32),
                ("n_cols", C.c_int64), ("n_rows", C.c_int64)]


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
        lib.ebsd_pf_read_header.argtypes = [C.c_char_p, C.POINTER(PFInfo)]
        lib.ebsd_pf_read_header.restype = C.c_int
        lib.ebsd_pf_read_positions.argtypes = [C.c_char_p, C.POINTER(PFInfo), C.c_void_p]
        lib.ebsd_pf_read_positions.restype = C.c_int
        lib.ebsd_pf_read.argtypes = [C.c_char_p, C.POINTER(PFInfo), C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                     C.c_void_p, C.c_int]
        lib.ebsd_pf_read.restype = C.c_int
        lib._up_bound = True
    return lib


def get_pattern_file_obj(path, file_type=''):
    """The reader for ``path`` by extension or ``file_type`` (ebsd_pattern.py:33-117): UP1 / UP2,
    TFPAT (.pat) and EBSP (.ebsp); the HDF5 formats raise NotImplementedError, an unknown
    extension ValueError as in the reference."""
    p = np.atleast_1d(path)[0]
    ftype = str.upper(file_type)
    if ftype == '':
        ext = str.lower(Path(str(p)).suffix)
        kinds = {'.up1': 'UP1', '.up2': 'UP2', '.pat': 'TFPAT', '.ebsp': 'EBSP', '.oh5': 'OH5', '.h5': 'H5',
                 '.h5oina': 'H5OINA', '.dm5': 'DM5'}
        if ext not in kinds:
            raise ValueError('Error: extension not recognized')
        ftype = kinds[ext]
    if ftype in ('UP1', 'UP2', 'UP'):
        f = UPFile(p)
    elif ftype == 'TFPAT':
        f = TFPatFile(p)
    elif ftype == 'EBSP':
        f = EBSPFile(p)
    else:
        raise NotImplementedError(f"pattern files of type {ftype!r} are not read here (UP1 / UP2, EBSP, TFPAT)")
    f.read_header()
    return f


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


def pat_flt2int(patterns, typeout=None, method='clip', scalevalue=0.98, maxScale=None):
    """Patterns [n, H, W] (or one [H, W]) as an unsigned integer type (ebsd_pattern.py:118-182).
    ``typeout`` None picks uint16 when the largest value is above 258, else uint8; a floating
    type returns the patterns cast to it.  Methods: 'clip' -- clipped to [0, top] (top the
    type's largest value, or maxScale if smaller), truncated by the cast; 'fullscale' -- the
    minimum moved to 0, then scaled so that maxScale (default: the largest value) maps to
    scalevalue * top, clipped and rounded; 'scale' -- a negative minimum lifted to 0, then
    scaled the same way and rounded.  Another method gives zeros."""
    arr = patterns.patterns if isinstance(patterns, EBSDPatterns) else patterns
    if arr.ndim == 2:
        arr = arr.reshape(1, arr.shape[0], arr.shape[1])
    lo_val, hi_val = arr.min(), arr.max()
    if typeout is None:
        typeout = np.uint16 if hi_val > 258 else np.uint8
    if isinstance(typeout(0), np.floating):
        return arr.astype(typeout)
    top = 65535 if isinstance(typeout(0), np.uint16) else 255
    if isinstance(typeout(0), np.uint16):
        typeout = np.uint16
    if method == 'clip':
        ceiling = top if maxScale is None else min(maxScale, top)
        return np.ascontiguousarray(arr.clip(0, ceiling).astype(typeout))
    if method not in ('fullscale', 'scale'):
        return np.zeros(arr.shape, dtype=typeout)
    work = arr.astype(np.float32)
    if method == 'fullscale':
        work = work - lo_val
    elif lo_val < 0:
        work += 0 - lo_val
    peak = work.max() if maxScale is None else maxScale
    work *= scalevalue * top / peak
    if method == 'fullscale':
        work = work.clip(0, top)
    return np.ascontiguousarray(np.around(work).astype(typeout))


class EBSDPatternFile:
    """What every pattern-file reader shares (ebsd_pattern.py:208-433): the path, the scan
    attributes, ``read_data`` over a format's ``pat_reader``."""

    def __init__(self, path=None, filetype=None):
        self.filepath = None
        self.set_filepath(path)
        self.vendor = None
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
        self.hexflag = False
        self.filetype = filetype
        self.filedatatype = np.uint8

    def set_filepath(self, path=None):
        if path is not None:
            self.filepath = Path(str(np.atleast_1d(path)[0])).expanduser().resolve()

    def read_header(self, path=None, bitdepth=None):
        raise NotImplementedError

    def pat_reader(self, patStart=0, nPatToRead=1):
        raise NotImplementedError

    def set_scan_rc(self, rc=(0, 0)):
        """For files that do not record the scan shape (ebsd_pattern.py:419-422)."""
        self.nCols = np.uint64(rc[1])
        self.nRows = np.uint64(rc[0])
        self.nPatterns = np.uint64(self.nCols * self.nRows)

    def copy_obj(self):
        import copy
        return copy.deepcopy(self)

    def read_data(self, path=None, convertToFloat=False, patStartCount=[0, -1], returnArrayOnly=False):
        """Patterns from the file (ebsd_pattern.py:236-329), as float32 with ``convertToFloat``.
        ``patStartCount``: a run [start, count] (count -1: to the end, 0: one pattern) or a slab
        [[col, row], [ncol, nrow]] of the scan (a negative size: to the edge), clamped to the
        file.  Returns (patterns, xy locations), or with ``returnArrayOnly`` False an
        ``EBSDPatterns`` that also carries the file's scan attributes and the request."""
        if path is not None:
            self.set_filepath(path)
            self.read_header()
        if self.version is None:
            self.read_header()
        typeout = np.float32 if convertToFloat else self.filedatatype
        req = np.asarray(patStartCount, dtype=np.int64)
        if req.ndim == 1:
            start, count = self._clamp_run(req[0], req[-1])
            raw, xyloc = self.pat_reader(start, count)
            patterns, origin, extent = raw.astype(typeout), start, count
        else:
            origin, extent, patterns, xyloc = self._read_slab(req, typeout, convertToFloat)
        if returnArrayOnly:
            return patterns, xyloc
        out = EBSDPatterns()
        out.vendor, out.file, out.filetype = self.vendor, Path(self.filepath).expanduser(), self.filetype
        out.patternW, out.patternH = self.patternW, self.patternH
        out.nFileCols, out.nFileRows = np.uint64(self.nCols), np.uint64(self.nRows)
        out.nPatterns = np.array(extent)
        out.hexflag, out.xStep, out.yStep = self.hexflag, self.xStep, self.yStep
        out.patStart = np.array(origin)
        out.patterns, out.xyLocations = patterns, xyloc
        return out

    def _clamp_run(self, start, count):
        """A run request clamped to the file: count -1 reads to the end, 0 reads one pattern."""
        start, count = np.int64(start), np.int64(count)
        if count == -1:
            count = np.int64(self.nPatterns - start)
        if count == 0:
            count = np.int64(1)
        if start + count > self.nPatterns:
            count = np.int64(self.nPatterns - start)
        return start, count

    def _read_slab(self, req, typeout, convertToFloat):
        """A [[col, row], [ncol, nrow]] block of the scan, one run read per scan row."""
        col0, row0 = np.int64(req[0, 0]), np.int64(req[0, 1])
        ncol, nrow = np.int64(req[1, 0]), np.int64(req[1, 1])
        ncol = np.int64(self.nCols - col0) if ncol < 0 else ncol
        nrow = np.int64(self.nRows - row0) if nrow < 0 else nrow
        ncol = min(ncol, np.int64(self.nCols - col0))
        nrow = min(nrow, np.int64(self.nRows - row0))
        ncol, nrow = np.uint64(ncol), np.uint64(nrow)
        total = np.int64(ncol * nrow)
        patterns = np.zeros([total, self.patternH, self.patternW], dtype=typeout)
        xyloc = np.zeros([total, 2], dtype=np.float32)
        width = int(ncol)
        for r in range(int(nrow)):
            first = np.int64(np.int64(np.int64(row0 + r) * self.nCols) + col0)
            pats, xy = self.read_data(convertToFloat=convertToFloat, patStartCount=[first, ncol], returnArrayOnly=True)
            patterns[r * width:(r + 1) * width] = pats
            xyloc[r * width:(r + 1) * width] = xy
        return [col0, row0], [ncol, nrow], patterns, xyloc

    def write_data(self, newpatterns=None, patStartCount=[0, -1], writeHead=False, flt2int='clip', scalevalue=0.98,
                   maxScale=None):
        """Write patterns into the file (ebsd_pattern.py:335-400): a run [start, count] (count -1:
        all given patterns) or a slab [[col, row], [ncol, nrow]], converted to the file's pixel
        type by ``pat_flt2int``.  The file must exist (``copy_file``, or write_up / write_ebsp /
        write_tfpat for a new one)."""
        if not os.path.isfile(self.filepath):
            raise FileNotFoundError(f"{self.filepath}: create the file first (copy_file or write_up / write_ebsp / "
                                    "write_tfpat)")
        if isinstance(newpatterns, EBSDPatterns):
            pats = newpatterns.patterns
        else:
            pats = np.asarray(newpatterns)
            if pats.ndim == 2:
                pats = pats.reshape(1, pats.shape[0], pats.shape[1])
        npats = pats.shape[0]
        mx = pats.max() if maxScale is None else maxScale
        pse = np.asarray(patStartCount)
        if pse.ndim == 1:
            patStart = np.int64(pse[0])
            nPatToWrite = np.int64(pse[-1])
            if nPatToWrite == -1:
                nPatToWrite = npats
            if nPatToWrite == 0:
                nPatToWrite = 1
            if (patStart + nPatToWrite) > self.nPatterns:
                nPatToWrite = self.nPatterns - patStart
            pat2write = pat_flt2int(pats, typeout=self.filedatatype, method=flt2int, scalevalue=scalevalue,
                                    maxScale=None)
            self.pat_writer(pat2write, int(patStart), int(nPatToWrite), self.filedatatype)
        else:
            colstart, ncolwrite = np.int64(pse[0, 0]), np.int64(pse[1, 0])
            rowstart, nrowwrite = np.int64(pse[0, 1]), np.int64(pse[1, 1])
            if ncolwrite < 0:
                ncolwrite = np.int64(self.nCols - colstart)
            if nrowwrite < 0:
                nrowwrite = np.int64(self.nRows - rowstart)
            if (colstart + ncolwrite) > self.nCols:
                ncolwrite = np.int64(self.nCols - colstart)
            if (rowstart + nrowwrite) > self.nRows:
                nrowwrite = np.int64(self.nRows - rowstart)
            for i in range(int(nrowwrite)):
                pstart = np.int64(np.int64(np.int64(rowstart + i) * self.nCols) + colstart)
                self.write_data(newpatterns=pats[int(i * ncolwrite):int((i + 1) * ncolwrite)],
                                patStartCount=[pstart, ncolwrite], writeHead=False, flt2int=flt2int,
                                scalevalue=0.98, maxScale=mx)

    def pat_writer(self, pat2write, patStart, nPatToWrite, typewrite):
        raise NotImplementedError

    def copy_file(self, newpath, **kwargs):
        """A copy of the file at ``newpath`` (default: the path + '.copy'), ebsd_pattern.py:402-410."""
        import shutil
        src = Path(self.filepath).expanduser().resolve()
        dst = Path(str(np.atleast_1d(newpath)[0])).expanduser().resolve() if newpath is not None \
            else Path(str(src) + '.copy')
        shutil.copyfile(src, dst)

    def _copy_header_only(self, newpath, head_bytes):
        """Header bytes copied, the rest of the file's length zero-filled (UPFile / TFPatFile
        copy_file with empty_data)."""
        src = Path(self.filepath).expanduser().resolve()
        dst = Path(str(np.atleast_1d(newpath)[0])).expanduser().resolve() if newpath is not None \
            else Path(str(src) + '.copy')
        with open(src, 'rb') as f:
            head = f.read(int(head_bytes))
            size = f.seek(0, 2)
        with open(dst, 'wb') as f:
            f.write(head)
            f.seek(size - 1, 0)
            f.write(b"\0")
        return dst

    def read_datamaxmin(self):  # files without stored data limits
        pass

    def write_datamaxmin(self):
        pass


class UPFile(EBSDPatternFile):
    """EDAX UP1 / UP2 reader with the reference ``UPFile`` interface."""

    def __init__(self, path=None):
        EBSDPatternFile.__init__(self, path, 'UP')
        self.vendor = 'EDAX'
        self.hexflag = 0
        self.filedatatype = None
        self.filePos = None
        self.extraPatterns = 0
        self._info = None

    def read_header(self, path=None, bitdepth=None):
        self.set_filepath(path)
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


    def pat_writer(self, pat2write, patStart, nPatToWrite, typewrite):
        """Patterns [patStart, patStart + nPatToWrite) in place (ebsd_pattern.py:622-635)."""
        per = int(self.patternW) * int(self.patternH) * np.dtype(typewrite).itemsize
        with open(self.filepath, 'r+b') as f:
            f.seek(per * int(patStart) + int(self.filePos))
            np.ascontiguousarray(pat2write[0:nPatToWrite], dtype=typewrite).tofile(f)

    def copy_file(self, newpath, **kwargs):
        """UPFile.copy_file (ebsd_pattern.py:680-706): with empty_data the header and a
        zero-filled body of the same length."""
        if kwargs.get('empty_data', False):
            self._copy_header_only(newpath, self.filePos)
            return
        EBSDPatternFile.copy_file(self, newpath)


class EBSPFile(EBSDPatternFile):
    """Oxford .ebsp reader with the reference ``EBSPFile`` interface (ebsd_pattern.py:709-958).
    Uncompressed files of versions 1-5; compressed files and version 0 raise (the reference
    does not read them either).  Where the reference's scan-shape guess indexes past the end
    (a single pattern, or one row of patterns), ``yStep`` is 0 here instead of an IndexError."""

    def __init__(self, path=None):
        EBSDPatternFile.__init__(self, path, 'EBSP')
        self.vendor = 'OXFORD'
        self.filedatatype = None
        self.filePos = None
        self.hasxypos = False
        self._info = None

    def read_header(self, path=None, bitdepth=None):
        """ebsd_pattern.py:724-918: version, record positions, pattern size and pixel type from
        the first record, then the scan shape and steps from the records' x, y footers."""
        self.set_filepath(path)
        lib = _bind()
        info = PFInfo()
        name = str(self.filepath).encode()
        _lib.check(lib.ebsd_pf_read_header(name, C.byref(info)), "ebsd_pf_read_header")
        self._info = info
        self.version = np.int64(info.version)
        pos = np.empty(int(info.n_patterns), dtype=np.uint64)
        _lib.check(lib.ebsd_pf_read_positions(name, C.byref(info), C.c_void_p(pos.ctypes.data)),
                   "ebsd_pf_read_positions")
        self.filePos = pos
        self.nPatterns = np.int64(info.n_patterns)
        self.patternW = np.uint32(info.W)
        self.patternH = np.uint32(info.H)
        self.filedatatype = {1: np.uint8, 2: np.uint16, 4: np.uint32}[info.bytes_per_px]
        self.hasxypos = bool(info.has_xy)
        self.nCols = self.nRows = self.xStep = self.yStep = None
        if not self.hasxypos:
            self.xStep = 1.0
            self.yStep = 1.0
            self.nCols = 1
            self.nRows = self.nPatterns
        else:
            xy = np.zeros((int(self.nPatterns), 2), dtype=np.float64)
            _lib.check(lib.ebsd_pf_read(name, C.byref(info), C.c_void_p(pos.ctypes.data), 0, int(self.nPatterns),
                                        None, C.c_void_p(xy.ctypes.data), 0), "ebsd_pf_read")
            xall, yall = xy[:, 0], xy[:, 1]
            self.xStep = xall[1] - xall[0] if xall.size > 1 else np.float64(0.0)
            if self.xStep > 1e-6:
                ncol = np.round((xall.max() - xall.min()) / self.xStep + 1)
            else:
                ncol = 1
            self.nCols = np.uint64(ncol)
            k = int(self.nCols)
            self.yStep = np.abs(yall[0] - yall[k]) if k < yall.size else np.float64(0.0)
            if self.yStep > 1e-6:
                nrow = np.round((yall.max() - yall.min()) / self.yStep + 1)
                self.nRows = np.int64(nrow)
            else:
                self.nRows = np.int64(self.nPatterns / self.nCols + 0.001)
        if self.nCols == 0:
            self.nCols = np.uint64(1)
        return 0

    def pat_reader(self, patStart=0, nPatToRead=1):
        """Patterns [patStart, patStart + nPatToRead) (zeros where a pattern is not stored) and
        their x, y from the record footers (float64; zeros without footers),
        ebsd_pattern.py:920-958."""
        patStart, nPatToRead = int(patStart), int(nPatToRead)
        out = np.empty((nPatToRead, int(self.patternH), int(self.patternW)), dtype=self.filedatatype)
        xyloc = np.zeros((nPatToRead, 2), dtype=np.float64)
        _lib.check(_bind().ebsd_pf_read(str(self.filepath).encode(), C.byref(self._info),
                                        C.c_void_p(self.filePos.ctypes.data), patStart, nPatToRead,
                                        C.c_void_p(out.ctypes.data), C.c_void_p(xyloc.ctypes.data), 0),
                   "ebsd_pf_read")
        return out, xyloc


    def pat_writer(self, pat2write, patStart, nPatToWrite, typewrite):
        """Records of patterns [patStart, patStart + nPatToWrite) in place: the record header,
        the pixels and, with positions, the footer of x, y relative to the scan centre
        (EBSPFile.pat_writer, ebsd_pattern.py:1055-1088; version-5 files get their 6-word
        header back).  Patterns that are not stored are skipped.  Records that follow one
        another in the file are packed into one array and written with one call."""
        h, w = int(self.patternH), int(self.patternW)
        pdt = np.dtype(typewrite)
        nbytes = h * w * np.dtype(self.filedatatype).itemsize
        words = 6 if int(self.version) >= 5 else 4
        flag = 1 if int(self.version) >= 2 else 0
        names, formats, offsets = ['head', 'pix'], [(np.uint32, (words,)), (pdt, (h * w,))], [0, 4 * words]
        size = 4 * words + h * w * pdt.itemsize
        if self.hasxypos:
            if flag:
                names += ['fx', 'x', 'fy', 'y']
                formats += [np.uint8, np.float64, np.uint8, np.float64]
                offsets += [size, size + 1, size + 9, size + 10]
                size += 18
            else:
                names += ['x', 'y']
                formats += [np.float64, np.float64]
                offsets += [size, size + 8]
                size += 16
        rec = np.dtype({'names': names, 'formats': formats, 'offsets': offsets, 'itemsize': size})
        p0, n = int(patStart), int(nPatToWrite)
        pos = np.asarray(self.filePos[p0:p0 + n], dtype=np.int64)
        idx = np.arange(p0, p0 + n)
        pats = np.asarray(pat2write[0:n]).reshape(n, h * w)
        with open(self.filepath, 'r+b') as f:
            k = 0
            while k < n:
                if pos[k] <= 0:
                    k += 1
                    continue
                e = k + 1
                while e < n and pos[e] == pos[e - 1] + size:
                    e += 1
                out = np.zeros(e - k, dtype=rec)
                out['head'][:, -3:] = (h, w, nbytes)
                out['pix'] = pats[k:e]
                if self.hasxypos:
                    row, col = np.divmod(idx[k:e], int(self.nCols))
                    out['x'] = (col.astype(np.float64) - float(self.nCols * 0.5)) * self.xStep
                    out['y'] = (row.astype(np.float64) - float(self.nRows * 0.5)) * self.yStep
                    if flag:
                        out['fx'] = 1
                        out['fy'] = 1
                f.seek(int(pos[k]))
                out.tofile(f)
                k = e


class TFPatFile(EBSDPatternFile):
    """ThermoFisher .pat reader with the reference ``TFPatFile`` interface
    (ebsd_pattern.py:1090-1225, :1302-1322): uint16 patterns whatever the header's bit depth,
    the stored background pattern, the step from a ``.ebsd`` file of the same name when there
    is one."""

    def __init__(self, path=None):
        EBSDPatternFile.__init__(self, path, 'TFPAT')
        self.vendor = 'THERMOFISHER'
        self.filedatatype = None
        self.bitdepth = 8
        self.filePos = None
        self.hasxypos = False
        self.hasbackground = True
        self.background = None
        self.isscan = True
        self.xypx = None
        self.xStep = 1.0
        self.yStep = 1.0
        self._info = None

    def read_header(self, path=None, bitdepth=None):
        """ebsd_pattern.py:1113-1167."""
        self.set_filepath(path)
        info = PFInfo()
        _lib.check(_bind().ebsd_pf_read_header(str(self.filepath).encode(), C.byref(info)), "ebsd_pf_read_header")
        self._info = info
        self.version = np.uint32(info.version)
        self.filedatatype = np.uint16
        self.nCols = np.uint32(info.n_cols)
        self.nRows = np.uint32(info.n_rows)
        self.patternW = np.uint32(info.W)
        self.patternH = np.uint32(info.H)
        self.bitdepth = np.uint8(info.bitdepth)
        self.hasbackground = bool(info.has_background)
        self.filePos = np.uint32(info.first_record) if self.hasbackground else 25
        self.nPatterns = np.int64(info.n_patterns)
        if self.hasbackground:
            self.background = self.read_backgroundpattern()
        self.read_stepsize()
        return 0

    def read_stepsize(self):
        """The step from the float64 45 bytes before the end of the ``.ebsd`` file of the same
        name, kept when 0 < step < 2000 (ebsd_pattern.py:1169-1187)."""
        side = Path(str(self.filepath)).with_suffix('.ebsd')
        if not side.is_file() or side.stat().st_size < 45:
            return -1
        with open(side, 'rb') as f:
            f.seek(-45, 2)
            step = np.frombuffer(f.read(8), dtype=np.float64)
        if (step > 0) and (step < 2000):
            self.xStep = step[0]
            self.yStep = step[0]
        return 0

    def read_backgroundpattern(self):
        """The stored background pattern, uint16 [H, W] at byte 25 (ebsd_pattern.py:1302-1322)."""
        if self.patternW is None or self.patternH is None:
            self.read_header()
        if not self.hasbackground:
            return -1
        n = int(self.patternW) * int(self.patternH)
        with open(self.filepath, 'rb') as f:
            f.seek(25)
            back = np.frombuffer(f.read(2 * n), dtype=np.uint16)
        if back.size != n:
            raise RuntimeError("pattern file: background pattern past the end of the file")
        return back.reshape(int(self.patternH), int(self.patternW)).copy()

    def get_backgroundpattern(self):
        return self.background

    def pat_reader(self, patStart=0, nPatToRead=1):
        """Patterns [patStart, patStart + nPatToRead) and their positions: the records' pixel
        locations relative to the scan centre, times the step (float32), ebsd_pattern.py:1190-1225."""
        patStart, nPatToRead = int(patStart), int(nPatToRead)
        out = np.empty((nPatToRead, int(self.patternH), int(self.patternW)), dtype=np.uint16)
        loc = np.empty((nPatToRead, 2), dtype=np.uint32)
        _lib.check(_bind().ebsd_pf_read(str(self.filepath).encode(), C.byref(self._info), None, patStart, nPatToRead,
                                        C.c_void_p(out.ctypes.data), C.c_void_p(loc.ctypes.data), 0),
                   "ebsd_pf_read")
        xyloc = loc.astype(np.float32)
        xyloc[:, 0] -= self.nCols * 0.5
        xyloc[:, 1] -= self.nRows * 0.5
        xyloc[:, 0] *= self.xStep
        xyloc[:, 1] *= self.yStep
        return out, xyloc


    def pat_writer(self, pat2write, patStart, nPatToWrite, typewrite=None, bitdepth=None):
        """Records of patterns [patStart, patStart + nPatToWrite) in place: (column, row) and
        the pixels clipped to 2**bitdepth - 1 (TFPatFile.pat_writer, ebsd_pattern.py:1266-1300)."""
        bitdepth = int(self.bitdepth if bitdepth is None else bitdepth)
        h, w = int(self.patternH), int(self.patternW)
        n = int(nPatToWrite)
        recs = np.empty(n, dtype=np.dtype([('loc', np.uint32, (2,)), ('pat', np.uint16, (h, w))]))
        idx = np.arange(int(patStart), int(patStart) + n)
        recs['loc'][:, 0] = idx % int(self.nCols)
        recs['loc'][:, 1] = idx // int(self.nCols)
        recs['pat'] = pat_flt2int(np.asarray(pat2write[0:n]), typeout=np.uint16, method='clip',
                                  maxScale=(1 << bitdepth) - 1)
        with open(self.filepath, 'r+b') as f:
            f.seek(int(self.filePos) + int(patStart) * (h * w * 2 + 8))
            recs.tofile(f)
        return 0

    def copy_file(self, newpath, **kwargs):
        """TFPatFile.copy_file (ebsd_pattern.py:1327-1360): with empty_data the header (and
        background) and a zero-filled body; the .ebsd file of the same name is copied along."""
        import shutil
        src = Path(self.filepath).expanduser().resolve()
        if kwargs.get('empty_data', False):
            dst = self._copy_header_only(newpath, self.filePos)
        else:
            dst = Path(str(np.atleast_1d(newpath)[0])).expanduser().resolve() if newpath is not None \
                else Path(str(src) + '.copy')
            shutil.copyfile(src, dst)
        side = src.with_suffix('.ebsd')
        if side.exists():
            shutil.copyfile(side, Path(dst).with_suffix('.ebsd'))


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


def _scan_shape(n, nCols, nRows):
    if nCols is None:
        nCols, nRows = n, 1
    if nRows is None:
        nRows = n // nCols
    if int(nCols) * int(nRows) != n:
        raise ValueError("nCols * nRows must equal the number of patterns")
    return int(nCols), int(nRows)


def write_ebsp(path, patterns, nCols=None, nRows=None, xStep=1.0, yStep=1.0, version=2, hasxypos=True):
    """Write patterns [n, H, W] (uint8 or uint16) as an Oxford .ebsp file.  Versions 1-4 in the
    layout EBSPFile.write_header / pat_writer produce (ebsd_pattern.py:960-1088): minus the
    version as an int64, from version 4 one zero byte, the table of record positions, then per
    pattern a record header (0, H, W, pixel bytes as uint32), the pixels, and the footer -- x,
    y (float64) of the pattern relative to the scan centre, each behind a flag byte 1 from
    version 2, or a single flag byte 0 without positions (version 1 always has them).
    Version 5 (6-word record headers: 0, 0, 0, H, W, pixel bytes) is laid out as
    EBSPFile.read_header reads it: the table ends in an entry H + (W << 32)."""
    pats = np.asarray(patterns)
    if pats.ndim == 2:
        pats = pats[None]
    if pats.dtype not in (np.uint8, np.uint16):
        raise ValueError("patterns must be uint8 or uint16")
    pats = np.ascontiguousarray(pats)
    n, h, w = pats.shape
    nCols, nRows = _scan_shape(n, nCols, nRows)
    version = int(version)
    if not 1 <= version <= 5:
        raise ValueError("version must be 1-5")
    if version == 1:
        hasxypos = True
    words = 6 if version >= 5 else 4
    nbytes = h * w * pats.dtype.itemsize
    footer = (16 if version == 1 else 18) if hasxypos else 1
    head = 9 if version >= 4 else 8
    table_end = head + 8 * n + (8 if version >= 5 else 0)
    rec = 4 * words + nbytes + footer
    pos = np.arange(n, dtype=np.uint64) * np.uint64(rec) + np.uint64(table_end)
    base = 4 * words + nbytes
    names, formats, offsets = ['head', 'pix'], [(np.uint32, (words,)), (pats.dtype, (h * w,))], [0, 4 * words]
    if not hasxypos:
        names, formats, offsets = names + ['flag'], formats + [np.uint8], offsets + [base]
    elif version >= 2:
        names += ['fx', 'x', 'fy', 'y']
        formats += [np.uint8, np.float64, np.uint8, np.float64]
        offsets += [base, base + 1, base + 9, base + 10]
    else:
        names += ['x', 'y']
        formats += [np.float64, np.float64]
        offsets += [base, base + 8]
    recs = np.zeros(n, dtype=np.dtype({'names': names, 'formats': formats, 'offsets': offsets, 'itemsize': rec}))
    recs['head'][:, -3:] = (h, w, nbytes)
    recs['pix'] = pats.reshape(n, h * w)
    if hasxypos:
        col = np.arange(n) % nCols
        row = np.arange(n) // nCols
        recs['x'] = (col.astype(np.float64) - float(nCols * 0.5)) * xStep
        recs['y'] = (row.astype(np.float64) - float(nRows * 0.5)) * yStep
        if version >= 2:
            recs['fx'] = 1
            recs['fy'] = 1
    with open(os.path.expanduser(str(path)), 'wb') as f:
        f.write(np.uint64((1 << 64) - version).tobytes())
        if version >= 4:
            f.write(b'\x00')
        f.write(pos.tobytes())
        if version >= 5:
            f.write(np.uint64(h + (w << 32)).tobytes())
        recs.tofile(f)


def write_tfpat(path, patterns, nCols=None, nRows=None, bitdepth=16, background=None, version=1, isscan=True):
    """Write uint16 patterns [n, H, W] as a ThermoFisher .pat file in the layout
    TFPatFile.write_header / pat_writer produce (ebsd_pattern.py:1227-1300): the 25-byte header
    (version, columns, rows, width, height as uint32, scan flag -1 / 0 as int16, bit depth
    uint8, background flag -1 / 0 as int16), the background pattern when one is given, then
    per pattern its (column, row) as two uint32 and the pixels clipped to 2**bitdepth - 1."""
    pats = np.asarray(patterns)
    if pats.ndim == 2:
        pats = pats[None]
    n, h, w = pats.shape
    nCols, nRows = _scan_shape(n, nCols, nRows)
    top = min((1 << int(bitdepth)) - 1, 65535)
    pats = np.ascontiguousarray(np.clip(pats, 0, top).astype(np.uint16))
    with open(os.path.expanduser(str(path)), 'wb') as f:
        np.array([version, nCols, nRows, w, h], dtype=np.uint32).tofile(f)
        np.asarray(-1 if isscan else 0, dtype=np.int16).tofile(f)
        np.asarray(bitdepth, dtype=np.uint8).tofile(f)
        if background is None:
            np.asarray(0, dtype=np.int16).tofile(f)
        else:
            np.asarray(-1, dtype=np.int16).tofile(f)
            np.ascontiguousarray(np.asarray(background, dtype=np.uint16).reshape(h, w)).tofile(f)
        recs = np.empty(n, dtype=np.dtype([('loc', np.uint32, (2,)), ('pat', np.uint16, (h, w))]))
        recs['loc'][:, 0] = np.arange(n) % nCols
        recs['loc'][:, 1] = np.arange(n) // nCols
        recs['pat'] = pats
        recs.tofile(f)
