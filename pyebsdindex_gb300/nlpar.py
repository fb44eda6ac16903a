"""NLPAR (non-local pattern averaging) on the GPU, on arrays and on pattern files.

The reference's ``NLPAR`` (nlpar_cpu.py:47-1072, OpenCL nlpar_cl.py) reads and writes pattern
files.  Here the computation runs on arrays held in host or device memory, so that it can sit
directly in front of band detection without a file round trip:

    nl = NLPAR(lam=0.7, searchradius=3)
    smooth = nl.calcnlpar_array(patterns, nrows, ncols)       # same shape, float32
    bands = band_detect_plan.find_bands(smooth)

and the reference's file interface -- ``setfile``, ``calcsigma``, ``opt_lambda``,
``calcnlpar``, ``auto_nlpar`` -- runs the same kernels on UP1 / UP2, .ebsp and .pat files
(pyebsdindex_gb300.ebsd_pattern), with the reference's scan tiling, halos, sigma merging
and output file:

    nl = NLPAR("scan.up1", searchradius=3)
    nl.opt_lambda()                   # sets nl.lam
    out = nl.calcnlpar()              # writes scan_NLPAR_l{lam:.2f}sr3.up1, returns its path

``calcsigma_array`` restates ``NLPAR.sigma_numba`` (nlpar_cpu.py:753-796) and
``calcnlpar_array`` restates ``NLPAR.nlpar_nb`` (nlpar_cpu.py:821-936) as ``calcnlpar_cpu``
calls them for one tile covering the whole scan (nlpar_cpu.py:486-509).  Device kernels:
csrc/nlpar.cu.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["NLPAR", "scan_tiles"]


def host_memory_bytes():
    """Total host memory (what psutil.virtual_memory().total reports on Linux)."""
    import os
    try:
        return int(os.sysconf("SC_PAGE_SIZE")) * int(os.sysconf("SC_PHYS_PAGES"))
    except (ValueError, OSError, AttributeError):
        return 64 << 30


def scan_tiles(patdim, ncol, nrow, target_bytes, col_overlap=0, row_overlap=0):
    """The reference's scan tiling (NLPAR._calcchunks, nlpar_cpu.py:973-1065): column and row
    ranges [start, end) as int arrays [n, 2].  At least two column tiles when ncol >= nrow
    (two row tiles otherwise), about target_bytes of float32 input+output per tile, tiles
    overlapping by the given rows / columns on each side."""
    col_overlap = min(col_overlap, ncol - 1)
    row_overlap = min(row_overlap, nrow - 1)
    nchunks = int(np.ceil(patdim[-1] * patdim[-2] * 8 * ncol * nrow / target_bytes))

    def ranges(n, count, overlap):
        step = max(n / count, 1)
        count = max(int(np.ceil(max(n / step, 1))), 1)
        step = max(int(np.round(step)), 1)
        span = min(step + 2 * overlap, n)
        out = []
        for c in range(count):
            out.append([int(c * step) - int(overlap), int(c * step + span) - int(overlap)])
            if out[-1][1] > n:
                break
        out = np.array(out, dtype=int)
        out[0, 0], out[-1, 1] = 0, n
        if len(out) > 1:
            out[-1, 0] = max(0, out[-2, 1] - 2 * int(overlap) - 1)
        return out, count

    cols, ncount = ranges(ncol, max(np.round(np.sqrt(nchunks * float(ncol) / nrow)), 2 if ncol >= nrow else 1),
                          col_overlap)
    # the row count divides by the column count before the column list stops early
    rows, _ = ranges(nrow, max(np.ceil(nchunks / ncount), 2 if nrow > ncol else 1), row_overlap)
    return cols, rows


def _bind():
    lib = _lib.load()
    if not getattr(lib, "_nlpar_bound", False):
        lib.ebsd_nlpar_sigma.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                         C.c_float, C.c_int, C.c_void_p, C.c_void_p]
        lib.ebsd_nlpar_sigma.restype = C.c_int
        lib.ebsd_nlpar.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_float,
                                   C.c_float, C.c_int32, C.c_float, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_void_p]
        lib.ebsd_nlpar.restype = C.c_int
        lib.ebsd_nlpar_out.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                       C.c_float, C.c_float, C.c_int32, C.c_float, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ebsd_nlpar_out.restype = C.c_int
        lib.ebsd_nlpar_pairs_out.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                             C.c_float, C.c_float, C.c_int32, C.c_float, C.c_void_p, C.c_int, C.c_int,
                                             C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ebsd_nlpar_pairs_out.restype = C.c_int
        lib.ebsd_nlpar_sigma_tile.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ebsd_nlpar_sigma_tile.restype = C.c_int
        lib.ebsd_nlpar_lambda_metric.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_double,
                                                 C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ebsd_nlpar_lambda_metric.restype = C.c_int
        lib._nlpar_bound = True
    return lib


class _Tile:
    """One scan tile of an NLPAR file run: rows [r0, r0 + nr) x columns [c0, c0 + nc) are read;
    the interior rows [ir0, ir0 + inr) x columns [ic0, ic0 + inc) of it are written."""
    __slots__ = ("r0", "nr", "c0", "nc", "ir0", "inr", "ic0", "inc")

    def __init__(self, r0, nr, c0, nc, ir0, inr, ic0, inc):
        self.r0, self.nr, self.c0, self.nc = r0, nr, c0, nc
        self.ir0, self.inr, self.ic0, self.inc = ir0, inr, ic0, inc


def _halo_tiles(rows, cols, sr):
    """The tiles of ``scan_tiles``' row and column ranges, row by row; each drops ``sr`` halo
    rows / columns on every side it shares with a neighbouring tile (nlpar_cpu.py:400-426)."""
    nrt, nct = len(rows), len(cols)
    for a in range(nrt):
        r0, r1 = int(rows[a, 0]), int(rows[a, 1])
        top = sr if a > 0 else 0
        bottom = (r1 - r0) - sr if a < nrt - 1 else r1 - r0
        for b in range(nct):
            c0, c1 = int(cols[b, 0]), int(cols[b, 1])
            left = sr if b > 0 else 0
            right = (c1 - c0) - sr if b < nct - 1 else c1 - c0
            yield _Tile(r0, r1 - r0, c0, c1 - c0, top, bottom - top, left, right - left)


def _diff_offsets(nrows, ncols, sr, diff_offset, block):
    """nlpar_nb's centre-weight additions for a non-zero diff_offset (nlpar_cpu.py:880-925), as
    its loops run one after another over the computed block (col0, row0, ncol, nrow) of a tile:
    one float32 array of per-slot additions lives for the whole call; the pixels are visited
    column by column (rows inner), and each visit adds diff_offset to the pixel's own window slot
    and zeroes all others.  So a pixel's addition is diff_offset summed (in float32) over the run
    of consecutive visits, ending with it, whose own slot is the same.  Returns [nrows, ncols]
    float32 (0 outside the block)."""
    c0, r0, nc, nr = block
    wn = 2 * sr + 1
    cols = np.arange(c0, c0 + nc)
    rows = np.arange(r0, r0 + nr)
    xs = np.array([window_start(i, sr, ncols) for i in cols])
    ys = np.array([window_start(j, sr, nrows) for j in rows])
    own = ((rows - ys)[None, :] * wn + (cols - xs)[:, None]).ravel()  # visit order: column-major
    cuts = np.nonzero(np.diff(own) != 0)[0] + 1
    adds = np.concatenate([np.add.accumulate(np.full(len(run), diff_offset, dtype=np.float32))
                           for run in np.split(own, cuts)])
    out = np.zeros((nrows, ncols), dtype=np.float32)
    out[r0:r0 + nr, c0:c0 + nc] = adds.reshape(nc, nr).T
    return out


def window_start(i, sr, n):
    """First index of the (2 sr + 1)-wide search window of position i along a scan axis of n,
    shifted inward at the edges (nlpar_cpu.py:872-878)."""
    return max(i - sr, 0) - max(i + sr - (n - 1), 0)


class NLPAR:
    """NLPAR parameters with the reference constructor (nlpar_cpu.py:47-79)."""

    def __init__(self, filename=None, lam=0.7, searchradius=3, dthresh=0.0, diff_offset=0.0,
                 saturation_protect=True, stem_scale=False, automask=True, nrows=None, ncols=None,
                 gpu_id=0, **kwargs):
        self.lam = lam
        self.searchradius = searchradius
        self.dthresh = dthresh
        self.diff_offset = diff_offset
        self.saturation_protect = saturation_protect
        self.stem_scale = stem_scale
        self.automask = automask
        self.filepath = None
        self.hdfdatapath = None
        self.filepathout = None
        self.hdfdatapathout = None
        self.setfile(filename)
        self.mask = None
        self.sigma = None
        self.sigmann = 1
        self.nrows = nrows
        self.ncols = ncols
        self.gpu_id = int(gpu_id or 0)

    @staticmethod
    def makeautomask(h, w):
        """Circular mask, radius 0.98*min(h, w)/2, centred (nlpar_cpu.py:737-750)."""
        r = min(h, w) * 0.98 * 0.5
        x = np.arange(w, dtype=np.float32)
        x = np.minimum(x, w - x).reshape(1, w)
        y = np.arange(h, dtype=np.float32)
        y = np.minimum(y, h - y).reshape(h, 1)
        m = (np.sqrt(y ** 2 + x ** 2) < r).astype(np.uint8)
        return np.roll(m, (int(h / 2), int(w / 2)), axis=(0, 1))

    # -- helpers ---------------------------------------------------------------------------
    def _prepare(self, data, nrows, ncols):
        import torch
        nrows = int(nrows if nrows is not None else self.nrows)
        ncols = int(ncols if ncols is not None else self.ncols)
        is_torch = isinstance(data, torch.Tensor)
        t = data if is_torch else torch.from_numpy(np.ascontiguousarray(data))
        shape = tuple(t.shape)
        h, w = shape[-2], shape[-1]
        if int(np.prod(shape[:-2])) != nrows * ncols:
            raise ValueError(f"data holds {int(np.prod(shape[:-2]))} patterns, expected nrows*ncols = {nrows * ncols}")
        dev = torch.device("cuda", self.gpu_id) if not (is_torch and t.is_cuda) else t.device
        t = t.to(dev).reshape(nrows * ncols, h * w).to(torch.float32).contiguous()
        if self.automask is True and self.mask is None:
            self.mask = self.makeautomask(h, w)
        if self.mask is None:
            self.mask = np.ones((h, w), dtype=np.uint8)
        ind = torch.from_numpy(np.nonzero(np.asarray(self.mask).ravel())[0].astype(np.int32)).to(dev)
        return t, ind, nrows, ncols, shape, is_torch, dev

    def calcsigma_array(self, data, nrows=None, ncols=None, saturation_protect=None):
        """Noise sigma per scan pixel, [nrows, ncols] float32 (sigma_numba, nn = 1)."""
        import torch
        lib = _bind()
        sp = self.saturation_protect if saturation_protect is None else saturation_protect
        t, ind, nrows, ncols, shape, is_torch, dev = self._prepare(data, nrows, ncols)
        sig = torch.empty((nrows, ncols), dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _lib.check(lib.ebsd_nlpar_sigma(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(),
                                        float(t.max().item()), int(bool(sp)), sig.data_ptr(), stream),
                   "ebsd_nlpar_sigma")
        return sig if is_torch else sig.cpu().numpy()

    def _sigma_tiles(self, data, nrows, ncols, saturation_protect, target_bytes):
        import torch
        lib = _bind()
        sp = self.saturation_protect if saturation_protect is None else saturation_protect
        t, ind, nrows, ncols, shape, is_torch, dev = self._prepare(data, nrows, ncols)
        h, w = shape[-2], shape[-1]
        if target_bytes is None:
            target_bytes = min(32e9, host_memory_bytes() // 4)
        cols, rows = scan_tiles([w, h], ncols, nrows, target_bytes, col_overlap=1, row_overlap=1)
        sig = torch.full((nrows, ncols), 1e18, dtype=torch.float32, device=dev)
        d2 = torch.zeros((nrows, ncols, 9), dtype=torch.float32, device=dev)
        n2 = torch.zeros((nrows, ncols, 9), dtype=torch.float32, device=dev)
        tmax = max((r1 - r0) * (c1 - c0) for r0, r1 in rows for c0, c1 in cols)
        work = torch.empty(tmax * 19 + 1, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        for r0, r1 in rows:
            for c0, c1 in cols:
                _lib.check(lib.ebsd_nlpar_sigma_tile(t.data_ptr(), nrows, ncols, t.shape[1], int(r0), int(r1), int(c0),
                                                     int(c1), ind.data_ptr(), ind.numel(), int(bool(sp)),
                                                     sig.data_ptr(), d2.data_ptr(), n2.data_ptr(), work.data_ptr(),
                                                     stream), "ebsd_nlpar_sigma_tile")
        return sig, d2, n2, is_torch

    def calcsigma_tiles_array(self, data, nrows=None, ncols=None, saturation_protect=None, target_bytes=None):
        """sigma, normalised neighbour distances d2 and counts n2 ([nrows, ncols, 9]) as
        NLPAR.calcsigma_cpu computes them for the lambda optimisation (nlpar_cpu.py:157-264):
        sigma_numba per scan tile (tiles from ``scan_tiles``, one row / column of overlap) with
        the reference's uint64 window arithmetic -- each tile's first row and column get empty
        windows -- merged tile by tile.  Device tensors for torch input, else numpy."""
        sig, d2, n2, is_torch = self._sigma_tiles(data, nrows, ncols, saturation_protect, target_bytes)
        if is_torch:
            return sig, d2, n2
        return sig.cpu().numpy(), d2.cpu().numpy(), n2.cpu().numpy()

    def opt_lambda_array(self, data, nrows=None, ncols=None, target_weights=(0.5, 0.34, 0.25), autoupdate=True,
                         dthresh=None, saturation_protect=None, target_bytes=None, verbose=0):
        """NLPAR.opt_lambda_cpu (nlpar_cpu.py:94-155) on the device: sigma and the normalised
        neighbour distances per scan tile (``calcsigma_tiles_array``), then, for each target
        weight, scipy's bounded Nelder-Mead from lambda = 1 (the reference's call and options)
        on the objective mean |tw - 1 / sum_q exp(-max(d2_q, dthresh) / lam^2)|, evaluated on
        the device (every second row and column for scans of 1e6 pixels or more).  Sets
        ``self.lam`` to the median when ``autoupdate``; returns the lambda values."""
        import torch
        import scipy.optimize as opt
        lib = _bind()
        if dthresh is not None:
            self.dthresh = dthresh
        dth = np.float32(self.dthresh if np.isscalar(self.dthresh) else self.dthresh[0])
        sig, d2, _, _ = self._sigma_tiles(data, nrows, ncols, saturation_protect, target_bytes)
        nr, nc = int(sig.shape[0]), int(sig.shape[1])
        stride = 1 if nr * nc < 1e6 else 2
        dev = d2.device
        work = torch.empty(256, dtype=torch.float64, device=dev)
        res = torch.empty(1, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream

        def objective(lam, tw):
            _lib.check(lib.ebsd_nlpar_lambda_metric(d2.data_ptr(), nr, nc, stride, float(dth),
                                                    float(np.asarray(lam).ravel()[0]), float(tw), work.data_ptr(),
                                                    res.data_ptr(), stream), "ebsd_nlpar_lambda_metric")
            return float(res.item())

        vals = []
        for tw in np.asarray(target_weights):
            r = opt.minimize(objective, 1.0, args=(tw,), method='Nelder-Mead', bounds=[[0.001, 10.0]],
                             options={'fatol': 0.0001})
            vals.append(r['x'])
        vals = np.asarray(vals).flatten()
        if verbose >= 2:
            print("Range of lambda values: ", vals, "Optimal Choice: ", np.median(vals))
        if autoupdate:
            self.lam = np.median(vals)
        if self.sigma is None:
            self.sigma = sig.cpu().numpy()
        return vals

    def calcnlpar_array(self, data, nrows=None, ncols=None, lam=None, searchradius=None, dthresh=None,
                        saturation_protect=None, sigma=None, reset_sigma=False, out_dtype=None,
                        centre_offset=None):
        """NLPAR-averaged patterns, same shape as ``data``.  ``sigma`` (or a previously computed
        ``self.sigma``) is reused unless ``reset_sigma``; else it is estimated first, as
        calcnlpar_cpu does (nlpar_cpu.py:486-493).  ``out_dtype``: float32 (default), or
        np.uint8 / np.uint16 -- the averaged values stored as the reference writes its NLPAR
        output file (pat_flt2int 'clip': clipped to the type's range, truncated), straight from
        the averaging kernel, e.g. as the input of band detection on the device.
        ``centre_offset`` [nrows, ncols]: added to each pixel's own window weight (the
        diff_offset additions of nlpar_nb)."""
        import torch
        lib = _bind()
        if lam is not None:
            self.lam = lam
        if searchradius is not None:
            self.searchradius = searchradius
        if dthresh is not None:
            self.dthresh = dthresh
        sp = self.saturation_protect if saturation_protect is None else saturation_protect
        t, ind, nrows, ncols, shape, is_torch, dev = self._prepare(data, nrows, ncols)
        stream = torch.cuda.current_stream(dev).cuda_stream
        dmax = float(t.max().item())
        sr = int(self.searchradius)
        # radii 1..3: sigma, weights and average in one call that sums each unordered pair once
        pairs = 1 <= sr <= 3
        compute_sigma = False
        if sigma is not None:
            sig = torch.as_tensor(np.asarray(sigma, dtype=np.float32) if not isinstance(sigma, torch.Tensor) else sigma,
                                  device=dev).to(torch.float32).reshape(nrows, ncols).contiguous()
        elif self.sigma is not None and not reset_sigma and np.shape(self.sigma) == (nrows, ncols):
            sig = torch.as_tensor(np.asarray(self.sigma, dtype=np.float32), device=dev)
        else:
            sig = torch.empty((nrows, ncols), dtype=torch.float32, device=dev)
            compute_sigma = True
            if not pairs:
                _lib.check(lib.ebsd_nlpar_sigma(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(),
                                                dmax, int(bool(sp)), sig.data_ptr(), stream), "ebsd_nlpar_sigma")
        winsz = (2 * sr + 1) ** 2
        nfwd = sr * (2 * sr + 1) + sr
        nedge = 2 * sr * (nrows + ncols - 2 * sr)
        work = torch.empty(nrows * ncols * (winsz + (2 * nfwd + 8 if pairs else 0)) + (2 * nedge * winsz if pairs else 0)
                           + 1, dtype=torch.float32, device=dev)
        odt = np.dtype(np.float32 if out_dtype is None else out_dtype)
        if odt == np.float32:
            out, code = torch.empty_like(t), _lib.EBSD_F32
        elif odt == np.uint8:
            out, code = torch.empty(t.shape, dtype=torch.uint8, device=dev), _lib.EBSD_U8
        elif odt == np.uint16:
            # torch's uint16 has few device operations: allocated as int16, viewed as uint16
            out, code = torch.empty(t.shape, dtype=torch.int16, device=dev), _lib.EBSD_U16
        else:
            raise TypeError(f"out_dtype {odt} (float32, uint8 or uint16)")
        coff = None
        if centre_offset is not None:
            coff = torch.as_tensor(np.asarray(centre_offset, dtype=np.float32) if not torch.is_tensor(centre_offset)
                                   else centre_offset, device=dev).to(torch.float32).reshape(-1).contiguous()
            if coff.numel() != nrows * ncols:
                raise ValueError("centre_offset holds one value per scan pixel")
        lam32, dth32 = float(np.float32(self.lam)), float(np.float32(self.dthresh))
        rc = -1
        if pairs:
            rc = lib.ebsd_nlpar_pairs_out(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(), dmax,
                                          lam32, sr, dth32, sig.data_ptr(), int(compute_sigma), int(bool(sp)),
                                          work.data_ptr(), code, out.data_ptr(),
                                          None if coff is None else coff.data_ptr(), stream)
            if rc != _lib.EBSD_E_UNSUPPORTED:
                _lib.check(rc, "ebsd_nlpar_pairs_out")
        if rc != 0:
            # the per-slot kernels (radii beyond 3, or staged tiles too large for the pair kernels)
            if compute_sigma and pairs:
                _lib.check(lib.ebsd_nlpar_sigma(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(),
                                                dmax, int(bool(sp)), sig.data_ptr(), stream), "ebsd_nlpar_sigma")
            _lib.check(lib.ebsd_nlpar_out(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(), dmax,
                                          lam32, sr, dth32, sig.data_ptr(), int(bool(sp)), work.data_ptr(), code,
                                          out.data_ptr(), None if coff is None else coff.data_ptr(), stream),
                       "ebsd_nlpar_out")
        self.sigma = sig.cpu().numpy()
        out = out.reshape(shape)
        if odt == np.uint16:
            # torch's uint16 has few operations: returned as a uint16 view where torch has the type
            if not is_torch:
                return out.cpu().numpy().view(np.uint16)
            return out.view(torch.uint16) if hasattr(torch, "uint16") else out
        return out if is_torch else out.cpu().numpy()

    # -- the reference's file interface (nlpar_cpu.py:81-92, :94-281, :283-540, :542-677) ------
    def setfile(self, filepath=None):
        """The input pattern file (nlpar_cpu.py:542-552)."""
        self.filepath = None
        self.hdfdatapath = None
        pathtemp = np.atleast_1d(filepath)
        if pathtemp[0] is not None:
            from pathlib import Path
            self.filepath = Path(str(pathtemp[0]))
            self.hdfdatapath = pathtemp[1] if pathtemp.size > 1 else None

    def getinfileobj(self):
        """The input file's reader; its scan shape becomes nrows / ncols unless they are set, in
        which case they override the file's (nlpar_cpu.py:633-656)."""
        from . import ebsd_pattern
        if self.filepath is None:
            return None
        f = ebsd_pattern.get_pattern_file_obj(self.filepath)
        if f.nRows is not None:
            if self.nrows is None:
                self.nrows = f.nRows
            else:
                f.nRows = self.nrows
        if f.nCols is not None:
            if self.ncols is None:
                self.ncols = f.nCols
            else:
                f.nCols = self.ncols
        return f

    def setoutfile(self, patternfile, filepath=None):
        """The output file (nlpar_cpu.py:554-631): ``filepath`` when given (not the input
        file), else the input's name with ``_NLPAR_l{lam:.2f}sr{sr}`` before the extension; the
        input's header copied there with an empty body (EBSP files are copied whole)."""
        from pathlib import Path
        self.filepathout = None
        self.hdfdatapathout = None
        fpath = np.atleast_1d(filepath)[0]
        if fpath is not None:
            self.filepathout = Path(str(fpath)).expanduser().resolve()
            if self.filepathout.exists() and self.filepathout.samefile(patternfile.filepath):
                raise ValueError('Error: File input and output are exactly the same.')
            patternfile.copy_file([self.filepathout, None], empty_data=True)
            return
        if patternfile is not None:
            p = Path(patternfile.filepath)
            appnd = "_NLPAR_l{:1.2f}".format(self.lam) + "sr{:d}".format(self.searchradius)
            newfilepath = str(p.parent / Path(p.stem + appnd + p.suffix))
            patternfile.copy_file(newfilepath, empty_data=True)
            self.filepathout = newfilepath

    def getoutfileobj(self):
        """The output file's reader with the scan shape in use (nlpar_cpu.py:658-677)."""
        from . import ebsd_pattern
        if self.filepathout is None:
            return None
        f = ebsd_pattern.get_pattern_file_obj(self.filepathout)
        if self.nrows is not None:
            f.nRows = self.nrows
        else:
            self.nrows = f.nRows
        if self.ncols is not None:
            f.nCols = self.ncols
        else:
            self.ncols = f.nCols
        return f

    @staticmethod
    def _first(v):
        return v if np.isscalar(v) else np.asarray(v).ravel()[0]

    def _file_scan(self, stem_scale):
        """The whole scan of the input file as float32 [nrows * ncols, H, W] (square-rooted
        above the file's minimum with stem_scale, as calcsigma_cpu does)."""
        f = self.getinfileobj()
        if f is None:
            raise ValueError("no input file: NLPAR(filename) or setfile(path) first")
        nrows, ncols = int(self.nrows), int(self.ncols)
        data, _ = f.read_data(patStartCount=[[0, 0], [ncols, nrows]], convertToFloat=True, returnArrayOnly=True)
        if stem_scale:
            data = np.sqrt(data.astype(np.float32) - np.float32(data.min())).astype(np.float32)
        return f, data, nrows, ncols

    @staticmethod
    def _target_bytes(chunksize):
        return float(chunksize) if chunksize > 0 else min(32e9, host_memory_bytes() // 4)

    def calcsigma(self, chunksize=0, nn=1, saturation_protect=None, automask=None, stem_scale=None, verbose=2,
                  **kwargs):
        """NLPAR.calcsigma_cpu (nlpar_cpu.py:186-281) on the input file: sigma [nrows, ncols]
        and the normalised neighbour distances d2 and counts n2 [nrows, ncols, 9], per scan tile
        of about ``chunksize`` bytes (0: the reference's default), merged as the reference
        merges them.  The scan is read once and held on the device as float32: host and device
        memory must hold 4 * nrows * ncols * H * W bytes (the reference reads tile by tile)."""
        if int(nn) != 1:
            raise NotImplementedError("only nn = 1 (the reference's default) is built")
        self.sigmann = 1
        if saturation_protect is not None:
            self.saturation_protect = saturation_protect
        if automask is not None:
            self.automask = automask
        if stem_scale is not None:
            self.stem_scale = stem_scale
        _, data, nrows, ncols = self._file_scan(bool(self._first(self.stem_scale)))
        return self.calcsigma_tiles_array(data, nrows, ncols, saturation_protect=bool(self._first(self.saturation_protect)),
                                          target_bytes=self._target_bytes(chunksize))

    def opt_lambda(self, target_weights=(0.5, 0.34, 0.25), autoupdate=True, dthresh=None, verbose=2, chunksize=0,
                   saturation_protect=None, automask=None, stem_scale=None, **kwargs):
        """NLPAR.opt_lambda_cpu (nlpar_cpu.py:94-184) on the input file: the lambda values for
        the target weights (``opt_lambda_array`` on the file's scan), their median in ``lam``
        when ``autoupdate``.  Like ``calcsigma``, holds the whole scan as float32 on the host and
        the device (4 * nrows * ncols * H * W bytes)."""
        if saturation_protect is not None:
            self.saturation_protect = saturation_protect
        if automask is not None:
            self.automask = automask
        if stem_scale is not None:
            self.stem_scale = stem_scale
        _, data, nrows, ncols = self._file_scan(bool(self._first(self.stem_scale)))
        vals = self.opt_lambda_array(data, nrows, ncols, target_weights=target_weights, autoupdate=autoupdate,
                                     dthresh=dthresh, saturation_protect=bool(self._first(self.saturation_protect)),
                                     target_bytes=self._target_bytes(chunksize), verbose=0)
        if verbose >= 1:
            print("Range of lambda values: ", vals)
            print("Optimal Choice: ", np.median(vals))
        return vals

    def _tile_sigma(self, data, nrows, ncols, saturation_protect):
        """sigma_numba with nn = 1 over one tile (nlpar_cpu.py:486-490)."""
        return np.asarray(self.calcsigma_array(data, nrows, ncols, saturation_protect=saturation_protect))

    def _tile_nlpar(self, data, nrows, ncols, lam, sr, dthresh, saturation_protect, sigma, centre_offset=None):
        """nlpar_nb over one tile with the tile's merged sigma (nlpar_cpu.py:496-509) and, with a
        diff_offset, the per-pixel centre-weight additions; the object's own parameters and
        sigma are left as they were."""
        keep = (self.lam, self.searchradius, self.dthresh, self.sigma)
        try:
            return np.asarray(self.calcnlpar_array(data, nrows, ncols, lam=lam, searchradius=sr, dthresh=dthresh,
                                                   saturation_protect=saturation_protect, sigma=sigma,
                                                   centre_offset=centre_offset))
        finally:
            self.lam, self.searchradius, self.dthresh, self.sigma = keep

    def backsub(self, data):
        """Subtract a smooth background from every pattern of ``data`` [n, H, W] in place
        (nlpar_cpu.py:679-734): a 2-D Gaussian on a tilted plane fitted by least squares to the
        patterns' mean over the mask (started from the full range of the masked mean at its
        brightest pixel, widths of a sixth of the pattern), its own mean removed; the plain
        mean pattern, mean removed, when the fit does not converge.  Host preprocessing of a
        tile, as in the reference."""
        from .band_detect import _fit_gaussian_plane
        mean = np.mean(data, axis=0)
        ny, nx = data.shape[-2], data.shape[-1]
        if self.mask is None:
            self.mask = self.makeautomask(ny, nx) if self.automask is True else np.ones((ny, nx), np.uint8)
        inside = np.asarray(self.mask).ravel() != 0
        z = mean.ravel()[inside]
        yy, xx = np.indices((ny, nx), dtype=float)
        brightest = np.unravel_index(mean.argmax(), mean.shape)
        start = [z.max() - z.min(), brightest[1], brightest[0], nx / 2.355, ny / 2.355, z.min(), 0, 0]
        fitted = _fit_gaussian_plane(xx.ravel(), yy.ravel(), inside, z, start)
        if fitted is None:
            print('Warning: no convergence on back subtract ... using mean of the patterns.')
            model = mean
        else:
            model = fitted.reshape(ny, nx)
        data -= model - np.mean(model)
        return data

    def calcnlpar(self, chunksize=0, searchradius=None, lam=None, dthresh=None, saturation_protect=None,
                  automask=None, stem_scale=None, filename=None, fileout=None, reset_sigma=False, backsub=False,
                  rescale=False, verbose=2, diff_offset=None, **kwargs):
        """NLPAR.calcnlpar_cpu (nlpar_cpu.py:283-540) on the input file, into the output file
        (``setoutfile``); returns the output path.

        The scan is processed in tiles of about ``chunksize`` bytes (0: the reference's default
        of a quarter of host memory, at most 32 GB), each read with ``searchradius`` rows and
        columns of halo from its neighbours, in the reference's order.  Per tile: optionally
        square-rooted above the file's minimum (``stem_scale``) and background-subtracted
        (``backsub``); its noise sigma merged into ``self.sigma`` by minimum unless a sigma is
        already set (e.g. by ``opt_lambda``); the weighted average on the device (with
        ``diff_offset``, its centre-weight additions); the interior kept, squared back
        (``stem_scale``) or stretched to the output type's range (``rescale``), and written
        clipped to the output file's pixel type.  The output file's data minimum and maximum
        are set from what was written.  With ``reset_sigma`` the sigma is estimated anew (the
        reference's calcnlpar_cpu fails with reset_sigma set)."""
        params = self._run_parameters(searchradius, lam, dthresh, saturation_protect, automask, stem_scale,
                                      diff_offset)
        sr, stem = params["sr"], params["stem"]
        if filename is not None:
            self.setfile(filepath=filename)
        src = self.getinfileobj()
        if src is None:
            raise ValueError("no input file: NLPAR(filename), setfile(path) or filename=")
        self.setoutfile(src, filepath=fileout)
        dst = self.getoutfileobj()
        nrows, ncols = np.int64(self.nrows), np.int64(self.ncols)
        dst.nCols = ncols if dst.nCols is None else dst.nCols
        dst.nRows = nrows if dst.nRows is None else dst.nRows
        width, height = int(src.patternW), int(src.patternH)
        cols, rows = scan_tiles([width, height], int(ncols), int(nrows), self._target_bytes(chunksize),
                                col_overlap=sr, row_overlap=sr)
        if self.automask is True and self.mask is None:
            self.mask = self.makeautomask(height, width)
        if self.mask is None:
            self.mask = np.ones((height, width), dtype=np.uint8)
        estimate = self._scan_sigma(int(nrows), int(ncols), reset_sigma)
        top = None
        if rescale and np.issubdtype(dst.filedatatype, np.integer):
            top = np.iinfo(dst.filedatatype).max
        floor = self._file_minimum(src, rows, cols) if stem else None
        if verbose >= 1:
            print("lambda:", self.lam, "search radius:", self.searchradius, "dthresh:", self.dthresh)
        lo_written, hi_written = np.inf, -np.inf
        tiles = list(_halo_tiles(rows, cols, sr))
        for done, t in enumerate(tiles, 1):
            data, _ = src.read_data(patStartCount=[[t.c0, t.r0], [t.nc, t.nr]], convertToFloat=True,
                                    returnArrayOnly=True)
            if stem:
                data = np.sqrt(data.astype(np.float32) - floor).astype(np.float32)
            if backsub:
                data = self.backsub(data)
            window_sigma = self._merge_tile_sigma(data, t, estimate, params["sp"])
            centre = None
            if params["diff_offset"] != 0.0:
                centre = _diff_offsets(t.nr, t.nc, sr, params["diff_offset"], (t.ic0, t.ir0, t.inc, t.inr))
            avg = self._tile_nlpar(data, t.nr, t.nc, params["lam"], sr, params["dthresh"], params["sp"],
                                   window_sigma, centre)
            out = avg.reshape(t.nr, t.nc, -1)[t.ir0:t.ir0 + t.inr, t.ic0:t.ic0 + t.inc, :]
            if stem:
                out = out ** 2 + floor
            out = out.reshape(t.inr * t.inc, height, width)
            if top is not None:
                for pat in out:
                    pat -= pat.min()
                    pat *= np.float32(top) / pat.max()
            lo_written, hi_written = min(lo_written, np.min(out)), max(hi_written, np.max(out))
            dst.write_data(newpatterns=out, patStartCount=[[np.int64(t.c0 + t.ic0), np.int64(t.r0 + t.ir0)],
                                                           [np.int64(t.inc), np.int64(t.inr)]],
                           flt2int='clip', scalevalue=1.0)
            if verbose >= 2:
                print("tiles complete: ", done, "/", len(tiles), sep='', end='\r')
        if verbose >= 2:
            print('', end='')
        dst.datamin, dst.datamax = lo_written, hi_written
        dst.write_datamaxmin()
        return str(dst.filepath)

    def _run_parameters(self, searchradius, lam, dthresh, saturation_protect, automask, stem_scale, diff_offset):
        """Update the object's parameters from the given ones; the scalars a run uses."""
        for name, value in (("searchradius", searchradius), ("lam", lam), ("dthresh", dthresh),
                            ("saturation_protect", saturation_protect), ("automask", automask),
                            ("stem_scale", stem_scale), ("diff_offset", diff_offset)):
            if value is not None:
                setattr(self, name, value)
        return {"sr": int(self._first(self.searchradius)), "lam": np.float32(self._first(self.lam)),
                "dthresh": np.float32(self._first(self.dthresh)),
                "sp": bool(self._first(self.saturation_protect)), "stem": bool(self._first(self.stem_scale)),
                "diff_offset": np.float32(self._first(self.diff_offset))}

    def _scan_sigma(self, nrows, ncols, reset):
        """Prepare ``self.sigma`` for a run over an nrows x ncols scan (nlpar_cpu.py:365-389);
        True when it is to be estimated tile by tile.  An unset (or reset) sigma starts at 1e24
        everywhere and is estimated; one value is spread over the scan and kept; an array whose
        rows and columns both differ from the scan's is replaced and estimated."""
        sig = None if reset else self.sigma
        estimate = sig is None
        if estimate:
            sig = np.full((nrows, ncols), 1e24, dtype=np.float32)
        elif np.asarray(sig).size == 1:
            sig = np.full((nrows, ncols), np.asarray(sig).ravel()[0], dtype=np.float32)
        shape = np.asarray(sig).shape
        if shape[0] != nrows and shape[1] != ncols:
            sig, estimate = np.full((nrows, ncols), 1e24, dtype=np.float32), True
        self.sigma = np.asarray(sig, dtype=np.float32)
        return estimate

    def _merge_tile_sigma(self, data, t, estimate, sp):
        """The sigma a tile's windows use: when estimating, the tile's own sigma merged into
        ``self.sigma`` by minimum (nlpar_cpu.py:486-493); else ``self.sigma`` over the tile."""
        block = self.sigma[t.r0:t.r0 + t.nr, t.c0:t.c0 + t.nc]
        if estimate:
            block[...] = np.minimum(block, self._tile_sigma(data, t.nr, t.nc, sp))
        return np.ascontiguousarray(block)

    def _file_minimum(self, src, rows, cols):
        """The input file's smallest value (nlpar_cpu.py:948-969): the file's stored limits, or a
        pass over the scan tile by tile; stored on the file object."""
        src.read_datamaxmin()
        if src.datamin is None or src.datamax is None:
            lo, hi = np.inf, -np.inf
            for r0, r1 in rows:
                for c0, c1 in cols:
                    data, _ = src.read_data(patStartCount=[[int(c0), int(r0)], [int(c1 - c0), int(r1 - r0)]],
                                            convertToFloat=True, returnArrayOnly=True)
                    lo, hi = min(lo, data.min()), max(hi, data.max())
            src.datamin, src.datamax = lo, hi
            src.write_datamaxmin()
        return src.datamin

    def auto_nlpar(self, filename=None, fileout=None, lindex=1, **kwargs):
        """opt_lambda, then calcnlpar with the lambda of target weight ``lindex`` unless ``lam``
        is given (nlpar_cpu.py:81-92)."""
        if filename is not None:
            self.setfile(filename)
        lam = self.opt_lambda(autoupdate=True, **kwargs)
        if 'lam' not in kwargs:
            kwargs['lam'] = lam[int(lindex)]
        return self.calcnlpar(fileout=fileout, **kwargs)
