"""NLPAR (non-local pattern averaging) on the GPU, with array input and output.

The reference's ``NLPAR`` (nlpar_cpu.py:47-1072, OpenCL nlpar_cl.py) reads and writes pattern
files; here the same computation runs on arrays held in host or device memory so that it can
sit directly in front of band detection without a file round trip:

    nl = NLPAR(lam=0.7, searchradius=3)
    smooth = nl.calcnlpar_array(patterns, nrows, ncols)       # same shape, float32
    bands = band_detect_plan.find_bands(smooth)

``calcsigma_array`` restates ``NLPAR.sigma_numba`` (nlpar_cpu.py:753-796) and
``calcnlpar_array`` restates ``NLPAR.nlpar_nb`` (nlpar_cpu.py:821-936) as ``calcnlpar_cpu``
calls them for one tile covering the whole scan (nlpar_cpu.py:486-509).  Device kernels:
csrc/nlpar.cu.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["NLPAR"]


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
        lib._nlpar_bound = True
    return lib


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
        self.filepath = filename
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

    def calcnlpar_array(self, data, nrows=None, ncols=None, lam=None, searchradius=None, dthresh=None,
                        saturation_protect=None, sigma=None, reset_sigma=False):
        """NLPAR-averaged patterns, same shape as ``data``, float32.  ``sigma`` (or a previously
        computed ``self.sigma``) is reused unless ``reset_sigma``; else it is estimated first,
        as calcnlpar_cpu does (nlpar_cpu.py:486-493)."""
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
        if sigma is not None:
            sig = torch.as_tensor(np.asarray(sigma, dtype=np.float32) if not isinstance(sigma, torch.Tensor) else sigma,
                                  device=dev).to(torch.float32).reshape(nrows, ncols).contiguous()
        elif self.sigma is not None and not reset_sigma and np.shape(self.sigma) == (nrows, ncols):
            sig = torch.as_tensor(np.asarray(self.sigma, dtype=np.float32), device=dev)
        else:
            sig = torch.empty((nrows, ncols), dtype=torch.float32, device=dev)
            _lib.check(lib.ebsd_nlpar_sigma(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(),
                                            float(t.max().item()), int(bool(sp)), sig.data_ptr(), stream),
                       "ebsd_nlpar_sigma")
        self.sigma = sig.cpu().numpy()
        sr = int(self.searchradius)
        work = torch.empty((nrows * ncols, (2 * sr + 1) ** 2), dtype=torch.float32, device=dev)
        out = torch.empty_like(t)
        _lib.check(lib.ebsd_nlpar(t.data_ptr(), nrows, ncols, t.shape[1], ind.data_ptr(), ind.numel(),
                                  float(t.max().item()), float(np.float32(self.lam)), sr, float(np.float32(self.dthresh)),
                                  sig.data_ptr(), int(bool(sp)), work.data_ptr(), out.data_ptr(), stream),
                   "ebsd_nlpar")
        out = out.reshape(shape)
        return out if is_torch else out.cpu().numpy()
