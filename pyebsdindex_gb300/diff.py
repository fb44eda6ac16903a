"""Differentiable band-sharpness objective with hand-written adjoint kernels.

Forward, per pattern of a scan grid (all on the GPU):

    x --NLPAR(lam)--> y --minus Gaussian blur(sigma)--> z --Radon--> r --LoG--> c
    J = mean over patterns of sum_i softmax(c_i / tau) c_i    (soft-argmax band sharpness)

* NLPAR: the weighted neighbour average of nlpar_cpu.py:821-936 with its weights computed from
  the (detached) input and lambda; the weights' dependence on lambda is differentiated
  (``ebsd_nlpar_lambda_grad``), their dependence on the pattern distances is not.
* Radon: the band-detection ray means (radon_fast.py:281-310) as a sparse operator R (empty
  rays give 0); backward is the back-projection R^T through the transposed lookup table.
* LoG: padding (theta mirror / rho edge, band_detect.py:573-580) followed by the LoG
  convolution (band_detect.py:596-606), restricted to the Radon interior, as a sparse operator
  M; backward is M^T (correlation with the kernel folded back through the padding map).
* The Gaussian background blur and the soft-argmax objective are small dense torch operations.

The reference has no differentiable path (its ``DIFF_NLPAR`` class is an empty placeholder,
nlpar.py:75-77).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["radon_csr", "log_csr", "transpose_csr", "LinOp", "BandSharpness"]


def _bind():
    lib = _lib.load()
    if not getattr(lib, "_diff_bound", False):
        P = C.c_void_p
        lib.ebsd_linop_create.argtypes = [C.c_int64, C.c_int64, P, P, P, C.c_int, C.POINTER(P)]
        lib.ebsd_linop_apply.argtypes = [P, C.c_int, P, C.c_int64, P, P]
        lib.ebsd_linop_destroy.argtypes = [P]
        lib.ebsd_nlpar_weights.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, C.c_float, C.c_float,
                                           C.c_int32, C.c_float, P, C.c_int, P, P, P]
        lib.ebsd_nlpar_apply.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, P, P]
        lib.ebsd_nlpar_apply_t.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, P, P]
        lib.ebsd_nlpar_lambda_grad.argtypes = [P, P, C.c_int32, C.c_int32, C.c_int32, P, P, C.c_int32, C.c_float,
                                               P, P]
        lib.ebsd_nlpar_apply64.argtypes = lib.ebsd_nlpar_apply.argtypes
        lib.ebsd_nlpar_apply_t64.argtypes = lib.ebsd_nlpar_apply_t.argtypes
        lib.ebsd_nlpar_lambda_grad64.argtypes = lib.ebsd_nlpar_lambda_grad.argtypes
        for f in ("ebsd_linop_create", "ebsd_linop_apply", "ebsd_linop_destroy", "ebsd_nlpar_weights",
                  "ebsd_nlpar_apply", "ebsd_nlpar_apply_t", "ebsd_nlpar_lambda_grad", "ebsd_nlpar_apply64",
                  "ebsd_nlpar_apply_t64", "ebsd_nlpar_lambda_grad64"):
            getattr(lib, f).restype = C.c_int
        lib._diff_bound = True
    return lib


# ------------------------------------------------------------------------------------------
# sparse operators built from a band-detection plan
# ------------------------------------------------------------------------------------------
def radon_csr(bd):
    """R[ray, pixel] = 1/count(ray) over the ray's pixels; rays row-major (rho, theta)."""
    rp = bd.radonPlan
    H, W = int(rp.imDim[0]), int(rp.imDim[1])
    lut = rp.indexPlan.reshape(-1, rp.indexPlan.shape[-1])
    valid = lut < H * W
    cnt = valid.sum(1)
    rowptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    col = lut[valid].astype(np.int32)
    val = np.repeat((1.0 / np.maximum(cnt, 1)).astype(np.float32), cnt)
    return rowptr, col, val, (lut.shape[0], H * W)


def log_csr(bd):
    """Interior LoG response as a linear map of the interior Radon: every tap of the
    'same'-mode convolution (zero outside the padded array) reads a padded cell, which the
    padding rule maps back to one interior cell."""
    nR, nT = int(bd.radonPlan.nRho), int(bd.radonPlan.nTheta)
    p0, p1 = int(bd.padding[0]), int(bd.padding[1])
    R, Tp = nR + 2 * p0, nT + 2 * p1
    k = np.asarray(bd.kernel, dtype=np.float32).reshape(np.asarray(bd.kernel).shape[-2:])
    k0, k1 = k.shape
    h0, h1 = k0 // 2, k1 // 2

    def src(r, c):
        i, j = r - p0, c - p1
        ic = min(max(i, 0), nR - 1)
        if j < 0:
            return (nR - 1 - ic) * nT + (nT + j)
        if j >= nT:
            return (nR - 1 - ic) * nT + (j - nT)
        return ic * nT + j

    rows, cols, vals = [], [], []
    for i in range(nR):
        for j in range(nT):
            r, c = i + p0, j + p1
            acc = {}
            for a in range(k0):
                rr = r + h0 - a
                if rr < 0 or rr >= R:
                    continue
                for b in range(k1):
                    cc = c + h1 - b
                    if cc < 0 or cc >= Tp:
                        continue
                    s = src(rr, cc)
                    acc[s] = acc.get(s, 0.0) + float(k[a, b])
            for s, v in sorted(acc.items()):
                rows.append(i * nT + j)
                cols.append(s)
                vals.append(v)
    rows = np.asarray(rows, dtype=np.int64)
    rowptr = np.zeros(nR * nT + 1, dtype=np.int64)
    np.add.at(rowptr, rows + 1, 1)
    return np.cumsum(rowptr).astype(np.int64), np.asarray(cols, np.int32), np.asarray(vals, np.float32), \
        (nR * nT, nR * nT)


def transpose_csr(rowptr, col, val, shape):
    nrows, ncols = shape
    rows = np.repeat(np.arange(nrows, dtype=np.int64), np.diff(rowptr))
    order = np.lexsort((rows, col))
    tcol = rows[order].astype(np.int32)
    tval = val[order]
    trow = np.zeros(ncols + 1, dtype=np.int64)
    np.add.at(trow, col.astype(np.int64) + 1, 1)
    return np.cumsum(trow).astype(np.int64), tcol, tval, (ncols, nrows)


class LinOp:
    """A device CSR operator (ebsd_linop)."""

    def __init__(self, rowptr, col, val, shape, device=0):
        lib = _bind()
        self._lib = lib
        self.rowptr = np.ascontiguousarray(rowptr, np.int64)
        self.col = np.ascontiguousarray(col, np.int32)
        self.val = np.ascontiguousarray(val, np.float32)
        self.shape = (int(shape[0]), int(shape[1]))
        h = C.c_void_p()
        _lib.check(lib.ebsd_linop_create(self.shape[0], self.shape[1], self.rowptr.ctypes.data, self.col.ctypes.data,
                                         self.val.ctypes.data, int(device), C.byref(h)), "ebsd_linop_create")
        self.handle = h

    def __call__(self, x):
        import torch
        x = x.contiguous()
        n = x.shape[0]
        y = torch.empty((n, self.shape[0]), dtype=x.dtype, device=x.device)
        _lib.check(self._lib.ebsd_linop_apply(self.handle, int(x.dtype == torch.float64), x.data_ptr(), n,
                                              y.data_ptr(), torch.cuda.current_stream(x.device).cuda_stream),
                   "ebsd_linop_apply")
        return y

    def dense(self):
        """Dense float64 copy (for reference computations)."""
        d = np.zeros(self.shape)
        rows = np.repeat(np.arange(self.shape[0]), np.diff(self.rowptr))
        np.add.at(d, (rows, self.col), self.val.astype(np.float64))
        return d

    def __del__(self):
        try:
            if self.handle.value:
                self._lib.ebsd_linop_destroy(self.handle)
        except Exception:
            pass


def _linop_fn():
    import torch

    class LinOpFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, op, opT):
            ctx.opT = opT
            return op(x)

        @staticmethod
        def backward(ctx, g):
            return ctx.opT(g.contiguous()), None, None

    return LinOpFn


def _nlpar_fn():
    import torch

    class NLPARFn(torch.autograd.Function):
        """y = W(lambda) x with W from the detached input (nlpar_nb weights); float32 or float64
        patterns (the weights are computed in float32 either way)."""

        @staticmethod
        def forward(ctx, x, lam, sigma, ind, datamax, nrows, ncols, sr, dthresh, sat):
            lib = _bind()
            st = torch.cuda.current_stream(x.device).cuda_stream
            winsz = (2 * sr + 1) ** 2
            xd = x.detach().contiguous()
            x32 = xd.to(torch.float32).contiguous()
            w = torch.empty((nrows * ncols, winsz), dtype=torch.float32, device=x.device)
            m = torch.empty_like(w)
            lamf = float(lam.detach().cpu())
            _lib.check(lib.ebsd_nlpar_weights(x32.data_ptr(), nrows, ncols, x32.shape[1], ind.data_ptr(), ind.numel(),
                                              float(datamax), lamf, sr, float(dthresh), sigma.data_ptr(), int(sat),
                                              w.data_ptr(), m.data_ptr(), st), "ebsd_nlpar_weights")
            y = torch.empty_like(xd)
            if xd.dtype == torch.float64:
                w64 = w.to(torch.float64)
                _lib.check(lib.ebsd_nlpar_apply64(xd.data_ptr(), nrows, ncols, xd.shape[1], w64.data_ptr(), sr,
                                                  y.data_ptr(), st), "ebsd_nlpar_apply64")
            else:
                _lib.check(lib.ebsd_nlpar_apply(xd.data_ptr(), nrows, ncols, xd.shape[1], w.data_ptr(), sr,
                                                y.data_ptr(), st), "ebsd_nlpar_apply")
            ctx.save_for_backward(xd, w, m)
            ctx.info = (nrows, ncols, sr, lamf)
            ctx.lam_dtype = lam.dtype
            return y

        @staticmethod
        def backward(ctx, g):
            lib = _bind()
            xd, w, m = ctx.saved_tensors
            nrows, ncols, sr, lamf = ctx.info
            g = g.contiguous().to(xd.dtype)
            st = torch.cuda.current_stream(g.device).cuda_stream
            gx = torch.empty_like(g)
            gl = torch.empty(nrows * ncols, dtype=torch.float64, device=g.device)
            if xd.dtype == torch.float64:
                w64 = w.to(torch.float64)
                _lib.check(lib.ebsd_nlpar_apply_t64(g.data_ptr(), nrows, ncols, g.shape[1], w64.data_ptr(), sr,
                                                    gx.data_ptr(), st), "ebsd_nlpar_apply_t64")
                _lib.check(lib.ebsd_nlpar_lambda_grad64(g.data_ptr(), xd.data_ptr(), nrows, ncols, g.shape[1],
                                                        w.data_ptr(), m.data_ptr(), sr, lamf, gl.data_ptr(), st),
                           "ebsd_nlpar_lambda_grad64")
            else:
                _lib.check(lib.ebsd_nlpar_apply_t(g.data_ptr(), nrows, ncols, g.shape[1], w.data_ptr(), sr,
                                                  gx.data_ptr(), st), "ebsd_nlpar_apply_t")
                _lib.check(lib.ebsd_nlpar_lambda_grad(g.data_ptr(), xd.data_ptr(), nrows, ncols, g.shape[1],
                                                      w.data_ptr(), m.data_ptr(), sr, lamf, gl.data_ptr(), st),
                           "ebsd_nlpar_lambda_grad")
            return gx, gl.sum().to(ctx.lam_dtype).reshape(()), None, None, None, None, None, None, None, None

    return NLPARFn


def gaussian_kernel1d(sigma, radius):
    import torch
    t = torch.arange(-radius, radius + 1, dtype=sigma.dtype, device=sigma.device)
    k = torch.exp(-0.5 * (t / sigma) ** 2)
    return k / k.sum()


class BandSharpness:
    """Soft-argmax band-sharpness objective of a scan grid of patterns (module-like callable).

    ``bd``: a configured ``BandDetect`` (Radon plan, LoG kernel, padding, rdnmask).
    Parameters: ``lam`` (NLPAR lambda), ``bg_sigma`` (background blur sigma) as torch scalars
    with ``requires_grad``; the input patterns may require grad too.  The input's dtype
    (float32, or float64 for gradient checks) sets the arithmetic of every stage except the
    NLPAR weights, which are computed in float32 as nlpar_nb does.
    """

    def __init__(self, bd, nrows, ncols, searchradius=2, dthresh=0.0, tau=1.0, bg_radius=None, device=0,
                 saturation_protect=True):
        import torch
        self.bd, self.nrows, self.ncols, self.sr = bd, int(nrows), int(ncols), int(searchradius)
        self.dthresh, self.tau, self.sat = float(dthresh), float(tau), bool(saturation_protect)
        H, W = int(bd.radonPlan.imDim[0]), int(bd.radonPlan.imDim[1])
        self.H, self.W = H, W
        self.bg_radius = bg_radius if bg_radius is not None else max(3, min(H, W) // 4)
        self.dev = torch.device("cuda", device)
        r = radon_csr(bd)
        self.R, self.RT = LinOp(*r, device=device), LinOp(*transpose_csr(*r), device=device)
        m = log_csr(bd)
        self.M, self.MT = LinOp(*m, device=device), LinOp(*transpose_csr(*m), device=device)
        self.rmask = torch.as_tensor(np.asarray(bd.rdnmask).reshape(-1), device=self.dev)
        from .nlpar import NLPAR
        mask = NLPAR.makeautomask(H, W)
        self.ind = torch.as_tensor(np.nonzero(mask.ravel())[0].astype(np.int32), device=self.dev)
        self._lin = _linop_fn()
        self._nl = _nlpar_fn()

    def sigma_of(self, x):
        """NLPAR noise sigma of the (detached) input, held fixed in the objective."""
        from .nlpar import NLPAR
        nl = NLPAR(lam=1.0, searchradius=self.sr, saturation_protect=self.sat)
        s = nl.calcsigma_array(x.detach().reshape(-1, self.H, self.W), self.nrows, self.ncols)
        return s.reshape(-1).contiguous()

    def stages(self, x, lam, bg_sigma, sigma=None):
        """All intermediate stages (for tests): y (NLPAR), z (background-subtracted), r (Radon),
        c (LoG), J."""
        import torch
        import torch.nn.functional as F
        n = self.nrows * self.ncols
        x = x.reshape(n, self.H * self.W)
        if sigma is None:
            sigma = self.sigma_of(x)
        datamax = float(x.detach().max())
        y = self._nl.apply(x, lam, sigma, self.ind, datamax, self.nrows, self.ncols, self.sr,
                           self.dthresh, self.sat)
        img = y.reshape(n, 1, self.H, self.W)
        k = gaussian_kernel1d(bg_sigma.to(x.dtype), self.bg_radius)
        pad = F.pad(img, (self.bg_radius, self.bg_radius, self.bg_radius, self.bg_radius), mode="reflect")
        blur = F.conv2d(F.conv2d(pad, k.reshape(1, 1, 1, -1)), k.reshape(1, 1, -1, 1))
        z = (img - blur).reshape(n, self.H * self.W)
        r = self._lin.apply(z.contiguous(), self.R, self.RT)
        c = self._lin.apply(r.contiguous(), self.M, self.MT)
        cm = c[:, self.rmask.bool()]
        s = torch.softmax(cm / self.tau, dim=1)
        J = (s * cm).sum(dim=1).mean()
        return y, z, r, c, J

    def __call__(self, x, lam, bg_sigma, sigma=None):
        return self.stages(x, lam, bg_sigma, sigma)[-1]
