"""Differentiable band-sharpness objective with hand-written forward and adjoint kernels.

Forward, per pattern of a scan grid (all on the GPU):

    x --NLPAR(lam)--> y --minus Gaussian blur(sigma)--> z --Radon--> r --LoG--> c
    J = mean over patterns of sum_i softmax(c_i / tau) c_i    (soft-argmax band sharpness)

* NLPAR: the weighted neighbour average of nlpar_cpu.py:821-936.  The weights are functions of
  lambda and of the patterns themselves -- through each pair's distance
  d = (SSD - n s) / (s sqrt(2 n)), s = sigma_p^2 + sigma_c^2 (nlpar_cpu.py:897-917), and
  through the noise sigma, the minimum over the 3x3 neighbours of SSD / (2 n)
  (nlpar_cpu.py:753-796) -- and every one of these dependences is differentiated
  (``ebsd_nlpar_weights_grad``: the pair SSDs of each window, the sigma's minimising pair, the
  lambda term), beside W^T g for the average itself.
* Background: y minus a reflect-padded separable Gaussian blur of radius ``bg_radius``
  (``ebsd_blur1d``: forward, adjoint, and d/dsigma through the taps' derivative).
* Radon: the band-detection ray means (radon_fast.py:281-310) as a sparse operator R (empty
  rays give 0); backward is the back-projection R^T through the transposed lookup table.
* LoG: padding (theta mirror / rho edge, band_detect.py:573-580) followed by the LoG
  convolution (band_detect.py:596-606), restricted to the Radon interior, as a sparse operator
  M; backward is M^T (correlation with the kernel folded back through the padding map).
* Objective: ``ebsd_softargmax`` computes each pattern's soft-argmax value and its gradient
  s_i (1 + (c_i - J) / tau) over the Radon-mask cells in one pass.

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
        lib.ebsd_linop_apply_cols.argtypes = [P, C.c_int, P, C.c_int64, C.c_int64, P, C.c_int64, P]
        lib.ebsd_linop_destroy.argtypes = [P]
        lib.ebsd_nlpar_weights.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, C.c_float, C.c_float,
                                           C.c_int32, C.c_float, P, C.c_int, P, P, P]
        lib.ebsd_nlpar_apply.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, P, P]
        lib.ebsd_nlpar_apply_t.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, P, P]
        lib.ebsd_nlpar_lambda_grad.argtypes = [P, P, C.c_int32, C.c_int32, C.c_int32, P, P, C.c_int32, C.c_float,
                                               P, P]
        lib.ebsd_blur1d.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int64, C.c_int32, C.c_int32, P, C.c_int32,
                                    P, P]
        lib.ebsd_softargmax.argtypes = [C.c_int, P, C.c_int64, C.c_int64, P, C.c_int32, C.c_double, P, P, P]
        lib.ebsd_nlpar_sigma_arg.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, C.c_float, C.c_int,
                                             P, P, P, P]
        lib.ebsd_nlpar_weights_d.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, C.c_float,
                                             C.c_float, C.c_int32, C.c_float, P, C.c_int, P, P, P, P, P]
        lib.ebsd_nlpar_weights_grad.argtypes = [C.c_int, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P, P,
                                                P, C.c_double, P, C.c_float, C.c_int, P, P, P, P, P, P]
        lib.ebsd_nlpar_apply64.argtypes = lib.ebsd_nlpar_apply.argtypes
        lib.ebsd_nlpar_apply_t64.argtypes = lib.ebsd_nlpar_apply_t.argtypes
        lib.ebsd_nlpar_lambda_grad64.argtypes = lib.ebsd_nlpar_lambda_grad.argtypes
        for f in ("ebsd_linop_create", "ebsd_linop_apply", "ebsd_linop_apply_cols", "ebsd_linop_destroy",
                  "ebsd_nlpar_weights",
                  "ebsd_nlpar_apply", "ebsd_nlpar_apply_t", "ebsd_nlpar_lambda_grad", "ebsd_nlpar_apply64",
                  "ebsd_nlpar_apply_t64", "ebsd_nlpar_lambda_grad64", "ebsd_blur1d", "ebsd_softargmax",
                  "ebsd_nlpar_sigma_arg", "ebsd_nlpar_weights_d", "ebsd_nlpar_weights_grad"):
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
        """y = A x for a batch x [n, ncols] (float32 / float64 CUDA tensor) -> y [n, nrows], run
        with the patterns along the fast axis (``ebsd_linop_apply_cols``): a batch held as the
        transpose of a contiguous [ncols, n] tensor -- e.g. another LinOp's result -- is read
        where it lies, and y is returned as the transpose of a contiguous [nrows, n] tensor."""
        import torch
        n = x.shape[0]
        xT = x.t()
        if not xT.is_contiguous():
            xT = xT.contiguous()
        yT = torch.empty((self.shape[0], n), dtype=x.dtype, device=x.device)
        _lib.check(self._lib.ebsd_linop_apply_cols(self.handle, int(x.dtype == torch.float64), xT.data_ptr(), n, n,
                                                   yT.data_ptr(), n, torch.cuda.current_stream(x.device).cuda_stream),
                   "ebsd_linop_apply_cols")
        return yT.t()

    def apply_rows(self, x):
        """The same product on a pattern-major batch x [n, ncols] (``ebsd_linop_apply``, one
        thread per output row and pattern) -> contiguous y [n, nrows]; equal bit for bit."""
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
            return ctx.opT(g), None, None

    return LinOpFn


def _nlpar_fn():
    import torch

    class NLPARFn(torch.autograd.Function):
        """y = W(lambda, x) x: the nlpar_nb average (nlpar_cpu.py:821-936) with its window
        weights computed in float32 from the input, as nlpar_nb does, for float32 or float64
        patterns.  ``sigma`` None: the noise sigma is computed from the input too
        (sigma_numba, nn = 1) and differentiated through its minimising pair; a given sigma is
        held fixed.  Backward: W^T g plus the weights' dependence on lambda, on each pair's
        distance and on the noise sigma."""

        @staticmethod
        def forward(ctx, x, lam, sigma, ind, pmask, datamax, nrows, ncols, sr, dthresh, sat):
            lib = _bind()
            st = torch.cuda.current_stream(x.device).cuda_stream
            npix, winsz = nrows * ncols, (2 * sr + 1) ** 2
            xd = x.detach().contiguous()
            x32 = xd.to(torch.float32).contiguous()
            npx = x32.shape[1]
            dev = x.device
            if sigma is None:
                sig2 = torch.empty(npix, dtype=torch.float32, device=dev)
                arg = torch.empty(npix, dtype=torch.int32, device=dev)
                nsig = torch.empty(npix, dtype=torch.float32, device=dev)
                _lib.check(lib.ebsd_nlpar_sigma_arg(x32.data_ptr(), nrows, ncols, npx, ind.data_ptr(), ind.numel(),
                                                    float(datamax), int(sat), sig2.data_ptr(), arg.data_ptr(),
                                                    nsig.data_ptr(), st), "ebsd_nlpar_sigma_arg")
            else:
                s32 = sigma.detach().to(torch.float32).reshape(-1).contiguous()
                sig2 = (s32 * s32).contiguous()
                arg = torch.full((npix,), -1, dtype=torch.int32, device=dev)
                nsig = torch.ones(npix, dtype=torch.float32, device=dev)
            w = torch.empty((npix, winsz), dtype=torch.float32, device=dev)
            m, dS, dsg = torch.empty_like(w), torch.empty_like(w), torch.empty_like(w)
            lamf = float(lam.detach().cpu())
            _lib.check(lib.ebsd_nlpar_weights_d(x32.data_ptr(), nrows, ncols, npx, ind.data_ptr(), ind.numel(),
                                                float(datamax), lamf, sr, float(dthresh), sig2.data_ptr(), int(sat),
                                                w.data_ptr(), m.data_ptr(), dS.data_ptr(), dsg.data_ptr(), st),
                       "ebsd_nlpar_weights_d")
            y = torch.empty_like(xd)
            if xd.dtype == torch.float64:
                w64 = w.to(torch.float64)
                _lib.check(lib.ebsd_nlpar_apply64(xd.data_ptr(), nrows, ncols, npx, w64.data_ptr(), sr,
                                                  y.data_ptr(), st), "ebsd_nlpar_apply64")
            else:
                _lib.check(lib.ebsd_nlpar_apply(xd.data_ptr(), nrows, ncols, npx, w.data_ptr(), sr,
                                                y.data_ptr(), st), "ebsd_nlpar_apply")
            ctx.save_for_backward(xd, w, m, dS, dsg, arg, nsig, pmask)
            ctx.info = (nrows, ncols, sr, lamf, float(datamax), int(sat))
            ctx.lam_dtype = lam.dtype
            return y

        @staticmethod
        def backward(ctx, g):
            lib = _bind()
            xd, w, m, dS, dsg, arg, nsig, pmask = ctx.saved_tensors
            nrows, ncols, sr, lamf, datamax, sat = ctx.info
            npix, winsz = nrows * ncols, (2 * sr + 1) ** 2
            g = g.contiguous().to(xd.dtype)
            npx = g.shape[1]
            st = torch.cuda.current_stream(g.device).cuda_stream
            f64 = xd.dtype == torch.float64
            gx = torch.empty_like(g)
            if f64:
                _lib.check(lib.ebsd_nlpar_apply_t64(g.data_ptr(), nrows, ncols, npx, w.to(torch.float64).data_ptr(),
                                                    sr, gx.data_ptr(), st), "ebsd_nlpar_apply_t64")
            else:
                _lib.check(lib.ebsd_nlpar_apply_t(g.data_ptr(), nrows, ncols, npx, w.data_ptr(), sr, gx.data_ptr(),
                                                  st), "ebsd_nlpar_apply_t")
            scratch = torch.empty(3 * npix * winsz + npix, dtype=torch.float64, device=g.device)
            gl = torch.empty(npix, dtype=torch.float64, device=g.device)
            gw = torch.empty_like(g)
            _lib.check(lib.ebsd_nlpar_weights_grad(int(f64), g.data_ptr(), xd.data_ptr(), nrows, ncols, npx, sr,
                                                   w.data_ptr(), m.data_ptr(), dS.data_ptr(), dsg.data_ptr(),
                                                   float(lamf), pmask.data_ptr(), float(datamax), int(sat),
                                                   arg.data_ptr(), nsig.data_ptr(), scratch.data_ptr(), gl.data_ptr(),
                                                   gw.data_ptr(), st), "ebsd_nlpar_weights_grad")
            return (gx + gw, gl.sum().to(ctx.lam_dtype).reshape(()), None, None, None, None, None, None, None, None,
                    None)

    return NLPARFn


def gaussian_taps(sigma, radius):
    """Normalised Gaussian taps k_t = exp(-t^2 / (2 sigma^2)) / sum, t = -radius..radius, and
    their derivative dk_t / dsigma = k_t (t^2 - sum_u k_u u^2) / sigma^3 (sigma's dtype)."""
    import torch
    t = torch.arange(-radius, radius + 1, dtype=sigma.dtype, device=sigma.device)
    e = torch.exp(-0.5 * (t / sigma) ** 2)
    k = e / e.sum()
    t2 = t * t
    dk = k * (t2 - (k * t2).sum()) / sigma ** 3
    return k.contiguous(), dk.contiguous()


def _blur(lib, x, taps, r, H, W, axis, adjoint=False):
    import torch
    out = torch.empty_like(x)
    _lib.check(lib.ebsd_blur1d(int(x.dtype == torch.float64), int(adjoint), axis, x.data_ptr(), x.shape[0], H, W,
                               taps.data_ptr(), r, out.data_ptr(), torch.cuda.current_stream(x.device).cuda_stream),
               "ebsd_blur1d")
    return out


def _background_fn():
    import torch

    class BackgroundFn(torch.autograd.Function):
        """z = y - blur_sigma(y): separable Gaussian of radius r with reflect padding, along x
        then along y (ebsd_blur1d).  Backward: g - blur^T g, and dJ/dsigma = -<g, dblur/dsigma y>
        with dblur/dsigma = Y(k) X(dk) + Y(dk) X(k)."""

        @staticmethod
        def forward(ctx, y, sigma, r, H, W):
            lib = _bind()
            k, dk = gaussian_taps(sigma.detach().to(y.dtype), r)
            yd = y.detach().contiguous()
            tx = _blur(lib, yd, k, r, H, W, axis=1)
            z = yd - _blur(lib, tx, k, r, H, W, axis=0)
            ctx.save_for_backward(yd, tx, k, dk)
            ctx.info = (r, H, W)
            ctx.sdt = sigma.dtype
            return z

        @staticmethod
        def backward(ctx, g):
            lib = _bind()
            yd, tx, k, dk = ctx.saved_tensors
            r, H, W = ctx.info
            g = g.contiguous().to(yd.dtype)
            gy = g - _blur(lib, _blur(lib, g, k, r, H, W, axis=0, adjoint=True), k, r, H, W, axis=1, adjoint=True)
            db = _blur(lib, tx, dk, r, H, W, axis=0) + _blur(lib, _blur(lib, yd, dk, r, H, W, axis=1), k, r, H, W,
                                                                   axis=0)
            gs = -(g * db).sum()
            return gy, gs.to(ctx.sdt).reshape(()), None, None, None

    return BackgroundFn


def _softargmax_fn():
    import torch

    class SoftArgmaxFn(torch.autograd.Function):
        """J = mean_p sum_i softmax(c_p / tau)_i c_pi over the cells ``cells`` (ebsd_softargmax,
        which also returns dJ_p / dc)."""

        @staticmethod
        def forward(ctx, c, cells, tau):
            lib = _bind()
            c = c.detach().contiguous()
            n, ncell = c.shape
            Jp = torch.empty(n, dtype=torch.float64, device=c.device)
            grad = torch.zeros_like(c)
            _lib.check(lib.ebsd_softargmax(int(c.dtype == torch.float64), c.data_ptr(), n, ncell, cells.data_ptr(),
                                           cells.numel(), float(tau), Jp.data_ptr(), grad.data_ptr(),
                                           torch.cuda.current_stream(c.device).cuda_stream), "ebsd_softargmax")
            ctx.save_for_backward(grad)
            return Jp.mean().to(c.dtype)

        @staticmethod
        def backward(ctx, gJ):
            (grad,) = ctx.saved_tensors
            return grad * (gJ.to(grad.dtype) / grad.shape[0]), None, None

    return SoftArgmaxFn


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
        self.cells = torch.as_tensor(np.nonzero(np.asarray(bd.rdnmask).reshape(-1))[0].astype(np.int32), device=self.dev)
        from .nlpar import NLPAR
        mask = NLPAR.makeautomask(H, W)
        self.ind = torch.as_tensor(np.nonzero(mask.ravel())[0].astype(np.int32), device=self.dev)
        self.pmask = torch.as_tensor(mask.ravel().astype(np.uint8), device=self.dev)
        self._lin = _linop_fn()
        self._nl = _nlpar_fn()
        self._bg = _background_fn()
        self._sa = _softargmax_fn()

    def sigma_of(self, x):
        """NLPAR noise sigma of the (detached) input (to hold it fixed: pass it to ``stages``)."""
        from .nlpar import NLPAR
        nl = NLPAR(lam=1.0, searchradius=self.sr, saturation_protect=self.sat)
        s = nl.calcsigma_array(x.detach().reshape(-1, self.H, self.W), self.nrows, self.ncols)
        return s.reshape(-1).contiguous()

    def stages(self, x, lam, bg_sigma, sigma=None):
        """All intermediate stages (for tests): y (NLPAR), z (background-subtracted), r (Radon),
        c (LoG), J.  ``sigma``: None computes the NLPAR noise sigma from ``x`` and differentiates
        through it; a given sigma is held fixed."""
        n = self.nrows * self.ncols
        x = x.reshape(n, self.H * self.W)
        datamax = float(x.detach().max())
        y = self._nl.apply(x, lam, sigma, self.ind, self.pmask, datamax, self.nrows, self.ncols, self.sr,
                           self.dthresh, self.sat)
        z = self._bg.apply(y.contiguous(), bg_sigma, self.bg_radius, self.H, self.W)
        r = self._lin.apply(z.contiguous(), self.R, self.RT)
        c = self._lin.apply(r, self.M, self.MT)  # r stays in the operators' pattern-minor layout
        J = self._sa.apply(c.contiguous(), self.cells, self.tau)
        return y, z, r, c, J

    def __call__(self, x, lam, bg_sigma, sigma=None):
        return self.stages(x, lam, bg_sigma, sigma)[-1]
