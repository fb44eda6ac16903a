"""Radon plan: the ray lookup table and the band-to-pole conversion.

Mirrors the interface of the reference's ``radon_fast.Radon`` (radon_fast.py:43-397) --
attribute names, argument meaning and errors -- so that callers that read ``radonPlan.theta``,
``.rho``, ``.nTheta``, ``.nRho``, ``.imDim``, ``.mask``, ``.maskindex``, ``.indexPlan`` or call
``.radon2pole`` keep working.  The table is built on the host once per pattern size (as in the
reference) and re-encoded for the GPU by ``ebsd_plan_create``.
"""
from __future__ import annotations

import numpy as np

RADEG = 180.0 / np.pi
DEGRAD = np.pi / 180.0


class Radon:
    def __init__(self, image=None, imageDim=None, nTheta=180, nRho=90, rhoMax=None, mask=None,
                 maskindex=None, missingval=-1.0):
        self.nTheta = nTheta
        self.nRho = nRho
        self.rhoMax = rhoMax
        self.mask = mask
        self.maskindex = maskindex
        self.missingval = missingval
        self.indexPlan = None
        if image is None and imageDim is None:
            self.theta = None
            self.rho = None
            self.imDim = None
        else:
            self.imDim = np.asarray(image.shape[-2:] if image is not None else imageDim[-2:])
            self.radon_plan_setup()

    # radon_fast.py:168-191
    def _masksetup(self, mask=None, maskindex=None):
        if mask is not None:
            self.mask = np.array(mask).astype(int)
        if maskindex is not None:
            self.maskindex = np.array(maskindex).astype(np.int64)
        if self.imDim is not None:
            nPx = int(self.imDim[0]) * int(self.imDim[1])
            if self.mask is None:
                self.mask = np.ones(self.imDim)
            if self.maskindex is None:
                self.maskindex = np.arange(nPx, dtype=np.int64).reshape(self.imDim)
            if self.maskindex.max() >= nPx:
                raise Exception("max of index array must be less than the total number of pixel in the array")

    def radon_plan_setup(self, image=None, imageDim=None, nTheta=None, nRho=None, rhoMax=None, mask=None,
                         maskindex=None):
        """Build ``indexPlan[nRho, nTheta, max(H, W)]`` (radon_fast.py:64-165).

        Each ray at angle theta and offset rho samples one pixel per image column when
        ``|sin theta| >= sqrt(2)/2`` (``y = round(a*x + b1)``), else one pixel per row
        (``x = round(a*y + b1)``); rounding is half-to-even in float64.  Samples outside the
        image, on masked pixels, or remapped to a negative maskindex become the sentinel
        ``H*W + 1``; each ray's indices are sorted ascending.  theta and rho are float32 with
        the reference's operation order, and sin/cos are numpy's float32 ufuncs.
        """
        if image is None and imageDim is not None:
            self.imDim = np.asarray(imageDim, dtype=np.int64)
        elif image is not None:
            self.imDim = np.asarray(np.shape(image)[-2:])
        if self.imDim is None:
            return -1
        if mask is not None:
            self.mask = mask
        if maskindex is not None:
            self.maskindex = maskindex
        self._masksetup()
        if nTheta is not None:
            self.nTheta = nTheta
        if nRho is not None:
            self.nRho = nRho
        if rhoMax is not None:
            self.rhoMax = rhoMax
        if self.rhoMax is None:
            self.rhoMax = np.linalg.norm(self.imDim) * 0.5
        H, W = int(self.imDim[0]), int(self.imDim[1])
        nPx = H * W
        nT, nR = int(self.nTheta), int(self.nRho)

        step = float(2 * self.rhoMax) / nR
        self.theta = (np.arange(nT, dtype=np.float32) * np.float32(180.0)) / np.float32(nT)
        if isinstance(self.rhoMax, np.float32):
            offs = np.float32(self.rhoMax - np.float32(step))
        else:
            offs = np.float64(self.rhoMax) - step
        self.rho = (np.arange(nR, dtype=np.float32) * np.float32(step) - offs).astype(np.float32)

        ang = (self.theta * np.float32(DEGRAD)).astype(np.float32)
        s = np.sin(ang)
        c = np.cos(ang)
        by_col = np.abs(s) >= (np.sqrt(2.0) * 0.5)
        slope = (np.where(by_col, -c, -s) / np.where(by_col, s, c)).astype(np.float32)
        x0 = -1.0 * (W - 1) * 0.5
        y0 = -1.0 * (H - 1) * 0.5
        off = x0 * c.astype(np.float64) + y0 * s.astype(np.float64)

        sentinel = nPx + 1
        L = max(H, W)
        plan = np.full((nR, nT, L), sentinel, dtype=np.int64)
        xs = np.arange(W, dtype=np.int64)
        ys = np.arange(H, dtype=np.int64)
        rho64 = self.rho.astype(np.float64)
        for t in range(nT):
            inter = rho64 - off[t]
            if by_col[t]:
                inter = (inter / np.float64(s[t]))[:, None]
                yy = np.round(np.float64(slope[t]) * xs.astype(np.float64)[None, :] + inter).astype(np.int64)
                bad = (yy < 0) | (yy >= H)
                plan[:, t, :W] = np.where(bad, sentinel, np.clip(xs[None, :] + W * yy, 0, sentinel))
            else:
                inter = (inter / np.float64(c[t]))[:, None]
                xx = np.round(np.float64(slope[t]) * ys.astype(np.float64)[None, :] + inter).astype(np.int64)
                bad = (xx < 0) | (xx >= W)
                plan[:, t, :H] = np.where(bad, sentinel, np.clip(xx + W * ys[None, :], 0, sentinel))
        keep = np.concatenate((np.asarray(self.mask).ravel().astype(np.int64), [0, 0]))
        remap = np.concatenate((np.asarray(self.maskindex).ravel().astype(np.int64), [-1, -1]))
        flat = plan.ravel()
        flat = np.where(keep[flat] > 0, flat, sentinel)
        flat = np.where(remap[flat] >= 0, remap[flat], sentinel)
        self.indexPlan = np.sort(flat.reshape(nR, nT, L), axis=-1)

    def ray_counts(self):
        """Number of in-mask pixels on each ray, [nRho, nTheta]."""
        nPx = int(self.imDim[0]) * int(self.imDim[1])
        return (self.indexPlan < nPx).sum(axis=-1)

    def radon2pole(self, bandData, PC=None, vendor='EDAX'):
        """Band (theta, rho) -> unit plane normal in the detector frame (radon_fast.py:314-397,
        Krieger Lassen 1994 eq. 3.1.6).  The band is the detector line through the foot point
        p = (rho cos, rho sin) + image centre with direction r = (-sin, cos, 0) (origin at the
        bottom-left pixel); its plane normal is r x (p - t) for the vendor's source point t
        (``source_points``).  float32 throughout, each product rounded before its difference as
        the reference's np.cross rounds it, so the normals equal the reference's bit for bit."""
        if PC is None:
            PC = DEFAULT_PC
        theta = np.asarray(bandData['theta'])
        rho = np.asarray(bandData['rho'])
        n_pat = theta.shape[0]
        t = source_points(PC, n_pat, self.imDim, vendor)[:, None, :]    # [n_pat, 1, 3]
        s, c = np.sin(theta), np.cos(theta)
        rows, cols = np.asarray(self.imDim, dtype=np.float32)[:2]
        # p - t, component by component (p lies in the detector plane)
        v0 = (rho * c + cols * 0.5) - t[..., 0]
        v1 = (rho * s + rows * 0.5) - t[..., 1]
        zero = np.zeros_like(s)
        v2 = zero - t[..., 2]
        ns = -1 * s
        normal = np.stack([c * v2 - zero * v1, zero * v0 - ns * v2, ns * v1 - c * v0], axis=-1)
        flat = normal.reshape(-1, 3)
        flat /= np.linalg.norm(flat, axis=1).clip(1e-12).reshape(-1, 1)
        return flat.reshape(normal.shape)


DEFAULT_PC = np.array([0.471659, 0.675044, 0.630139])


def source_points(PC, n_pat, imDim, vendor='EDAX'):
    """Source point t [n_pat, 3] (float32) of each pattern in the detector frame of
    ``Radon.radon2pole`` from its pattern centre, per vendor convention (radon_fast.py:348-378):
    EDAX (x W, y H, z -min(H, W)); Oxford (x, y, z scaled by W, z negated); EMsoft ((xpc, ypc,
    L, pixel size): x negated, shifted by the image centre, z = -L / pixel size); kikuchipy and
    Bruker (x W, y H, z -H, y measured from the top).  One pattern centre serves every pattern
    unless one is given per pattern."""
    ven = str.upper(vendor)
    width = 4 if ven == 'EMSOFT' else 3
    pc = np.asarray(PC, dtype=np.float32)
    if pc.ndim < 2 or pc.shape[0] != n_pat:
        pc = np.broadcast_to((pc if pc.ndim < 2 else pc[0])[:width], (n_pat, width))
    pc = np.array(pc, dtype=np.float32)
    rows, cols = np.asarray(imDim, dtype=np.float32)[:2]
    if ven == 'EMSOFT':
        t = pc[:, 0:3]
        t[:, 2] /= pc[:, 3]
        t[:, 0] *= -1.0
        t += np.array([cols / 2.0, rows / 2.0, 0.0])
        t[:, 2] *= -1.0
        return t
    scale = {'EDAX': (cols, rows, -np.min([rows, cols])), 'OXFORD': (cols, cols, -cols),
             'KIKUCHIPY': (cols, rows, -rows), 'BRUKER': (cols, rows, -rows)}.get(ven)
    t = pc if scale is None else pc * np.array(scale)
    if ven in ('KIKUCHIPY', 'BRUKER'):
        t[:, 1] = rows - t[:, 1]
    return t


VENDORS = {"EDAX": 0, "OXFORD": 1, "EMSOFT": 2, "KIKUCHIPY": 3, "BRUKER": 4}


def radon2pole_gpu(theta, rho, imDim, PC=None, vendor='EDAX', stream=None):
    """``Radon.radon2pole`` on the device (libebsdgpu ``ebsd_radon2pole``): band ``theta`` /
    ``rho`` as CUDA float32 tensors [nPats, nBands] (e.g. the device fields of a find_bands
    call) -> unit plane normals, a CUDA tensor [nPats, nBands, 3].  ``PC``: one pattern centre
    ([3], or [4] for EMSOFT with the pixel size) or one per pattern ([nPats, 3/4]); ``imDim``:
    (rows, columns).  No counterpart on the reference's GPU path (radon2pole runs on the host,
    radon_fast.py:314-397)."""
    import ctypes as C
    import torch
    from . import _lib
    lib = _lib.load()
    if not hasattr(lib, "_r2p_bound"):
        lib.ebsd_radon2pole.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        lib.ebsd_radon2pole.restype = C.c_int
        lib._r2p_bound = True
    ven = str.upper(vendor)
    if ven not in VENDORS:
        raise ValueError(f"unknown vendor {vendor!r}")
    if PC is None:
        PC = np.array([0.471659, 0.675044, 0.630139])
    theta = theta.to(torch.float32).contiguous()
    rho = rho.to(torch.float32).contiguous()
    if theta.shape != rho.shape or theta.dim() != 2:
        raise ValueError("theta and rho must be [nPats, nBands] tensors of the same shape")
    n, nb = theta.shape
    pc = torch.as_tensor(np.asarray(PC, dtype=np.float32) if not torch.is_tensor(PC) else PC,
                         dtype=torch.float32, device=theta.device).contiguous()
    width = 4 if ven == 'EMSOFT' else 3
    if pc.dim() == 1:
        if pc.numel() < width:
            raise ValueError(f"{ven} pattern centres need {width} numbers")
        stride = 0
    else:
        if pc.shape[1] < width:
            raise ValueError(f"{ven} pattern centres need {width} numbers")
        stride = pc.shape[1] if pc.shape[0] == n else 0
    out = torch.empty((n, nb, 3), dtype=torch.float32, device=theta.device)
    st = stream if stream is not None else torch.cuda.current_stream(theta.device).cuda_stream
    _lib.check(lib.ebsd_radon2pole(C.c_void_p(theta.data_ptr()), C.c_void_p(rho.data_ptr()), int(n), int(nb),
                                   int(imDim[0]), int(imDim[1]), VENDORS[ven], C.c_void_p(pc.data_ptr()),
                                   int(stride), C.c_void_p(out.data_ptr()), C.c_void_p(int(st))),
               "ebsd_radon2pole")
    return out
