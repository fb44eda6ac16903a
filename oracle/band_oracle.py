"""CPU restatement of the reference band-detection path (the oracle).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import this module, and only as the checker.  The product package
never imports it.

Each function restates one step of the reference (PyEBSDIndex v0.3.10.1) and cites the
file:line it follows.  Array conventions match the reference: the padded Radon is
``[nRho + 2*pad0, nTheta + 2*pad1, nPats]`` (pattern index last), the LUT is
``indexPlan[nRho, nTheta, max(H, W)]`` int64 sorted ascending with sentinel ``H*W + 1``.

Two convolution modes are provided:
  * ``conv="fft"``   -- ``scipy.signal.fftconvolve(..., mode="same")`` exactly as
                        band_detect.py:605-606 does (the reference arithmetic);
  * ``conv="direct"`` -- a direct 2-D correlation-free convolution in float64, used as the
                        FP64 reference the device kernels are graded against.
``dtype=np.float64`` runs the whole pipeline in double precision (the FP64 oracle).
"""
from __future__ import annotations

import numpy as np
import scipy.ndimage as ndi
import scipy.signal as sig

RADEG = 180.0 / np.pi
DEGRAD = np.pi / 180.0


# --------------------------------------------------------------------------------------
# Plan: Radon lookup table (radon_fast.py:64-191) and band-detect setup (band_detect.py:138-294)
# --------------------------------------------------------------------------------------
def radon_theta_rho(nTheta, nRho, rhoMax):
    """theta/rho sample vectors, radon_fast.py:87-89 (float32, same operation order)."""
    deltaRho = float(2 * np.float32(rhoMax)) / nRho
    theta = (np.arange(nTheta, dtype=np.float32) * np.float32(180.0)) / np.float32(nTheta)
    rho = np.arange(nRho, dtype=np.float32) * np.float32(deltaRho) - np.float32(
        np.float32(rhoMax) - np.float32(deltaRho))
    return theta, rho


def radon_lut(imDim, nTheta, nRho, rhoMax, mask=None, maskindex=None):
    """Ray lookup table, radon_fast.py:64-165 (+ mask defaults radon_fast.py:168-191).

    For |sin(theta)| >= sqrt(2)/2 each ray samples one pixel per image column,
    ``y = round(a*x + b1)``; otherwise one pixel per row, ``x = round(a*y + b1)``
    (radon_fast.py:111-158).  ``np.round`` is round-half-to-even.  Out-of-image samples,
    masked pixels and negative maskindex entries become the sentinel ``H*W+1``
    (radon_fast.py:159-163); each ray's list is then sorted ascending (radon_fast.py:165).
    sin/cos are numpy's float32 ufuncs, as in radon_fast.py:97-98; their last-bit behaviour is
    numpy's (it differs between CPU back ends), so the table matches the reference run on the
    same host.
    """
    H, W = int(imDim[0]), int(imDim[1])
    nPx = H * W
    if mask is None:
        mask = np.ones((H, W))
    mask = np.asarray(mask)
    if maskindex is None:
        maskindex = np.arange(nPx, dtype=np.int64).reshape(H, W)
    maskindex = np.asarray(maskindex).astype(np.int64)
    if maskindex.max() >= nPx:
        raise ValueError("max of index array must be less than the total number of pixel in the array")

    theta, rho = radon_theta_rho(nTheta, nRho, rhoMax)
    xmin = -1.0 * (W - 1) * 0.5
    ymin = -1.0 * (H - 1) * 0.5
    targ = (theta * np.float32(DEGRAD)).astype(np.float32)
    sT = np.sin(targ)
    cT = np.cos(targ)
    steep = np.abs(sT) >= (np.sqrt(2.0) * 0.5)
    a = (np.float32(-1.0) * np.where(steep, cT, sT)).astype(np.float32)
    a = (a / np.where(steep, sT, cT)).astype(np.float32)
    b = xmin * cT.astype(np.float64) + ymin * sT.astype(np.float64)

    oob = nPx + 1
    L = max(H, W)
    plan = np.full((nRho, nTheta, L), oob, dtype=np.int64)
    mcol = np.arange(W, dtype=np.float64)
    nrow = np.arange(H, dtype=np.float64)
    for i in range(nTheta):
        b1 = rho.astype(np.float64) - b[i]
        if steep[i]:
            b1 = (b1 / np.float64(sT[i])).reshape(nRho, 1)
            iy = np.round(np.float64(a[i]) * mcol + b1).astype(np.int64)
            iy = np.where((iy < 0) | (iy >= H), oob, iy)
            idx = np.clip(np.arange(W, dtype=np.int64) + W * iy, 0, oob)
            plan[:, i, 0:W] = idx
        else:
            b1 = (b1 / np.float64(cT[i])).reshape(nRho, 1)
            ix = np.round(np.float64(a[i]) * nrow + b1).astype(np.int64)
            ix = np.where((ix < 0) | (ix >= W), oob, ix)
            idx = np.clip(ix + W * np.arange(H, dtype=np.int64), 0, oob)
            plan[:, i, 0:H] = idx
    flat = plan.ravel()
    m = np.concatenate((mask.ravel().astype(np.int64), np.array([0, 0], dtype=np.int64)))
    flat = np.where(m[flat] > 0, flat, oob)
    mi = np.concatenate((maskindex.ravel(), np.array([-1, -1], dtype=np.int64)))
    flat = np.where(mi[flat] >= 0, mi[flat], oob)
    plan = flat.reshape(nRho, nTheta, L)
    plan.sort(axis=-1)
    return plan, theta, rho


def log_kernel(rSigma, tSigma):
    """LoG kernel, peak padding, band_detect.py:277-290."""
    ksz = np.array([max(np.int64(4 * rSigma), 5), max(np.int64(4 * tSigma), 5)])
    ksz = ksz + ((ksz % 2) == 0)
    k = np.zeros(ksz, dtype=np.float32)
    k[int(ksz[0] / 2), int(ksz[1] / 2)] = 1
    k = -1.0 * ndi.gaussian_filter(k, [rSigma, tSigma], order=[2, 0])
    k *= 1.0 / np.max(k)
    peakPad = np.array(np.around([2 * ksz[0], 2 * ksz[1]]), dtype=np.int64)
    peakPad += 1 - np.mod(peakPad, 2)
    padding = np.array([max(peakPad[0], 11), max(peakPad[1], 11)])
    return k.astype(np.float32), peakPad, padding


class Plan:
    """Everything BandDetect.band_detect_setup derives for one pattern size.

    band_detect.py:186-193 (rhoMax, dRho), radon_fast.py:64-165 (LUT),
    band_detect.py:203-251 (rdnmask), band_detect.py:269-290 (sigmas, kernel, padding).
    """

    def __init__(self, patDim, nTheta=180, nRho=90, tSigma=None, rSigma=None, rhoMaskFrac=0.1,
                 nBands=9, mask=None, maskindex=None, background=None):
        H, W = int(patDim[0]), int(patDim[1])
        self.patDim = np.array([H, W])
        self.nTheta, self.nRho, self.nBands = int(nTheta), int(nRho), int(nBands)
        self.rhoMaskFrac = rhoMaskFrac
        if 0 < rhoMaskFrac < 1:
            self.rhoMax = 0.5 * np.float32(min(H, W))
        else:
            self.rhoMax = 0.5 * np.float32(np.sqrt(np.float32(H) ** 2 + np.float32(W) ** 2))
        self.dTheta = 180.0 / self.nTheta
        self.dRho = self.rhoMax / np.float32(self.nRho)
        self.lut, self.theta, self.rho = radon_lut((H, W), nTheta, nRho, self.rhoMax, mask, maskindex)
        self.nPx = H * W
        self.count = (self.lut < self.nPx).sum(axis=-1)
        # rdnmask: radon of the mask image without normalisation is the in-mask count
        # (band_detect.py:210-215), trimmed by rhoMaskFrac (band_detect.py:220-247).
        rdnmask = self.count > 0
        if rhoMaskFrac >= (1 - 1.0e-12):
            rdnmask = ndi.binary_erosion(rdnmask, structure=np.ones((3, 1)), iterations=int(rhoMaskFrac))
        elif rhoMaskFrac > 0:
            mskinx = max(int(self.nRho * rhoMaskFrac), 1)
            trim = rdnmask.copy()
            trim[0:mskinx, :] = 0
            trim[-mskinx:, :] = 0
            rdnmask = rdnmask & trim
        elif rhoMaskFrac < 0:
            cx = (np.arange(W) - W * 0.5) ** 2
            cy = (np.arange(H) - H * 0.5) ** 2
            cm = np.sqrt(cx.reshape(1, W) + cy.reshape(H, 1))
            cm = (cm < self.rhoMax * (1.0 + rhoMaskFrac)).astype(np.float32)
            vals = np.concatenate((cm.ravel(), [0, 0]))[np.minimum(self.lut, self.nPx)]
            rdnmask = rdnmask & ((vals.sum(-1) / np.maximum(self.count, 1) > 0) & (self.count > 0))
        self.rdnmask = rdnmask
        if tSigma is None:
            tSigma = 1.0 / self.dTheta
        if rSigma is None:
            rSigma = 0.5 / np.float32(self.dRho)
        self.tSigma, self.rSigma = tSigma, rSigma
        self.kernel, self.peakPad, self.padding = log_kernel(rSigma, tSigma)
        self.background = background


# --------------------------------------------------------------------------------------
# Per-chunk pipeline
# --------------------------------------------------------------------------------------
def radon_gather(plan: Plan, pats, dtype=np.float32):
    """Mean of in-mask samples along each ray, radon_fast.py:242-310.

    Background subtraction in float64 then cast (radon_fast.py:255-259).  The float32 sum runs
    sequentially over the ray's sorted LUT entries (rdn_loops, radon_fast.py:299-305) -- the
    loop below adds a zero for finished rays, which leaves a float sum unchanged.  Empty rays
    keep ``missingval = -1`` (radon_fast.py:265).  Returns the padded array (padding cells -1).
    """
    n = pats.shape[0]
    H, W = plan.patDim
    if plan.background is None:
        img = pats.reshape(n, -1).astype(dtype)
    else:
        img = (pats - plan.background).reshape(n, -1).astype(dtype)
    img = np.concatenate((img, np.zeros((n, 2), dtype=dtype)), axis=1)  # sentinel slots
    p0, p1 = plan.padding
    lut = np.minimum(plan.lut, plan.nPx)  # clamp sentinel to a zero slot
    acc = np.zeros((plan.nRho, plan.nTheta, n), dtype=dtype)
    imgT = np.ascontiguousarray(img.T)  # [nPx+2, n]
    for k in range(lut.shape[2]):
        col = lut[:, :, k]
        if np.all(col >= plan.nPx):
            break
        acc += imgT[col]
    cnt = plan.count.astype(dtype)[:, :, None]
    val = np.where(cnt >= 1, acc / np.where(cnt >= 1, cnt, 1), dtype(-1.0)).astype(dtype)
    out = np.full((plan.nRho + 2 * p0, plan.nTheta + 2 * p1, n), -1.0, dtype=dtype)
    out[p0:p0 + plan.nRho, p1:p1 + plan.nTheta, :] = val
    return out


def radon_pad(plan: Plan, radon):
    """theta mirror-with-rho-flip then rho edge replication, in place, band_detect.py:573-580."""
    p0, p1 = plan.padding
    if p1 > 0:
        radon[:, 0:p1, :] = np.flip(radon[:, -2 * p1:-p1, :], axis=0)
        radon[:, -p1:, :] = np.flip(radon[:, p1:2 * p1, :], axis=0)
    if p0 > 0:
        radon[0:p0, :, :] = radon[p0, :, :][None]
        radon[-p0:, :, :] = radon[-p0 - 1, :, :][None]
    return radon


def conv_direct(radon, kernel, dtype=np.float64):
    """'same'-mode 2-D convolution with zero extension, evaluated directly in ``dtype``."""
    k = kernel.astype(dtype)
    k0, k1 = k.shape
    h0, h1 = k0 // 2, k1 // 2
    R, T, n = radon.shape
    src = np.zeros((R + 2 * h0, T + 2 * h1, n), dtype=dtype)
    src[h0:h0 + R, h1:h1 + T] = radon
    out = np.zeros((R, T, n), dtype=dtype)
    for i in range(k0):
        for j in range(k1):
            # convolution flips the kernel: out[r,c] = sum k[i,j] * src[r + h0 - (i - h0), ...]
            out += k[k0 - 1 - i, k1 - 1 - j] * src[i:i + R, j:j + T]
    return out


def rdn_conv(plan: Plan, radon, conv="fft", dtype=np.float32):
    """band_detect.py:562-637: pad, convolve with the LoG, per-pattern min/mean/max.

    The statistics slice uses ``shprdn[1]`` (the padded theta size) as the rho bound,
    exactly as band_detect.py:627-630 does.
    """
    radon = radon_pad(plan, radon)
    shp = radon.shape
    if conv == "fft":
        k = plan.kernel[:, :, None]
        rdnConv = sig.fftconvolve(radon, k, mode="same")
    else:
        rdnConv = conv_direct(radon, plan.kernel, dtype=np.float64)
    rdnConv = rdnConv.astype(dtype)
    p0, p1 = plan.padding
    sl = rdnConv[p0:shp[1] - p0, p1:shp[1] - p1, :]
    mns = sl.min(axis=0).min(axis=0)
    mxs = sl.max(axis=0).max(axis=0)
    ave = np.mean(sl, axis=(0, 1))
    return rdnConv, [mns, ave, mxs]


def rdn_local_max(plan: Plan, rdn):
    """band_detect.py:639-664: 11x11 max filter (window clipped at the array edge), exact
    equality with the convolved value, AND the rho/theta mask placed in the padded frame."""
    pk0, pk1 = plan.peakPad
    d = ndi.maximum_filter(rdn, size=(1, pk1, 1), mode="nearest")
    d = ndi.maximum_filter(d, size=(pk0, 1, 1), mode="nearest")
    lmax = d == rdn
    p0, p1 = plan.padding
    m = np.zeros((plan.nRho + 2 * p0, plan.nTheta + 2 * p1, 1), dtype=bool)
    m[p0:-p0, p1:-p1, 0] = plan.rdnmask
    return lmax & m


def band_label(plan: Plan, rdnConv, lmax, dtype=np.float32):
    """band_label_numba, band_detect.py:691-809, one pattern at a time.

    Candidates are sorted by convolved value, largest first (np.argsort, band_detect.py:734,
    ties broken here by the stable order of np.nonzero); a band is valid only if its value is
    > 0 (:739).  FWHM width from the log-values at rho +-1 (:748-753); sub-pixel location by
    the Taylor step on the 3x3 neighbourhood normalised by its sum, with the two 0.875
    fallbacks (:764-792).  Returned locations are in the padded frame.
    """
    nB = plan.nBands
    n = rdnConv.shape[2]
    f = dtype
    bmax = np.full((n, nB), -2.0e6, dtype=f)
    bavemax = np.full((n, nB), -2.0e6, dtype=f)
    bvalid = np.zeros((n, nB), dtype=np.int8)
    bmaxloc = np.zeros((n, nB, 2), dtype=f)
    baveloc = np.zeros((n, nB, 2), dtype=f)
    bwidth = np.zeros((n, nB), dtype=f)
    for q in range(n):
        R = rdnConv[:, :, q]
        rr, cc = np.nonzero(lmax[:, :, q])
        vals = R[rr, cc]
        srt = np.argsort(-vals, kind="stable")
        for i in range(min(nB, len(srt))):
            r, c = int(rr[srt[i]]), int(cc[srt[i]])
            if not (R[r, c] > 0.0):
                continue
            bmaxloc[q, i] = (r, c)
            bmax[q, i] = R[r, c]
            bwidth[q, i] = 0.0
            if np.min(R[r - 1:r + 2, c]) > 0.0:
                a = (np.log(R[r + 1, c]) - np.log(R[r - 1, c])) * f(0.5) - np.log(bmax[q, i])
                if a < -1.e-8:
                    bwidth[q, i] = 2.0 * np.sqrt(np.log(2.0) / (-1.0 * a))
            nn = R[r - 1:r + 2, c - 1:c + 2].copy()
            sumnn = np.sum(nn)
            sumnn = sumnn if sumnn > 1e-12 else f(1e-12)
            nn = (nn / sumnn).astype(f)
            bavemax[q, i] = sumnn / f(9)
            dx = f(0.5) * (nn[1, 2] - nn[1, 0])
            dy = f(0.5) * (nn[2, 1] - nn[0, 1])
            dxx = nn[1, 2] + nn[1, 0] - f(2) * nn[1, 1]
            dyy = nn[2, 1] + nn[0, 1] - f(2) * nn[1, 1]
            dxy = f(0.25) * (nn[2, 2] - nn[0, 2] - nn[2, 0] + nn[0, 0])
            det = dxx * dyy - dxy * dxy
            det = det if np.fabs(det) > 1e-12 else f(1.0e-12)
            det = f(1.0) / det
            dc = (dyy * dx - dxy * dy) * det
            rc = (dxx * dy - dxy * dx) * det
            if (np.abs(dc) > 0.875) or (np.abs(rc) > 0.875):
                det = dxx * dyy
                det = det if np.fabs(det) > 1e-12 else f(1.0e-12)
                det = f(1.0) / det
                dc = (dyy * dx) * det
                rc = (dxx * dy) * det
                if (np.abs(dc) > 0.875) or (np.abs(rc) > 0.875):
                    dc = f(0.0)
                    rc = f(0.0)
            baveloc[q, i, 0] = r - rc
            baveloc[q, i, 1] = c - dc
            bvalid[q, i] = 1
    return bmax, bavemax, bmaxloc, baveloc, bvalid, bwidth


def record_dtype(nPhases=10):
    """The band record, band_detect.py:110-115."""
    return np.dtype([('id', np.int32), ('max', np.float32), ('normmax', np.float32),
                     ('maxloc', np.float32, (2)), ('avemax', np.float32), ('aveloc', np.float32, (2)),
                     ('pqmax', np.float32), ('width', np.float32), ('theta', np.float32), ('rho', np.float32),
                     ('valid', np.int8),
                     ('band_match_index', np.int64, (nPhases,)),
                     ('bandfit', np.float64, (nPhases,))])


def find_bands(plan: Plan, patterns, chunksize=512, conv="fft", dtype=np.float32, nPhases=10,
               return_intermediates=False):
    """BandDetect.find_bands, band_detect.py:411-526 (chunk loop, normmax, theta/rho)."""
    if patterns.ndim == 2:
        patterns = patterns[None]
    nP = patterns.shape[0]
    out = np.zeros((nP, plan.nBands), dtype=record_dtype(nPhases))
    if chunksize <= 0:
        chunksize = max(nP, 1)
    inter = []
    for s in range(0, nP, chunksize):
        e = min(nP, s + chunksize)
        rdn = radon_gather(plan, patterns[s:e], dtype=dtype)
        conv_out, (mn, ave, _mx) = rdn_conv(plan, rdn, conv=conv, dtype=dtype)
        lmax = rdn_local_max(plan, conv_out)
        bmax, bavemax, bmaxloc, baveloc, bvalid, bwidth = band_label(plan, conv_out, lmax, dtype=dtype)
        ch = out[s:e]
        ch['max'] = bmax
        norm = bmax.astype(np.float32) - mn.reshape(-1, 1).astype(np.float32)
        norm /= (ave - mn).reshape(-1, 1).astype(np.float32).clip(1e-7)
        ch['normmax'] = norm
        ch['avemax'] = bavemax
        ch['maxloc'] = bmaxloc - plan.padding.reshape(1, 1, 2)
        ch['aveloc'] = baveloc.astype(np.float64) - plan.padding.reshape(1, 1, 2)
        ch['valid'] = bvalid
        ch['width'] = bwidth
        if return_intermediates:
            inter.append((conv_out, lmax, mn, ave))
    out['theta'] = np.pi - np.interp(out['aveloc'][:, :, 1], np.arange(plan.nTheta), plan.theta) / RADEG
    out['rho'] = -1.0 * np.interp(out['aveloc'][:, :, 0], np.arange(plan.nRho), plan.rho)
    if return_intermediates:
        return out, inter
    return out
