"""CPU restatement of the reference NLPAR kernels (oracle).

TEST INFRASTRUCTURE ONLY (imported by tests/ and the golden generator as the checker).

* ``automask``     -- NLPAR.makeautomask, nlpar_cpu.py:737-750
* ``sigma``        -- the noise estimate of NLPAR.sigma_numba, nlpar_cpu.py:753-796: for each
                      scan pixel the minimum over its clipped 3x3 neighbourhood of
                      SSD / (2 n) across masked, non-saturated pixels, square-rooted
* ``nlpar``        -- NLPAR.nlpar_nb, nlpar_cpu.py:821-936: per scan pixel, the normalised
                      distance to every pattern of its (2 sr + 1)^2 window (the window shifts
                      inward at the scan edges), weights exp(-max(d - dthresh, 0) / lam^2),
                      centre weight 1, and the weighted average over all pattern pixels

Arithmetic follows the reference's float32 operation order: the squared differences are
accumulated sequentially over the masked pixel list, the weights are summed and applied in
window order.  The loops are vectorised over scan pixels, so each accumulation is a numpy
float32 array operation that performs the same scalar roundings.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def automask(h, w):
    """Circular mask radius 0.98*min(h,w)/2 centred on the pattern, nlpar_cpu.py:737-750."""
    r = min(h, w) * 0.98 * 0.5
    x = np.arange(w, dtype=np.float32)
    x = np.minimum(x, w - x).reshape(1, w)
    y = np.arange(h, dtype=np.float32)
    y = np.minimum(y, h - y).reshape(h, 1)
    m = (np.sqrt(y ** 2 + x ** 2) < r).astype(np.uint8)
    return np.roll(m, (int(h / 2), int(w / 2)), axis=(0, 1))


def _pair_ssd(data, idx0, idx1, indices, mxval, n_init):
    """Sequential float32 SSD and count over the masked pixels for pattern pairs."""
    d2 = np.zeros(idx0.shape, dtype=np.float32)
    n2 = np.full(idx0.shape, n_init, dtype=np.float32)
    a_all = data[idx0]
    b_all = data[idx1]
    for q in indices:
        a = a_all[..., q]
        b = b_all[..., q]
        ok = (b < mxval) & (a < mxval)
        t = (a - b).astype(np.float32)
        d2 = np.where(ok, (d2 + t * t).astype(np.float32), d2)
        n2 = np.where(ok, (n2 + f32(1.0)).astype(np.float32), n2)
    return d2, n2


def sigma(data, nrows, ncols, indices, saturation_protect=True):
    """Per-scan-pixel noise sigma, nlpar_cpu.py:753-796 (nn = 1)."""
    data = np.asarray(data, dtype=np.float32)
    mxval = np.max(data)
    mxval = f32(mxval + 1.0) if not saturation_protect else f32(mxval * 0.9961)
    jj, ii = np.mgrid[0:nrows, 0:ncols]
    mind = np.full((nrows, ncols), 1e24, dtype=np.float32)
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            if dj == 0 and di == 0:
                continue
            jn, inn = jj + dj, ii + di
            ok = (jn >= 0) & (jn < nrows) & (inn >= 0) & (inn < ncols)
            idx0 = (ii + ncols * jj)[ok]
            idx1 = (inn + ncols * jn)[ok]
            d2, n2 = _pair_ssd(data, idx0, idx1, indices, mxval, f32(1.0e-12))
            s0 = (d2 / (n2 * f32(2.0)).astype(np.float32)).astype(np.float32)
            cand = np.where(d2 >= 1.e-3, s0, f32(1e24))
            cur = mind[ok]
            mind[ok] = np.minimum(cur, cand)
    return np.sqrt(mind).astype(np.float32)


def window_bounds(i, sr, n):
    """Search window along one scan axis, shifted inward at the edges (nlpar_cpu.py:872-878)."""
    start = max(i - sr, 0) - max(i + sr - (n - 1), 0)
    end = min(i + sr, n - 1) + max(sr - i, 0) + 1
    return start, end


def nlpar(data, lam, sr, dthresh, sig, nrows, ncols, indices, saturation_protect=True):
    """Weighted neighbour average of every scan pixel, nlpar_cpu.py:821-936."""
    data = np.asarray(data, dtype=np.float32)
    lam = f32(lam)
    lam2 = f32(1.0) / (lam * lam)
    dthresh = f32(dthresh)
    mxval = np.max(data)
    mxval = f32(mxval + f32(1.0)) if not saturation_protect else f32(mxval * f32(0.999))
    winsz = (2 * sr + 1) ** 2
    npx = nrows * ncols
    nbr = np.zeros((npx, winsz), dtype=np.int64)
    for j in range(nrows):
        ys, ye = window_bounds(j, sr, nrows)
        for i in range(ncols):
            xs, xe = window_bounds(i, sr, ncols)
            c = 0
            for jn in range(ys, ye):
                for inn in range(xs, xe):
                    nbr[i + ncols * j, c] = inn + ncols * jn
                    c += 1
    idx0 = np.repeat(np.arange(npx)[:, None], winsz, axis=1)
    centre = nbr == idx0
    s2 = (sig.astype(np.float32) ** 2).astype(np.float32).ravel()
    d2, n2 = _pair_ssd(data, idx0, nbr, indices, mxval, f32(0.0))
    ssum = (s2[idx0] + s2[nbr]).astype(np.float32)
    d2 = (d2 - (n2 * ssum).astype(np.float32)).astype(np.float32)
    dnorm = (ssum * np.sqrt((f32(2.0) * n2).astype(np.float32))).astype(np.float32)
    d2 = np.where(dnorm > f32(1.e-8), (d2 / np.where(dnorm > 0, dnorm, 1)).astype(np.float32),
                  (f32(1e6) * n2).astype(np.float32))
    w = np.where(centre, f32(-1.0e6), d2).astype(np.float32)
    w = np.maximum((w - dthresh).astype(np.float32), f32(0.0))
    w = np.exp((f32(-1.0) * w * lam2).astype(np.float32)).astype(np.float32)
    tot = np.zeros(npx, dtype=np.float32)
    for c in range(winsz):
        tot = (tot + w[:, c]).astype(np.float32)
    w = (w / tot[:, None]).astype(np.float32)
    out = np.zeros_like(data)
    for c in range(winsz):
        out = (out + (data[nbr[:, c]] * w[:, c:c + 1]).astype(np.float32)).astype(np.float32)
    return out
