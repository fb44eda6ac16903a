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

Arithmetic follows the reference's operation order and types: the squared differences are
accumulated sequentially over the masked pixel list, the weights are summed and applied in
window order.  ``sigma_numba`` keeps its sums in float32; in ``nlpar_nb`` the square
``np.float32(d0 - d1) ** np.int32(2)`` is float64 (float32 ** int32 promotes), so the
pair's sum, the subtraction of n (sigma0^2 + sigma1^2) and the division by the norm run in
float64 and the distance is rounded to float32 once, when the weight is stored
(nlpar_cpu.py:902-916).  That is the reference as it runs under numpy's promotion rules (the
import shim); numba types float32 ** int as float32, so the compiled reference, like the device
kernel, sums in float32.  For integer patterns whose pair sums stay below 2^24 the two agree;
for other data (stem_scale's square roots, large uint16 counts) they do not.  The loops are vectorised over scan pixels, so each accumulation is a numpy array
operation that performs the same scalar roundings.
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


def _pair_ssd64(data, idx0, idx1, indices, mxval):
    """nlpar_nb's pair sum (nlpar_cpu.py:902-909): float64 squares of the float32 differences,
    summed in float64 in masked-pixel order; the count in float32."""
    d2 = np.zeros(idx0.shape, dtype=np.float64)
    n2 = np.zeros(idx0.shape, dtype=np.float32)
    a_all = data[idx0]
    b_all = data[idx1]
    for q in indices:
        a = a_all[..., q]
        b = b_all[..., q]
        ok = (b < mxval) & (a < mxval)
        t = (a - b).astype(np.float32).astype(np.float64)
        d2 = np.where(ok, d2 + t * t, d2)
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


def diff_offsets(nrows, ncols, sr, diff_offset, calclim=None):
    """The per-pixel addition to the centre weight that nlpar_nb makes with a non-zero
    diff_offset (nlpar_cpu.py:880-925), as its loops run one after another: one array of
    per-slot additions (diff_step, float32) for the whole call; pixels of the calculated block
    ``calclim`` = (col0, row0, ncol, nrow) visited column by column, rows inner; at each pixel
    every window slot is visited in window order -- the pixel's own slot gains diff_offset, every
    other slot is set to 0 -- and the pixel's own slot value is added to its centre weight."""
    c0, r0, nc, nr = calclim if calclim is not None else (0, 0, ncols, nrows)
    winsz = (2 * sr + 1) ** 2
    step = np.zeros(winsz, dtype=np.float32)
    off = np.zeros((nrows, ncols), dtype=np.float32)
    for i in range(c0, c0 + nc):
        xs, xe = window_bounds(i, sr, ncols)
        for j in range(r0, r0 + nr):
            ys, ye = window_bounds(j, sr, nrows)
            own = (j - ys) * (xe - xs) + (i - xs)
            keep = step[own]
            step[:] = 0
            step[own] = f32(keep + f32(diff_offset))
            off[j, i] = step[own]
    return off


def nlpar(data, lam, sr, dthresh, sig, nrows, ncols, indices, saturation_protect=True, centre_offset=None):
    """Weighted neighbour average of every scan pixel, nlpar_cpu.py:821-936; ``centre_offset``
    [nrows, ncols] is added to each pixel's own weight (``diff_offsets``)."""
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
    d2, n2 = _pair_ssd64(data, idx0, nbr, indices, mxval)
    ssum = (s2[idx0] + s2[nbr]).astype(np.float32)
    d2 = d2 - (n2 * ssum).astype(np.float32).astype(np.float64)
    dnorm = (ssum * np.sqrt((f32(2.0) * n2).astype(np.float32))).astype(np.float32)
    d2 = np.where(dnorm > f32(1.e-8), (d2 / np.where(dnorm > 0, dnorm, 1).astype(np.float64)).astype(np.float32),
                  (f32(1e6) * n2).astype(np.float32))
    w = np.where(centre, f32(-1.0e6), d2).astype(np.float32)
    w = np.maximum((w - dthresh).astype(np.float32), f32(0.0))
    w = np.exp((f32(-1.0) * w * lam2).astype(np.float32)).astype(np.float32)
    if centre_offset is not None:
        co = np.asarray(centre_offset, dtype=np.float32).ravel()
        w = np.where(centre, (w + co[:, None]).astype(np.float32), w).astype(np.float32)
    tot = np.zeros(npx, dtype=np.float32)
    for c in range(winsz):
        tot = (tot + w[:, c]).astype(np.float32)
    w = (w / tot[:, None]).astype(np.float32)
    out = np.zeros_like(data)
    for c in range(winsz):
        out = (out + (data[nbr[:, c]] * w[:, c:c + 1]).astype(np.float32)).astype(np.float32)
    return out


# ---------------------------------------------------------------------------------------
# lambda optimisation: NLPAR.opt_lambda_cpu (nlpar_cpu.py:94-155) with calcsigma_cpu
# (nlpar_cpu.py:157-264) and _calcchunks (nlpar_cpu.py:973-1065)
# ---------------------------------------------------------------------------------------
def calcchunks(patdim, ncol, nrow, target_bytes, col_overlap=0, row_overlap=0):
    """Scan tiling of NLPAR._calcchunks (nlpar_cpu.py:973-1065): (column chunks, row chunks),
    each an int array [n, 2] of [start, end)."""
    col_overlap = min(col_overlap, ncol - 1)
    row_overlap = min(row_overlap, nrow - 1)
    mincol = 2 if ncol >= nrow else 1
    minrow = 2 if nrow > ncol else 1
    nbytes = patdim[-1] * patdim[-2] * 4 * 2 * ncol * nrow
    nchunks = int(np.ceil(nbytes / target_bytes))

    def axis(n, nch, overlap):
        step = max(n / nch, 1)
        nch = max(int(np.ceil(max(n / step, 1))), 1)
        step = max(int(np.round(step)), 1)
        stepov = min(step + 2 * overlap, n)
        out = []
        for c in range(nch):
            ch = [int(c * step) - int(overlap), int(c * step + stepov) - int(overlap)]
            out.append(ch)
            if ch[1] > n:
                break
        out = np.array(out, dtype=int)
        out[0, 0] = 0
        out[-1, 1] = n
        if len(out) > 1:
            out[-1, 0] = max(0, out[-2, 1] - 2 * int(overlap) - 1)
        return out, nch

    cols, ncol_chunks = axis(ncol, max(np.round(np.sqrt(nchunks * float(ncol) / nrow)), mincol), col_overlap)
    # the row count uses the column count before the column loop's early stop (nlpar_cpu.py:994)
    rows, _ = axis(nrow, max(np.ceil(nchunks / ncol_chunks), minrow), row_overlap)
    return cols, rows


def sigma_distances_chunk(data, nrows, ncols, indices, saturation_protect=True):
    """NLPAR.sigma_numba (nlpar_cpu.py:753-818) as calcsigma_cpu calls it, with nn and the
    row/column start-count arrays as uint64: ``j - nn`` wraps for the chunk's first row and
    column, whose windows are then empty (sigma sqrt(1e24), no distances).  Returns sigma
    [nrows, ncols] and the normalised distances / counts [nrows, ncols, 9] (numpy's float32
    scalar arithmetic for the normalisation, as the reference source evaluates under numpy)."""
    data = np.asarray(data, dtype=np.float32)
    n0 = f32(data.shape[-1])
    mxval = np.max(data)
    mxval = f32(mxval + 1.0) if not saturation_protect else f32(mxval * 0.9961)
    mind = np.full((nrows, ncols), 1e24, dtype=np.float32)
    dout = np.zeros((nrows, ncols, 9), np.float32)
    nout = np.zeros((nrows, ncols, 9), np.float32)
    nbr = np.full((nrows, ncols, 9, 2), -1, np.int64)
    jj, ii = np.mgrid[0:nrows, 0:ncols]
    live = (jj >= 1) & (ii >= 1)
    cstart = np.where(live, ii - 1, 0)
    cend = np.minimum(ii + 1, ncols - 1) + 1
    rstart = np.where(live, jj - 1, 0)
    width = cend - cstart
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            jn, inn = jj + dj, ii + di
            ok = live & (jn < nrows) & (inn < ncols)
            slot = (jn - rstart) * width + (inn - cstart)
            sj, si = jj[ok], ii[ok]
            sl = slot[ok]
            nbr[sj, si, sl, 0] = jn[ok]
            nbr[sj, si, sl, 1] = inn[ok]
            if dj == 0 and di == 0:
                nout[sj, si, sl] = n0
                continue
            d2, n2 = _pair_ssd(data, (ii + ncols * jj)[ok], (inn + ncols * jn)[ok], indices, mxval, f32(1.0e-12))
            nout[sj, si, sl] = n2
            dout[sj, si, sl] = d2
            s0 = (d2 / (n2 * f32(2.0)).astype(np.float32)).astype(np.float32)
            cand = np.where(d2 >= 1.e-3, s0, f32(1e24))
            mind[sj, si] = np.minimum(mind[sj, si], cand)
    sig = np.sqrt(mind).astype(np.float32)
    s2 = sig ** 2
    for j in range(nrows):
        for i in range(ncols):
            for q in range(9):
                if nout[j, i, q] > 0:
                    s12 = s2[j, i] + s2[nbr[j, i, q, 0], nbr[j, i, q, 1]]
                    dout[j, i, q] -= nout[j, i, q] * s12
                    dout[j, i, q] /= s12 * np.sqrt(2.0 * nout[j, i, q])
    return sig, dout, nout


def calcsigma_chunked(data, nrows, ncols, h, w, indices, saturation_protect, target_bytes):
    """calcsigma_cpu's tile loop (nlpar_cpu.py:205-262): sigma is the minimum over tiles; a
    tile's distances replace earlier ones where its counts are positive."""
    cols, rows = calcchunks([w, h], ncols, nrows, target_bytes, col_overlap=1, row_overlap=1)
    grid = np.asarray(data, np.float32).reshape(nrows, ncols, -1)
    sigma = np.zeros((nrows, ncols), np.float32) + 1e18
    n2 = np.zeros((nrows, ncols, 9), np.float32)
    d2 = np.zeros((nrows, ncols, 9), np.float32)
    for r0, r1 in rows:
        for c0, c1 in cols:
            chunk = grid[r0:r1, c0:c1].reshape((r1 - r0) * (c1 - c0), -1)
            sc, dc, nc = sigma_distances_chunk(chunk, r1 - r0, c1 - c0, indices, saturation_protect)
            sigma[r0:r1, c0:c1] = np.minimum(sigma[r0:r1, c0:c1], sc)
            n2[r0:r1, c0:c1] = np.select([nc > 0], [nc], default=n2[r0:r1, c0:c1])
            d2[r0:r1, c0:c1] = np.select([nc > 0], [dc], default=d2[r0:r1, c0:c1])
    return sigma, d2, n2


def lambda_metric(lam, d2, tw, dthresh):
    """The objective of opt_lambda_cpu (nlpar_cpu.py:107-113)."""
    temp = np.maximum(d2, dthresh)
    dw = np.exp(-(temp) / lam ** 2)
    w = np.sum(dw, axis=2) + 1e-12
    return np.mean(np.abs(tw - 1.0 / w))


def opt_lambda(d2, sigma_size, target_weights=(0.5, 0.34, 0.25), dthresh=0.0):
    """Bounded Nelder-Mead per target weight from lambda = 1 (nlpar_cpu.py:139-150)."""
    import scipy.optimize as opt
    dthresh = np.float32(dthresh)
    stride = 1 if sigma_size < 1e6 else 2
    out = []
    for tw in np.asarray(target_weights):
        r = opt.minimize(lambda_metric, 1.0, args=(d2[0::stride, 0::stride, :], tw, dthresh), method='Nelder-Mead',
                         bounds=[[0.001, 10.0]], options={'fatol': 0.0001})
        out.append(r['x'])
    return np.asarray(out).flatten()
