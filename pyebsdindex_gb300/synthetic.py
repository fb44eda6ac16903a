"""Seeded synthetic EBSD patterns (Kikuchi-band sums) for tests and benchmarks.

No public dataset is used.  A pattern is the sum of Gaussian-profile bands, one per FCC
{111}, {200}, {220}, {311} lattice plane (25 planes up to sign), rotated by a uniform random
quaternion (Shoemake's method) and projected gnomonically onto the detector.  The band trace
of a plane with unit normal ``n`` is the detector line ``n . (P - t) = 0``, where ``t`` is the
source point -- the same detector frame the reference's ``Radon.radon2pole`` uses
(radon_fast.py:363-396: origin at the bottom-left pixel, ``t = PC * [W, H, -min(H, W)]`` for
EDAX pattern centres).  A smooth 2-D Gaussian background is added, the expected counts are
scaled to a peak count, Poisson noise is drawn and the result is clipped to the integer range
of the output type, then a circular detector mask is applied.
"""
from __future__ import annotations

import numpy as np

__all__ = ["fcc_plane_normals", "random_quaternions", "quat_to_matrix", "circular_mask",
           "make_patterns", "voronoi_scan", "voronoi_scan_rows"]


def fcc_plane_normals():
    """Unit normals and relative intensities of the FCC {111},{200},{220},{311} planes."""
    fams = [((1, 1, 1), 1.0), ((2, 0, 0), 0.8), ((2, 2, 0), 0.6), ((3, 1, 1), 0.45)]
    normals, weights = [], []
    for hkl, w in fams:
        seen = set()
        h = np.array(hkl)
        for perm in {(h[0], h[1], h[2]), (h[0], h[2], h[1]), (h[1], h[0], h[2]),
                     (h[1], h[2], h[0]), (h[2], h[0], h[1]), (h[2], h[1], h[0])}:
            for sx in (1, -1):
                for sy in (1, -1):
                    for sz in (1, -1):
                        v = np.array(perm) * np.array([sx, sy, sz])
                        key = tuple(v) if tuple(v) > tuple(-v) else tuple(-v)
                        if key in seen or not np.any(v):
                            continue
                        seen.add(key)
                        normals.append(np.array(key, dtype=np.float64) / np.linalg.norm(key))
                        weights.append(w)
    return np.array(normals), np.array(weights)


def random_quaternions(rng, n):
    """Uniform random unit quaternions (Shoemake 1992)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    return np.stack([b * np.cos(2 * np.pi * u3), a * np.sin(2 * np.pi * u2),
                     a * np.cos(2 * np.pi * u2), b * np.sin(2 * np.pi * u3)], axis=-1)


def quat_to_matrix(q):
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], -2)


def circular_mask(h, w):
    """Circular detector mask of radius 0.98*min(h, w)/2 centred on the pattern
    (same geometry as nlpar_cpu.NLPAR.makeautomask, nlpar_cpu.py:737-750)."""
    r = min(h, w) * 0.98 * 0.5
    x = np.arange(w, dtype=np.float32)
    x = np.minimum(x, w - x).reshape(1, w)
    y = np.arange(h, dtype=np.float32)
    y = np.minimum(y, h - y).reshape(h, 1)
    m = (np.sqrt(y ** 2 + x ** 2) < r).astype(np.uint8)
    return np.roll(m, (int(h / 2), int(w / 2)), axis=(0, 1))


def _render(quats, h, w, pc, band_sigma, bg_amp, noise_only):
    normals, weights = fcc_plane_normals()
    n = quats.shape[0]
    R = quat_to_matrix(quats)                                  # [n,3,3]
    nd = np.einsum("nij,kj->nki", R, normals)                  # [n,25,3] detector-frame normals
    t = np.array([pc[0] * w, pc[1] * h, -pc[2] * min(h, w)])
    X = np.arange(w, dtype=np.float64).reshape(1, 1, w)
    Y = (h - 1 - np.arange(h, dtype=np.float64)).reshape(1, h, 1)
    img = np.zeros((n, h, w))
    for k in range(normals.shape[0]):
        nk = nd[:, k, :]
        den = np.sqrt(nk[:, 0] ** 2 + nk[:, 1] ** 2).clip(1e-9)
        d = (nk[:, 0, None, None] * (X - t[0]) + nk[:, 1, None, None] * (Y - t[1])
             - nk[:, 2, None, None] * t[2]) / den[:, None, None]
        img += weights[k] * np.exp(-0.5 * (d / band_sigma) ** 2)
    img[noise_only] = 0.0
    img /= np.maximum(img.reshape(n, -1).max(axis=1), 1e-12).reshape(n, 1, 1)
    yy, xx = np.mgrid[0:h, 0:w]
    bg = bg_amp * np.exp(-(((xx - 0.5 * w) / (0.45 * w)) ** 2 + ((yy - 0.6 * h) / (0.45 * h)) ** 2))
    return img + bg[None]


def make_patterns(n, h=60, w=60, seed=0, dtype=np.uint8, peak=200.0, pc=(0.46, 0.70, 0.64),
                  band_sigma=1.5, bg_amp=0.5, noise_frac=0.0, mask=True, start=0):
    """``n`` seeded patterns; pattern ``i`` uses ``np.random.default_rng(seed + start + i)``.

    ``noise_frac`` of the patterns (those whose per-pattern draw falls below it) carry no
    bands: background plus Poisson noise only.  Returns (patterns[n,h,w], quats[n,4],
    noise_only[n] bool).
    """
    quats = np.zeros((n, 4))
    noise_only = np.zeros(n, dtype=bool)
    lam_scale = np.zeros(n)
    rngs = [np.random.default_rng(seed + start + i) for i in range(n)]
    for i, g in enumerate(rngs):
        quats[i] = random_quaternions(g, 1)[0]
        noise_only[i] = g.random() < noise_frac
        lam_scale[i] = 1.0
    expected = _render(quats, h, w, pc, band_sigma, bg_amp, noise_only)
    expected /= expected.reshape(n, -1).max(axis=1).reshape(n, 1, 1)
    out = np.empty((n, h, w), dtype=np.float64)
    for i, g in enumerate(rngs):
        out[i] = g.poisson(peak * expected[i])
    if np.issubdtype(np.dtype(dtype), np.integer):
        info = np.iinfo(dtype)
        out = np.clip(out, info.min, info.max)
    if mask:
        out *= circular_mask(h, w)[None]
    return out.astype(dtype), quats, noise_only


def voronoi_scan(nrows, ncols, ngrains=300, h=80, w=80, seed=0, peak_range=(30.0, 200.0),
                 pc=(0.46, 0.70, 0.64)):
    """Scan grid of patterns from seeded Voronoi grains (uniform random orientations), each
    scan pixel with its own Poisson peak count drawn from ``peak_range``.  Returns uint8
    patterns[nrows*ncols, h, w] and the grain id map[nrows, ncols]."""
    g = np.random.default_rng(seed)
    seeds = g.random((ngrains, 2)) * np.array([nrows, ncols])
    gq = random_quaternions(g, ngrains)
    rr, cc = np.mgrid[0:nrows, 0:ncols]
    pts = np.stack([rr.ravel(), cc.ravel()], -1).astype(np.float64)
    gid = np.empty(pts.shape[0], dtype=np.int64)
    for s in range(0, pts.shape[0], 4096):
        d = ((pts[s:s + 4096, None, :] - seeds[None]) ** 2).sum(-1)
        gid[s:s + 4096] = d.argmin(1)
    peaks = g.uniform(peak_range[0], peak_range[1], size=pts.shape[0])
    mk = circular_mask(h, w)
    base = _render(gq, h, w, pc, 1.5, 0.5, np.zeros(ngrains, dtype=bool))
    base /= base.reshape(ngrains, -1).max(axis=1).reshape(ngrains, 1, 1)
    out = np.empty((pts.shape[0], h, w), dtype=np.uint8)
    for i in range(pts.shape[0]):
        lam = peaks[i] * base[gid[i]]
        out[i] = (np.clip(g.poisson(lam), 0, 255) * mk).astype(np.uint8)
    return out, gid.reshape(nrows, ncols)


def voronoi_scan_rows(nrows, ncols, r0, r1, ngrains=300, h=80, w=80, seed=0, peak_range=(30.0, 200.0),
                      pc=(0.46, 0.70, 0.64)):
    """Rows [r0, r1) of a seeded Voronoi-grain scan (grains, orientations and per-pixel peak
    counts as ``voronoi_scan`` draws them from ``seed``), with the Poisson noise of each row
    block drawn from its own stream ``(seed, r0)`` so that blocks can be generated in parallel.
    Returns uint8 patterns [(r1 - r0) * ncols, h, w]."""
    g = np.random.default_rng(seed)
    seeds = g.random((ngrains, 2)) * np.array([nrows, ncols])
    gq = random_quaternions(g, ngrains)
    peaks = g.uniform(peak_range[0], peak_range[1], size=nrows * ncols)
    rr, cc = np.mgrid[r0:r1, 0:ncols]
    pts = np.stack([rr.ravel(), cc.ravel()], -1).astype(np.float64)
    gid = np.empty(pts.shape[0], dtype=np.int64)
    for s in range(0, pts.shape[0], 4096):
        d = ((pts[s:s + 4096, None, :] - seeds[None]) ** 2).sum(-1)
        gid[s:s + 4096] = d.argmin(1)
    used = np.unique(gid)
    base = np.zeros((ngrains, h, w))
    base[used] = _render(gq[used], h, w, pc, 1.5, 0.5, np.zeros(len(used), dtype=bool))
    base[used] /= base[used].reshape(len(used), -1).max(axis=1).reshape(len(used), 1, 1)
    mk = circular_mask(h, w)
    noise = np.random.default_rng([seed, r0])
    out = np.empty((pts.shape[0], h, w), dtype=np.uint8)
    for i in range(pts.shape[0]):
        lam = peaks[r0 * ncols + i] * base[gid[i]]
        out[i] = (np.clip(noise.poisson(lam), 0, 255) * mk).astype(np.uint8)
    return out
