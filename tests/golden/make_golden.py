"""Generate the golden band-detection vectors from the reference PyEBSDIndex itself.

Run from the repository root on a machine that has the reference source tree:

    PYEBSDINDEX_REFERENCE=/path/to/PyEBSDIndex python tests/golden/make_golden.py

The reference's CPU ``BandDetect.find_bands`` (band_detect.py:411-526) is imported through
``oracle/refshim.py`` (numba, matplotlib and h5py replaced by stubs; the numeric code is the
reference's own Python) and run on seeded synthetic patterns and on the reference's own test
fixture ``pyebsdindex/tests/data/al_sim_20kv/al_sim_20kv.png`` (decoded here with zlib,
scaled to float32/255 as ``matplotlib.pyplot.imread`` does).  For the fixture the full
``EBSDIndexer.index_pats`` (band detection -> triplet voting -> quaternion) is also run, with
the pattern centre the reference's ``test_index_pats`` uses.

The NLPAR kernels (``NLPAR.sigma_numba`` and ``NLPAR.nlpar_nb``, nlpar_cpu.py:753-936) are
run on seeded Voronoi-grain scan grids the way ``calcnlpar_cpu`` calls them for one tile and
stored as ``tests/golden/nlpar_*.npz``.

Each band case is written to ``tests/golden/<name>.npz``: inputs, plan parameters (JSON), the plan
vectors the reference derived (theta, rho, rdnmask, kernel, per-ray counts, a hash of the LUT
and the LUT itself, ray ends stored as H*W+1) and every field of the band record array.
"""
from __future__ import annotations

import hashlib
import json
import os
import struct
import sys
import time
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refshim  # noqa: E402
from pyebsdindex_gb300 import synthetic as syn  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
FIELDS = ["id", "max", "normmax", "maxloc", "avemax", "aveloc", "pqmax", "width", "theta", "rho",
          "valid", "band_match_index", "bandfit"]


def read_png_gray8(path):
    """Minimal decoder for 8-bit greyscale, non-interlaced PNG (the fixture's format)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", None, None
    while pos < len(data):
        ln, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            w, h, depth, ctype, _c, _f, inter = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and ctype == 0 and inter == 0
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = zlib.decompress(idat)
    img = np.zeros((h, w), dtype=np.uint8)
    prev = np.zeros(w, dtype=np.int32)
    for r in range(h):
        ft = raw[r * (w + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=w, offset=r * (w + 1) + 1).astype(np.int32)
        cur = np.zeros(w, dtype=np.int32)
        for c in range(w):
            a = cur[c - 1] if c > 0 else 0
            b = prev[c]
            cc = prev[c - 1] if c > 0 else 0
            if ft == 0:
                v = line[c]
            elif ft == 1:
                v = line[c] + a
            elif ft == 2:
                v = line[c] + b
            elif ft == 3:
                v = line[c] + (a + b) // 2
            else:
                p = a + b - cc
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - cc)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else cc)
                v = line[c] + pred
            cur[c] = v & 0xFF
        img[r] = cur
        prev = cur
    return img


def lut_hash(lut):
    return hashlib.sha256(np.ascontiguousarray(lut.astype(np.int64)).tobytes()).hexdigest()


def run_case(ref, name, pats, params, mask=None, background=None, collect_bg=False, store_lut=True,
             index_pc=None, degenerate=()):
    bd = ref.band_detect.BandDetect(nTheta=params["nTheta"], nRho=params["nRho"],
                                    tSigma=params["tSigma"], rSigma=params["rSigma"],
                                    rhoMaskFrac=params["rhoMaskFrac"], nBands=params["nBands"])
    bd.band_detect_setup(patDim=pats.shape[-2:], patternmask=mask)
    if collect_bg:
        with np.errstate(all="ignore"):
            bd.collect_background(patsIn=pats)
        background = bd.backgroundsub
    elif background is not None:
        bd.backgroundsub = background
    t0 = time.time()
    out = refshim.find_bands(bd, pats, chunksize=params.get("chunksize", 512))
    dt = time.time() - t0
    rp = bd.radonPlan
    rec = {
        "patterns": pats,
        "params": json.dumps(params),
        "theta": rp.theta, "rho": rp.rho,
        "rdnmask": bd.rdnmask.astype(np.uint8),
        "kernel": bd.kernel[0].astype(np.float32),
        "padding": np.asarray(bd.padding), "peakPad": np.asarray(bd.peakPad),
        "rhoMax": np.float32(bd.rhoMax),
        "count": (rp.indexPlan < pats.shape[-1] * pats.shape[-2]).sum(-1).astype(np.int32),
        "lut_sha256": lut_hash(rp.indexPlan),
    }
    # patterns whose reference bands are set by FFT rounding noise (all-zero / constant input):
    # parity on them is checked against exact arithmetic instead (see the GPU tests)
    rec["degenerate"] = np.asarray(degenerate, dtype=np.int64)
    if mask is not None:
        rec["mask"] = np.asarray(mask).astype(np.uint8)
    if background is not None:
        rec["background"] = np.asarray(background, dtype=np.float64)
    if store_lut:
        # entries >= H*W all mean "end of ray"; store them as H*W+1 so uint16 holds them
        lut = np.minimum(rp.indexPlan, pats.shape[-1] * pats.shape[-2] + 1)
        rec["lut"] = lut.astype(np.uint16 if lut.max() < 65535 else np.int32)
    for f in FIELDS:
        rec["out_" + f] = out[f]
    if index_pc is not None:
        idx = ref.ebsd_index_single.EBSDIndexer(PC=index_pc, patDim=pats.shape[-2:],
                                                nTheta=params["nTheta"], nRho=params["nRho"],
                                                tSigma=params["tSigma"], rSigma=params["rSigma"],
                                                rhoMaskFrac=params["rhoMaskFrac"], nBands=params["nBands"])
        with np.errstate(all="ignore"):
            import warnings
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                data, banddata = idx.index_pats(pats)[0:2]
        rec["index_quat"] = data[-1]["quat"]
        rec["index_fit"] = data[-1]["fit"]
        rec["index_nmatch"] = data[-1]["nmatch"]
        rec["index_pc"] = np.asarray(index_pc)
        rec["index_band_theta"] = banddata["theta"]
        rec["index_band_rho"] = banddata["rho"]
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(f"{name}: {pats.shape} {pats.dtype} in {dt:.1f}s")


def nlpar_case(ref, name, nrows, ncols, h, w, sr, lam, dthresh, saturation_protect, seed, saturate=False):
    """NLPAR kernels exactly as calcnlpar_cpu calls them for a single tile
    (nlpar_cpu.py:486-509): sigma from sigma_numba with nn=1, then nlpar_nb over the grid."""
    N = ref.nlpar_cpu.NLPAR
    pats, _ = syn.voronoi_scan(nrows, ncols, ngrains=max(3, nrows * ncols // 12), h=h, w=w, seed=seed)
    if saturate:
        pats[::5, h // 2, :] = 255
    data = pats.reshape(nrows * ncols, h * w).astype(np.float32)
    mask = N.makeautomask(h, w)
    ind = np.asarray(mask.flatten().nonzero()[0], np.int64)
    t0 = time.time()
    with np.errstate(all="ignore"):
        sig = N.sigma_numba(data, 1, nrows, ncols, np.array([0, nrows], dtype=np.int64),
                            np.array([0, ncols], dtype=np.int64), ind, saturation_protect)[0]
        out = N.nlpar_nb(data, np.float32(lam), np.int64(sr), np.float32(dthresh), sig, nrows, ncols,
                         calclim=np.array([0, 0, ncols, nrows], dtype=np.int64), indices_in=ind,
                         saturation_protect=saturation_protect, diff_offset=np.float32(0.0))
    rec = dict(data=data, mask=mask, sigma=sig, out=out,
               params=json.dumps(dict(nrows=nrows, ncols=ncols, h=h, w=w, sr=sr, lam=lam, dthresh=dthresh,
                                      saturation_protect=saturation_protect)))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(f"{name}: {nrows}x{ncols} grid of {h}x{w} in {time.time() - t0:.1f}s")


def main():
    ref = refshim.load()
    nlpar_case(ref, "nlpar_8x10_40", 8, 10, 40, 40, sr=2, lam=0.7, dthresh=0.0, saturation_protect=True, seed=7)
    nlpar_case(ref, "nlpar_7x7_32_sat", 7, 7, 32, 32, sr=3, lam=0.9, dthresh=0.5, saturation_protect=False,
               seed=8, saturate=True)
    nlpar_case(ref, "nlpar_6x9_36_satp", 6, 9, 36, 36, sr=1, lam=0.5, dthresh=0.0, saturation_protect=True,
               seed=9, saturate=True)
    base = dict(nTheta=180, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1)

    # 60x60 uint8, nRho 90, nBands 8 (the CPU-runnable configuration), plus an all-zero and a
    # constant pattern (every Radon cell ties; no band is valid for the zero pattern).
    p, _, _ = syn.make_patterns(20, 60, 60, seed=1000, noise_frac=0.2)
    m60 = syn.circular_mask(60, 60)
    const = (np.full((60, 60), 50, dtype=np.uint8) * m60)
    p = np.concatenate([p, np.zeros((1, 60, 60), np.uint8), const[None]])
    run_case(ref, "c0_60_u8", p, dict(base, nRho=90, nBands=8), mask=m60, degenerate=(20, 21))

    # 80x80 uint8, nRho 120, nBands 9 (the batched configuration's pattern geometry).
    p, _, _ = syn.make_patterns(12, 80, 80, seed=2000, noise_frac=0.1)
    p[3] = syn.make_patterns(1, 80, 80, seed=2003, noise_frac=1.0)[0][0]
    run_case(ref, "c1_80_u8", p, dict(base, nRho=120, nBands=9), mask=syn.circular_mask(80, 80))

    # uint16 at 4000 counts with a fitted background (collect_background + backsub_fit).
    p, _, _ = syn.make_patterns(8, 60, 60, seed=3000, dtype=np.uint16, peak=4000.0)
    run_case(ref, "u16_bg_60", p, dict(base, nRho=90, nBands=10), mask=m60, collect_bg=True)

    # Non-square float32 patterns, default sigmas, rhoMaskFrac 0.15, no mask.
    p, _, _ = syn.make_patterns(6, 48, 64, seed=4000, mask=False)
    p = (p.astype(np.float32) / np.float32(255.0)).astype(np.float32)
    run_case(ref, "f32_rect_48x64", p, dict(nTheta=120, nRho=72, tSigma=None, rSigma=None,
                                             rhoMaskFrac=0.15, nBands=7))

    # Larger LoG kernel (sigma 2 -> 9x9 taps, 19-wide peak window, padding 19).
    p, _, _ = syn.make_patterns(4, 60, 60, seed=5000)
    run_case(ref, "sigma2_60_u8", p, dict(base, tSigma=2.0, rSigma=2.0, nRho=90, nBands=8), mask=m60)

    # rhoMaskFrac >= 1 (half-diagonal rhoMax, eroded mask) and < 0 (circle-limited).
    p, _, _ = syn.make_patterns(4, 40, 40, seed=6000, mask=False)
    run_case(ref, "rmf1_40_u8", p, dict(base, nRho=60, rhoMaskFrac=1.0, nBands=6))
    p, _, _ = syn.make_patterns(4, 40, 40, seed=6100, mask=False)
    run_case(ref, "rmfneg_40_u8", p, dict(base, nRho=60, rhoMaskFrac=-0.1, nBands=6))

    # The reference's own test fixture through find_bands and the full indexer
    # (EBSDIndexer defaults: tSigma 1.0, rSigma 1.2, rhoMaskFrac 0.15, nRho 90, nBands 9).
    png = os.path.join(refshim.REFERENCE_ROOT, "pyebsdindex", "tests", "data", "al_sim_20kv", "al_sim_20kv.png")
    al = (read_png_gray8(png).astype(np.float32) / np.float32(255.0)).astype(np.float32)
    run_case(ref, "al_sim_20kv", al[None], dict(nTheta=180, nRho=90, tSigma=1.0, rSigma=1.2,
                                                rhoMaskFrac=0.15, nBands=9),
             index_pc=(0.4, 0.72, 0.6))


if __name__ == "__main__":
    main()
