"""Golden vectors for triplet voting: the reference's ``BandIndexer.bandindex``.

Run from the repository root on a machine that has the reference source tree:

    python tests/golden/make_vote_golden.py           # writes tests/golden/vote_*.npz

Each case holds one phase library exactly as the reference's ``tripletvote.addphase`` builds it
(tripletvote.py:70-171, ``build_trip_lib`` :320-490: the triplet table, its permutation LUT and the
complete pole list with its angle table), a batch of band normals with their band intensities,
and what the reference's own ``bandindex`` (tripletvote.py:492-633, imported through
``oracle/refshim.py``, run in spawned worker processes) returns for them: quaternion, fit,
cm, pole match, nMatch, (ii, jj, band1, band2), acc_correct and the per-band fit -- plus the
vote's intermediates (weighted and plain accumulators, band family, band rank) and the TRIAD
assignment's per-band valid flags.

Inputs:
* ``vote_fcc_orient``: the reference's own band records of the 200 seeded 80x80 patterns in
  ``orient_80x80.npz``, turned into normals by the reference's ``radon2pole`` (EDAX, PC 0.46,
  0.70, 0.64) and weighted by the indexer's band intensity (_ebsd_index_single.py:751-758,
  captured from ``EBSDIndexer._indexbandsphase``), with the indexer's pq / iq.
* ``vote_{fcc,bcc,hcp}_syn*``: seeded synthetic normals -- nBands library poles (distinct up to
  sign) under a random rotation, 0.4 deg of angular noise, random signs, descending
  intensities; 8 % invalid bands (intensity 0), 5 % noise-only patterns.  Variants: simple
  QUEST weights, no early exit, 12 bands, 4 bands.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))

LIB_KEYS = ("polesCart", "familyid", "angTable", "nFamily", "famIndex")
OUT_NAMES = ("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit")

# name -> (libtype, n patterns, nBands, seed, overrides)
CASES = {
    "vote_fcc_syn": ("FCC", 300, 9, 100, {}),
    "vote_bcc_syn": ("BCC", 160, 9, 200, {}),
    "vote_hcp_syn": ("HCP", 80, 9, 300, {}),
    "vote_fcc_syn_simpleq": ("FCC", 100, 9, 400, {"simpleqweights": True}),
    "vote_fcc_syn_noearly": ("FCC", 100, 9, 500, {"nband_earlyexit": 100}),
    "vote_fcc_syn12": ("FCC", 60, 12, 600, {}),
    "vote_fcc_syn4": ("FCC", 60, 4, 700, {}),
}


def make_phase(ref, libtype, overrides):
    ph = ref.tripletvote.addphase(libtype=libtype)
    for k, v in overrides.items():
        setattr(ph, k, v)
    return ph


def quat_to_matrix(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def random_quat(rng):
    u1, u2, u3 = rng.random(3)  # Shoemake 1992
    return np.array([np.sqrt(u1) * np.cos(2 * np.pi * u3), np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
                     np.sqrt(1 - u1) * np.cos(2 * np.pi * u2), np.sqrt(u1) * np.sin(2 * np.pi * u3)])


def small_rotation(rng, sigma_deg):
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    a = np.deg2rad(rng.normal() * sigma_deg)
    return quat_to_matrix(np.concatenate(([np.cos(a / 2)], np.sin(a / 2) * axis)))


def synthetic_normals(lib, n, nb, seed):
    rng = np.random.default_rng(seed)
    poles = lib["polesCart"]
    keep = []
    for i in range(poles.shape[0]):
        if all(abs(poles[i] @ poles[k]) < 0.9999 for k in keep):
            keep.append(i)
    keep = np.array(keep)
    norms = np.zeros((n, nb, 3), np.float32)
    inten = np.zeros((n, nb), np.float32)
    for p in range(n):
        if rng.random() < 0.05:  # noise-only pattern
            v = rng.normal(size=(nb, 3))
            norms[p] = v / np.linalg.norm(v, axis=1, keepdims=True)
            inten[p] = np.sort(rng.uniform(0.0, 0.2, nb))[::-1]
            continue
        R = quat_to_matrix(random_quat(rng))
        pick = rng.choice(keep, size=nb, replace=len(keep) < nb)
        for b in range(nb):
            v = small_rotation(rng, 0.4) @ (R @ poles[pick[b]])
            norms[p, b] = v * (1.0 if rng.random() < 0.5 else -1.0)
        inten[p] = np.sort(rng.uniform(0.3, 1.0, nb))[::-1]
        bad = rng.random(nb) < 0.08
        inten[p, bad] = 0.0
        if bad.any():
            v = rng.normal(size=(int(bad.sum()), 3))
            norms[p, bad] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return norms, inten


def run_bandindex(ph, norms, inten):
    """The reference's bandindex with its vote and assignment intermediates recorded."""
    rec = {}
    vote, assign = ph._tripvote_numba, ph._assign_bands_nb2

    def vote_rec(*a):
        out = vote(*a)
        rec["accw"], rec["bandfam"], rec["bandrank"], _, rec["accn"] = out
        return out

    def assign_rec(*a):
        out = assign(*a)
        rec["polevalid"] = out[2]
        return out

    ph._tripvote_numba, ph._assign_bands_nb2 = vote_rec, assign_rec
    try:
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            res = ph.bandindex(norms, band_intensity=inten, band_widths=None)
    finally:
        ph._tripvote_numba, ph._assign_bands_nb2 = vote, assign
    out = {"out_" + k: np.asarray(v) for k, v in zip(OUT_NAMES, res)}
    out.update({"mid_" + k: np.asarray(v) for k, v in rec.items()})
    return out


def _worker(args):
    libtype, overrides, norms, inten = args
    from oracle import refshim
    ref = refshim.load()
    ph = make_phase(ref, libtype, overrides)
    return run_bandindex(ph, norms, inten)


def run_parallel(libtype, overrides, norms, inten, nproc):
    n = norms.shape[0]
    bounds = [(i * n // nproc, (i + 1) * n // nproc) for i in range(nproc)]
    jobs = [(libtype, overrides, norms[a:b], inten[a:b]) for a, b in bounds if b > a]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        parts = pool.map(_worker, jobs)
    return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}


def lib_arrays(ph):
    lib = {"lib_" + k: np.asarray(ph.completelib[k]) for k in LIB_KEYS}
    lib["lib_trip_angles"] = np.asarray(ph.angtriplets["angles"])
    lib["lib_trip_familyid"] = np.asarray(ph.angtriplets["familyid"])
    lib["lib_lut"] = np.asarray(ph.lut)
    lib["lib_nfam"] = np.array(ph.polefamilies.shape[0])
    lib["params"] = np.array(json.dumps({"angTol": float(ph.angTol), "nband_earlyexit": int(ph.nband_earlyexit),
                                         "high_fidelity": bool(ph.high_fidelity),
                                         "simpleqweights": bool(ph.simpleqweights)}))
    return lib


def orient_case(ref, nproc):
    """Band records of orient_80x80.npz -> the indexer's normals and intensities."""
    d = np.load(os.path.join(HERE, "orient_80x80.npz"))
    params = json.loads(str(d["params"]))
    pc = tuple(float(x) for x in d["pc"])
    idx = ref.ebsd_index_single.EBSDIndexer(PC=pc, patDim=(80, 80), **params)
    bd = idx.bandDetectPlan
    from pyebsdindex_gb300 import synthetic as syn
    bd.band_detect_setup(patDim=(80, 80), patternmask=syn.circular_mask(80, 80))
    n, nb = d["ref_theta"].shape
    recs = np.zeros((n, nb), dtype=bd.dataType)
    for f in ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
        recs[f] = d["ref_" + f]
    norms = bd.radonPlan.radon2pole(recs, PC=np.asarray(pc), vendor="EDAX")
    ph = idx.phaseLib[0]
    seen = {}
    real = ph.bandindex

    def capture(bandnorm, band_intensity=None, band_widths=None, verbose=0):
        seen["norms"] = np.array(bandnorm)
        seen["inten"] = np.array(band_intensity)
        return real(bandnorm, band_intensity=band_intensity, band_widths=band_widths, verbose=verbose)

    ph.bandindex = capture
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        indx, _ = idx._indexbandsphase(recs, norms)
    ph.bandindex = real
    assert seen["norms"].shape[0] == n, "every pattern goes to the vote on the first phase"
    out = run_parallel("FCC", {}, seen["norms"].astype(np.float32), seen["inten"].astype(np.float32), nproc)
    case = {"norms": seen["norms"].astype(np.float32), "inten": seen["inten"].astype(np.float32),
            "rec_max": recs["max"], "rec_normmax": recs["normmax"], "rec_theta": recs["theta"],
            "rec_rho": recs["rho"], "rec_valid": recs["valid"], "rhomax": np.asarray(bd.rhoMax),
            "ref_pq": indx["pq"][0], "ref_iq": indx["iq"][0]}
    case.update(out)
    case.update(lib_arrays(ph))
    return case


def main():
    from oracle import refshim
    ref = refshim.load()
    nproc = min(8, os.cpu_count() or 1)
    only = set(sys.argv[1:])
    t0 = time.time()
    if not only or "vote_fcc_orient" in only:
        case = orient_case(ref, nproc)
        np.savez_compressed(os.path.join(HERE, "vote_fcc_orient.npz"), **case)
        print(f"vote_fcc_orient: {case['norms'].shape[0]} patterns, {time.time() - t0:.1f}s, "
              f"nmatch>=3: {int((case['out_nmatch'] >= 3).sum())}")
    for name, (libtype, n, nb, seed, overrides) in CASES.items():
        if only and name not in only:
            continue
        t1 = time.time()
        ph = make_phase(ref, libtype, overrides)
        lib = {k: np.asarray(ph.completelib[k]) for k in LIB_KEYS}
        norms, inten = synthetic_normals(lib, n, nb, seed)
        out = run_parallel(libtype, overrides, norms, inten, nproc)
        case = {"norms": norms, "inten": inten}
        case.update(out)
        case.update(lib_arrays(ph))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **case)
        print(f"{name}: {n} patterns x {nb} bands, {time.time() - t1:.1f}s, "
              f"nmatch>=3: {int((case['out_nmatch'] >= 3).sum())}")


if __name__ == "__main__":
    main()
