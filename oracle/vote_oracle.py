"""CPU restatement of the reference's triplet voting (the oracle for the device band indexer).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import this module, and only as the checker.  The product package
never imports it.

Follows PyEBSDIndex v0.3.10.1 ``tripletvote.BandIndexer.bandindex`` (tripletvote.py:492-633)
step by step with the same numpy operations and dtypes, so that on the machine that made the
golden vectors it reproduces the reference's own outputs:

* ``band_intensity``  -- the indexer's band weights and pq / iq (_ebsd_index_single.py:751-763)
* ``tripvote``        -- ``_tripvote_numba`` (tripletvote.py:1021-1210)
* ``assign_bands``    -- ``_assign_bands_nb2`` (tripletvote.py:1483-1690)
* ``quest_weights``   -- ``_calc_quest_weights`` (tripletvote.py:856-901)
* ``refine_quest``    -- ``_refine_orientation_quest`` + ``_orientation_quest_nb``
                         (tripletvote.py:903-1020), with ``rotlib.quat_vectorL1N`` (rotlib.py:1641-1674)
* ``calc_cm``         -- ``_calc_cm`` (tripletvote.py:2057-2075)

Arithmetic follows the reference source as numpy evaluates it (NEP 50: a Python float meeting
a float32 value stays float32).  One rule is fixed where the reference leaves it to the
platform: ``bandindex`` ranks bands with ``np.argsort`` (tripletvote.py:529), whose order for
equal ranks depends on numpy's SIMD sort; here equal ranks keep band order (a stable sort),
as numba's small-array sort inside the jitted functions does.
"""
from __future__ import annotations

import numpy as np

RADEG = 180.0 / np.pi
F32 = np.float32


def band_intensity(mx, normmax, theta, rho, valid, rhomax):
    """Band weights for the vote and the pattern-quality numbers, _ebsd_index_single.py:751-763."""
    mx = np.asarray(mx, F32)
    theta = np.asarray(theta, F32)
    rho = np.asarray(rho, F32)
    rhomax = F32(rhomax)
    adj = (-1 * np.abs(rho) * 0.5 / rhomax + 1) * mx
    adj *= ((theta > (2 * np.pi / 180)).astype(F32) + 0.5) / 2
    adj *= ((theta < (178.0 * np.pi / 180)).astype(F32) + 0.5) / 2
    adj *= valid
    pq = np.mean(mx * valid, axis=1)
    iq = np.mean(np.asarray(normmax, F32) * valid, axis=1)
    return adj, pq, iq


def _argsort3(v):
    """The hard-coded three-element argsort of tripletvote.py:1035-1041."""
    s = [0, 1, 2]
    if v[s[0]] > v[s[2]]:
        s[2], s[0] = s[0], s[2]
    if v[s[0]] > v[s[1]]:
        s[1], s[0] = s[0], s[1]
    if v[s[1]] > v[s[2]]:
        s[2], s[1] = s[1], s[2]
    return s


def tripvote(bandnorms, band_intensity, lut, angTol, tripAngles, tripID, nfam):
    """Triplet vote, tripletvote.py:1021-1210.  Returns (accumulatorW, bandFam, bandRank,
    band_cm, accumulator) with the reference's dtypes."""
    npats, nb = bandnorms.shape[:2]
    tripAngles = np.asarray(tripAngles)
    tripID = np.asarray(tripID)
    lut = np.asarray(lut)
    accW = np.zeros((npats, nfam, nb), F32)
    accN = np.zeros((npats, nfam, nb), F32)
    band_cm = np.zeros((npats, nb), F32)
    bandRank = np.zeros((npats, nb), F32)
    bandFam = np.zeros((npats, nb), np.int32)
    for p in range(npats):
        bn = bandnorms[p]
        bandangs = np.abs(bn.dot(bn.T))
        bandangs = np.clip(bandangs, -1.0, 1.0)
        bandangs = np.arccos(bandangs) * RADEG
        for q in range(nb):
            if band_intensity[p, q] < 1e-6:
                bandangs[q, :] = 10000.0
                bandangs[:, q] = 10000.0
        aW = accW[p]
        aN = accN[p]
        for i in range(nb):
            for j in range(i + 1, nb):
                for k in range(j + 1, nb):
                    angtri = np.array([bandangs[i, j], bandangs[i, k], bandangs[j, k]], dtype=F32)
                    srt = _argsort3(angtri)
                    srt2 = lut[:, srt[0], srt[1], srt[2]]
                    unsrt = _argsort3(srt2)
                    a = angtri[srt]
                    t1 = np.abs(tripAngles[:, 0] - a[0])
                    t2 = np.abs(tripAngles[:, 1] - a[1])
                    t3 = np.abs(tripAngles[:, 2] - a[2])
                    hits = np.nonzero((t1 <= angTol) & (t2 <= angTol) & (t3 <= angTol))[0]
                    for qq in hits:
                        at0, at1, at2 = F32(t1[qq]), F32(t2[qq]), F32(t3[qq])
                        f = tripID[qq, :][unsrt]
                        w1 = angTol - 0.5 * (at0 + at1)
                        w2 = angTol - 0.5 * (at0 + at2)
                        w3 = angTol - 0.5 * (at1 + at2)
                        adds = [(f[0], i, w1), (f[1], j, w2), (f[2], k, w3)]
                        e1 = np.abs(a[0] - a[1]) < angTol
                        e2 = np.abs(a[1] - a[2]) < angTol
                        e3 = np.abs(a[2] - a[0]) < angTol
                        if e1:
                            adds += [(f[0], j, w1), (f[1], i, w2), (f[2], k, w3)]
                        if e2:
                            adds += [(f[0], i, w1), (f[1], k, w2), (f[2], j, w3)]
                        if e3:
                            adds += [(f[0], k, w1), (f[1], j, w2), (f[2], i, w3)]
                        if e1 and e2 and e3:
                            adds += [(f[0], k, w1), (f[1], i, w2), (f[2], j, w3),
                                     (f[0], j, w1), (f[1], k, w2), (f[2], i, w3)]
                        # the reference adds all weights of a step before the counts; the two
                        # accumulators are independent, so the order within a step is the same
                        for fam, band, w in adds:
                            aW[fam, band] += w
                            aN[fam, band] += 1
        # __trivotemetriccalc, tripletvote.py:1137-1171
        mxvote = np.zeros(nb, np.int32)
        tvotes = np.zeros(nb, np.int32)
        cm = np.zeros(nb, F32)
        fam = np.zeros(nb, np.int32)
        for b in range(nb):
            col = aW[:, b].flatten()
            mxval = F32(-1.0e12)
            sumval = F32(0.0)
            for v in col:
                sumval += v
                if v > mxval:
                    mxval = v
            mxvote[b] = mxval
            tvotes[b] = sumval
            if tvotes[b] < 1:
                cm[b] = 0.0
            else:
                s = np.sort(col)
                cm[b] = (s[-1] - s[-2]) / tvotes[b]
            mxval = F32(-1.0e12)
            for qq in range(col.size):
                if col[qq] > mxval:
                    mxval = col[qq]
                    fam[b] = qq
        bandRank[p, :] = (nb - np.arange(nb)) / nb * cm * mxvote
        bandFam[p, :] = fam
        band_cm[p, :] = cm
    return accW, bandFam, bandRank, band_cm, accN


def _triad_fit(ii, jj, nb, bn, rank_arg, fam, pflt, angTable, famIndex, nFamily, angTol, bndnorm):
    """One band pair of the TRIAD assignment, tripletvote.py:1487-1585."""
    eps = F32(1.0e-12)
    R = np.zeros((3, 3), F32)
    angFit = np.zeros(nb, F32)
    polematch = np.full(nb, -1, np.int64)
    polevalid = np.zeros(nb, np.uint8)
    whGood = np.zeros(nb, np.int64)
    nGood = 0
    bnd1 = rank_arg[-1 - ii]
    bnd2 = rank_arg[-1 - jj]
    v1 = bn[bnd1, :]
    f1 = fam[bnd1]
    v2 = bn[bnd2, :]
    f2 = fam[bnd2]
    ang01 = np.dot(v1, v2)
    if ang01 > F32(1.0):
        ang01 = F32(1.0 - eps)
    if ang01 < F32(-1.0):
        ang01 = F32(-1.0 + eps)
    paralleltest = np.arccos(np.fabs(ang01)) * RADEG
    if paralleltest > angTol:
        ang01 = np.arccos(ang01) * RADEG
        lo = int(famIndex[f2])
        wh12 = np.nonzero(np.abs(angTable[famIndex[f1], lo:lo + int(nFamily[f2])] - ang01) < angTol)[0]
        if wh12.size > 0:
            wh12 = wh12 + lo
            p1 = pflt[famIndex[f1], :]
            v1v2c = np.cross(v1, v2)
            v1v2c /= np.linalg.norm(v1v2c)
            A = np.zeros((3, 3), F32)
            B = np.zeros((3, 3), F32)
            b2 = np.cross(v1, v1v2c)
            B[0, :] = v1
            B[1, :] = v1v2c
            B[2, :] = b2
            A[:, 0] = p1
            score = -1.0
            for i in range(wh12.size):
                p2 = pflt[wh12[i], :]
                p2 = p2 / (np.linalg.norm(p2) + 1.0e-35)
                p1p2c = np.cross(p1, p2)
                p1p2c = p1p2c / (np.linalg.norm(p1p2c) + 1.0e-35)
                A[:, 1] = p1p2c
                A[:, 2] = np.cross(p1, p1p2c)
                AB = A.dot(B)
                test = pflt.dot(AB.dot(bndnorm))
                fitTry = np.zeros(nb, F32)
                for j in range(nb):
                    fitTry[j] = np.max(test[:, j])
                    fitTry[j] = -1.0 if fitTry[j] < -1.0 else fitTry[j]
                    fitTry[j] = 1.0 if fitTry[j] > 1.0 else fitTry[j]
                fitTry = np.arccos(fitTry) * RADEG
                wm = np.nonzero(fitTry < angTol)[0]
                with np.errstate(all="ignore"):
                    scoreTry = F32(wm.size) / (np.mean(fitTry[wm]) + 1e-6)
                if scoreTry > score:
                    score = scoreTry
                    angFit[:] = fitTry
                    for j in range(nb):
                        polematch[j] = np.argmax(test[:, j])
                        polevalid[j] = np.uint8(fitTry[j] < angTol)
                    R[:, :] = AB
            whGood = np.nonzero(angFit < angTol)[0].astype(np.int64)
            nGood = whGood.size
    return whGood, nGood, angFit, polematch, polevalid, R, bnd1, bnd2


def assign_bands(polesCart, angTable, famIndex, nFamily, angTol, n_band_early, bandnorms, rank_arg, bandFam):
    """TRIAD band assignment over band pairs in rank order, tripletvote.py:1483-1690.
    Returns (fit, polematch, polevalid, nMatch, whGood, ij, R, fitb)."""
    pflt = np.asarray(polesCart, F32)
    npats, nb = bandnorms.shape[:2]
    whGood_out = np.zeros((npats, nb), np.int64) - 1
    Rout = np.zeros((npats, 3, 3), F32)
    Rout[:, 0, 0] = Rout[:, 1, 1] = Rout[:, 2, 2] = 1.0
    pm_out = np.full((npats, nb), -1000, np.int64)
    pv_out = np.zeros((npats, nb), np.uint8)
    fit_out = np.full(npats, 360.0, F32)
    fitb_out = np.full((npats, nb), 360.0, F32)
    nMatch = np.zeros(npats, np.int64)
    ij = np.full((npats, 4), -1, np.int64)
    for p in range(npats):
        bn = bandnorms[p]
        bndnorm = np.transpose(np.asarray(bn, F32))
        best_fit = F32(360.0)
        best_n = 0
        done = False
        for ii in range(nb - 1):
            for jj in range(ii + 1, nb):
                wg, ng, af, pm, pv, R, b1, b2 = _triad_fit(ii, jj, nb, bn, rank_arg[p], bandFam[p], pflt,
                                                           angTable, famIndex, nFamily, angTol, bndnorm)
                if ng >= 3:
                    fit = F32(0.0)
                    for q in range(ng):
                        fit += F32(af[wg[q]])
                    fit /= F32(ng)
                    if best_n < ng or (best_n == ng and best_fit > fit):
                        best_fit, best_n = F32(fit), ng
                        fitb_out[p] = af
                        whGood_out[p, :ng] = wg
                        pm_out[p] = pm
                        pv_out[p] = pv
                        Rout[p] = R
                        ij[p] = (ii, jj, b1, b2)
                if best_n >= n_band_early:
                    done = True
                    break
            if done:
                break
        fit_out[p] = best_fit
        nMatch[p] = best_n
    return fit_out, pm_out, pv_out, nMatch, whGood_out, ij, Rout, fitb_out


def quest_weights(libFamID, accumulator, accumulator_nw, polematch, polevalid, band_intensity, nfit=6,
                  simpleqweights=True):
    """Band weights for the QUEST fit, tripletvote.py:856-901 (including the simple-weights
    branch's use of the loop counter as the band index, :883)."""
    npats, nb = polematch.shape
    weights = np.zeros((npats, nb), F32)
    for p in range(npats):
        w = np.zeros(nb)
        score = np.full(nb, -1.0, F32)
        pmatch = polematch[p].astype(np.int64)
        whGood = np.nonzero(polevalid[p] > 0)[0]
        if whGood.size < 3:
            continue
        if not simpleqweights:
            for q in range(whGood.size):
                g = whGood[q]
                a = libFamID[pmatch[g]]
                score[g] = accumulator[p, a, g]
                score[g] /= max(accumulator_nw[p, a, g], 1.0e-12)
        else:
            for q in range(whGood.size):
                score[whGood[q]] = band_intensity[p, q]
        srt = np.flip(np.argsort(score, kind="stable"))
        for s in srt[0:min(nfit, whGood.size)]:
            w[s] = band_intensity[p, s]
        w /= np.sum(w)
        weights[p, :] = w
    return weights


def quat_vector_l1n(q, v):
    """Rotate rows of ``v`` by quaternion ``q`` (passive, p = 1), rotlib.py:1641-1674."""
    w = q[0]
    r = q[1:4]
    out = np.zeros_like(v)
    for i in range(v.shape[0]):
        t = np.array([r[1] * v[i, 2] - r[2] * v[i, 1], r[2] * v[i, 0] - r[0] * v[i, 2],
                      r[0] * v[i, 1] - r[1] * v[i, 0]])
        t = t + w * v[i]
        t2 = np.array([r[1] * t[2] - r[2] * t[1], r[2] * t[0] - r[0] * t[2], r[0] * t[1] - r[1] * t[0]])
        out[i] = 2.0 * t2 + v[i]
    return out


def refine_quest(polesCart, bandnorms, polematch, polevalid, weights):
    """Weighted QUEST orientation fit, tripletvote.py:903-1020.  Returns (quat, fit_unweight,
    bdot_unweight) in float64."""
    npats, nb = bandnorms.shape[:2]
    wts = np.asarray(weights, np.float64)
    wts /= np.maximum(np.sum(wts, axis=1), 1e-12).reshape(-1, 1)
    pfl = np.asarray(polesCart[polematch.clip(0), :], np.float64)
    bnd = np.asarray(bandnorms, np.float64)
    qout = np.zeros((npats, 4))
    qout[:, 0] = 1.0
    fitout = np.full(npats, np.pi)
    mad = np.full(npats, -1.0)
    bdot = np.full((npats, nb), -1.0)
    I3 = np.identity(3)
    for p in range(npats):
        wp = wts[p]
        good = np.nonzero(wp > 1.0e-7)[0]
        if good.size < 3:
            continue
        wn = wp[good].reshape(-1, 1).copy()
        bn = bnd[p][good]
        pf = pfl[p][good]
        wn /= np.sum(wn)
        B = (wn * bn).T @ pf
        S = B + B.T
        z = np.asarray(np.sum(wn * np.cross(bn, pf), axis=0), np.float64)
        S2 = S @ S
        det = np.linalg.det(S)
        k = (S[1, 1] * S[2, 2] - S[1, 2] * S[2, 1]) + (S[0, 0] * S[2, 2] - S[0, 2] * S[2, 0]) + (
            S[0, 0] * S[1, 1] - S[1, 0] * S[0, 1])
        sig = 0.5 * (S[0, 0] + S[1, 1] + S[2, 2])
        sig2 = sig * sig
        d = z.T @ S2 @ z
        c = det + (z.T @ S @ z)
        b = sig2 + (z.T @ z)
        a = sig2 - k
        lam, it, dlam = 1.0, 0, 1e6
        while dlam > 1.0e-12 and it < 10:
            lam0 = lam
            lam = lam - (lam ** 4 - (a + b) * lam ** 2 - c * lam + (a * b + c * sig - d)) / (
                4 * lam ** 3 - 2 * (a + b) * lam - c)
            dlam = np.fabs(lam0 - lam)
            it += 1
        beta = lam - sig
        alpha = lam ** 2 - sig2 + k
        gamma = (lam + sig) * alpha - det
        X = (alpha * I3 + beta * S + S2) @ z
        qn = np.sqrt(gamma ** 2 + X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
        q = np.array([gamma, X[0], X[1], X[2]]) / qn
        if np.sign(gamma) < 0:
            q *= -1.0
        qout[p] = q
        fitout[p] = lam
        rot = quat_vector_l1n(q, bn)
        bd = np.sum(rot * pf, axis=1, dtype=np.float64)
        bdot[p, good] = bd
        mad[p] = np.mean(bd)
    return qout, mad, bdot


def calc_cm(accumulator, polematch, polevalid, libFamID):
    """Vote confidence of the matched bands, tripletvote.py:2057-2075."""
    npats = accumulator.shape[0]
    cm2 = -1 * np.ones(npats, F32)
    for p in range(npats):
        wm = np.nonzero(polevalid[p] > 0)[0]
        if wm.size < 3:
            continue
        cm2[p] = 0.0
        for m in wm:
            cm2[p] += F32(accumulator[p, libFamID[polematch[p, m]], m])
        cm2[p] /= np.sum(accumulator[p].clip(1))
    return cm2


def bandindex(lib, params, bandnorms, band_intensity=None):
    """``BandIndexer.bandindex`` (tripletvote.py:492-633) with ``high_fidelity`` on.

    ``lib``: dict with ``trip_angles``, ``trip_familyid``, ``lut``, ``nfam`` and the complete
    library ``polesCart``, ``familyid``, ``angTable``, ``nFamily``, ``famIndex``.  ``params``:
    ``angTol``, ``nband_earlyexit``, ``simpleqweights``.  Returns (quat, fit, cm, polematch,
    nMatch, ij, acc_correct, bandfit) and a dict of intermediates."""
    bn = np.asarray(bandnorms)
    if bn.ndim == 2:
        bn = bn[np.newaxis]
    npats, nb = bn.shape[:2]
    if band_intensity is None:
        band_intensity = np.ones((npats, nb))
    inten = np.asarray(band_intensity)
    if inten.ndim == 1:
        inten = inten[np.newaxis]
    angTol = float(params["angTol"])
    accW, bandFam, bandRank, band_cm, accN = tripvote(bn, inten, lib["lut"], angTol, lib["trip_angles"],
                                                      lib["trip_familyid"], int(lib["nfam"]))
    rank_arg = np.argsort(bandRank, axis=1, kind="stable").astype(np.int64)
    famID = np.asarray(lib["familyid"])
    fit, pm, pv, nMatch, whGood, ij, R, fitb = assign_bands(
        lib["polesCart"], np.asarray(lib["angTable"]), np.asarray(lib["famIndex"]), np.asarray(lib["nFamily"]),
        angTol, np.int64(params["nband_earlyexit"]), bn, rank_arg, bandFam)
    acc_correct = np.sum(np.array((pv > 0) & (famID[pm.clip(0)] == bandFam), dtype=int), axis=1).astype(np.int32)
    w = quest_weights(famID, accW, accN, pm, pv, inten, nfit=6, simpleqweights=bool(params["simpleqweights"]))
    quat, fitu, bdot = refine_quest(np.asarray(lib["polesCart"]), bn, pm, pv, w)
    bandfit = np.arccos(np.clip(bdot, -1.0, 1.0)) * RADEG
    fit = np.arccos(np.clip(fitu, -1.0, 1.0)) * RADEG
    cm2 = calc_cm(accW, pm, pv, famID)
    mid = {"accw": accW, "accn": accN, "bandfam": bandFam, "bandrank": bandRank, "polevalid": pv,
           "rank_arg": rank_arg, "weights": w}
    return (quat, fit, cm2, pm, nMatch, ij, acc_correct, bandfit), mid


def load_case(path):
    """A ``tests/golden/vote_*.npz`` case -> (lib, params, inputs dict, reference outputs dict)."""
    import json
    d = np.load(path)
    lib = {k[4:]: d[k] for k in d.files if k.startswith("lib_")}
    params = json.loads(str(d["params"]))
    ins = {k: d[k] for k in d.files if not k.startswith(("lib_", "out_", "mid_")) and k != "params"}
    outs = {k: d[k] for k in d.files if k.startswith(("out_", "mid_"))}
    return lib, params, ins, outs
