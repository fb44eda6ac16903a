"""Agreement of two band-record sets (band-detection accuracy figures).

Two detections of the same patterns -- e.g. the FP32 fused kernel and the FP64 per-stage
method, or this library and the reference's CPU ``find_bands`` -- are compared band by band.
Bands are matched within each pattern by their integer peak location (``maxloc``) rather
than by slot: the reference orders bands with an unstable argsort (band_detect.py:731-735),
so bands of equal height may sit in either slot.  For the matched bands the sub-pixel
location error is max(|aveloc_got - aveloc_ref|) over the two axes, in Radon pixels.

``compare_records`` is vectorised over patterns (an [n, nBands, nBands] location match), so a
few hundred thousand patterns take well under a second.
"""
from __future__ import annotations

import numpy as np

__all__ = ["compare_records", "cubic_misorientation_deg", "orientation_agreement"]

_FIELDS = ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")


def _field(rec, f):
    if isinstance(rec, dict):
        v = rec[f]
    else:
        v = rec[f]
    if type(v).__module__.startswith("torch"):
        v = v.detach().cpu().numpy()
    return np.asarray(v)


def compare_records(got, ref):
    """Match the valid bands of ``got`` to those of ``ref`` and return the agreement figures.

    ``got`` / ``ref``: record arrays of the reference's band dtype, or dicts of per-field
    arrays ([n, nBands] and [n, nBands, 2] for maxloc / aveloc; numpy or torch).  Returns a
    dict: ``bands`` (valid bands of ``ref``), ``matched`` (those with a valid band of ``got``
    at the same integer peak), ``peak_frac`` = matched / bands, ``valid_count_equal`` (fraction
    of patterns with the same number of valid bands), ``aveloc_max`` / ``aveloc_p99`` /
    ``aveloc_p50`` (sub-pixel error of the matched bands, Radon pixels), ``within_1e-3`` (the
    fraction of matched bands within 1e-3 px), ``max_rel`` (largest relative difference of the
    peak height ``max``), ``theta_max`` / ``rho_max`` (largest absolute differences).
    """
    rv = _field(ref, "valid") == 1
    gv = _field(got, "valid") == 1
    n, nb = rv.shape
    rl = np.rint(_field(ref, "maxloc")).astype(np.int64)
    gl = np.rint(_field(got, "maxloc")).astype(np.int64)
    # [n, ref band i, got band j]: same integer peak, both valid
    same = ((rl[:, :, None, 0] == gl[:, None, :, 0]) & (rl[:, :, None, 1] == gl[:, None, :, 1])
            & rv[:, :, None] & gv[:, None, :])
    has = same.any(axis=2)
    j = np.argmax(same, axis=2)
    q, i = np.nonzero(has)
    jj = j[q, i]
    bands = int(rv.sum())
    matched = int(has.sum())
    out = {"bands": bands, "matched": matched, "peak_frac": matched / bands if bands else 1.0,
           "valid_count_equal": float(np.mean(rv.sum(1) == gv.sum(1))) if n else 1.0}
    if matched:
        ra = _field(ref, "aveloc").astype(np.float64)[q, i]
        ga = _field(got, "aveloc").astype(np.float64)[q, jj]
        e = np.abs(ga - ra).max(axis=-1)
        rm = _field(ref, "max").astype(np.float64)[q, i]
        gm = _field(got, "max").astype(np.float64)[q, jj]
        out.update({
            "aveloc_max": float(e.max()), "aveloc_p99": float(np.percentile(e, 99)),
            "aveloc_p50": float(np.median(e)), "within_1e-3": float(np.mean(e <= 1e-3)),
            "max_rel": float((np.abs(gm - rm) / np.maximum(np.abs(rm), 1e-6)).max()),
            "theta_max": float(np.abs(_field(got, "theta").astype(np.float64)[q, jj]
                                      - _field(ref, "theta").astype(np.float64)[q, i]).max()),
            "rho_max": float(np.abs(_field(got, "rho").astype(np.float64)[q, jj]
                                    - _field(ref, "rho").astype(np.float64)[q, i]).max()),
        })
    else:
        out.update({"aveloc_max": 0.0, "aveloc_p99": 0.0, "aveloc_p50": 0.0, "within_1e-3": 1.0,
                    "max_rel": 0.0, "theta_max": 0.0, "rho_max": 0.0})
    return out


def _cubic_rotations():
    """The 24 proper rotations of the cube as unit quaternions (w, x, y, z): the identity, the
    half turns about the three axes, the quarter turns about them (both senses), the half turns
    about the six face diagonals and the third turns about the four body diagonals."""
    h = np.sqrt(0.5)
    q = [(1.0, 0.0, 0.0, 0.0)]
    for a in range(3):
        e = np.zeros(3)
        e[a] = 1.0
        q.append((0.0, *e))                       # half turn
        q.append((h, *(h * e)))                   # quarter turns
        q.append((h, *(-h * e)))
    for a, b in ((0, 1), (0, 2), (1, 2)):
        for s in (1.0, -1.0):
            e = np.zeros(3)
            e[a], e[b] = h, s * h
            q.append((0.0, *e))                   # half turns about face diagonals
    for sx in (1.0, -1.0):
        for sy in (1.0, -1.0):
            for sz in (1.0, -1.0):
                q.append((0.5, 0.5 * sx, 0.5 * sy, 0.5 * sz))  # third turns
    return np.asarray(q, dtype=np.float64)


def _qprod(a, b):
    aw, ax, ay, az = np.moveaxis(a, -1, 0)
    bw, bx, by, bz = np.moveaxis(b, -1, 0)
    return np.stack([aw * bw - ax * bx - ay * by - az * bz, aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx, aw * bz + ax * by - ay * bx + az * bw], axis=-1)


def cubic_misorientation_deg(q1, q2):
    """Smallest rotation angle (degrees) taking orientation q1 to q2 ([n, 4] quaternions) under
    cubic crystal symmetry.  Either frame convention is covered: an equivalent of q is q s or
    s q for a symmetry rotation s, and the rotation angle of a product does not change under
    cyclic permutation, so the candidates are conj(q1) q2 s and q2 conj(q1) s."""
    q1 = np.asarray(q1, dtype=np.float64)
    q2 = np.asarray(q2, dtype=np.float64)
    g = _cubic_rotations()[None]
    c1 = q1 * np.array([1.0, -1.0, -1.0, -1.0])
    wa = np.abs(_qprod(_qprod(c1, q2)[:, None, :], g)[..., 0]).max(-1)
    wb = np.abs(_qprod(_qprod(q2, c1)[:, None, :], g)[..., 0]).max(-1)
    return np.degrees(2.0 * np.arccos(np.clip(np.maximum(wa, wb), -1.0, 1.0)))


def orientation_agreement(q_got, nmatch_got, q_ref, nmatch_ref, tol_deg=0.01):
    """Agreement of two indexings of the same patterns (cubic phase): of the patterns that both
    index (at least three matched bands), the fraction whose orientations differ by at most
    ``tol_deg`` degrees, with the largest and 99th-percentile misorientation."""
    g = np.asarray(nmatch_got) >= 3
    r = np.asarray(nmatch_ref) >= 3
    both = g & r
    out = {"patterns": int(len(g)), "indexed_got": float(g.mean()) if len(g) else 1.0,
           "indexed_ref": float(r.mean()) if len(r) else 1.0, "both_indexed": int(both.sum())}
    if both.any():
        m = cubic_misorientation_deg(np.asarray(q_got)[both], np.asarray(q_ref)[both])
        out.update({"within_tol": float(np.mean(m <= tol_deg)), "tol_deg": tol_deg,
                    "mis_max_deg": float(m.max()), "mis_p99_deg": float(np.percentile(m, 99))})
    return out
