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

__all__ = ["compare_records"]

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
