"""Band-set comparison used by the parity tests.

Bands are matched per pattern by their integer peak location (``maxloc``): the reference
orders bands with an unstable argsort (band_detect.py:734), so exact ties may come out in a
different slot order while describing the same bands.
"""
import numpy as np

FLOAT_FIELDS = ("max", "normmax", "avemax", "width", "theta", "rho")


def as_dict(rec):
    if isinstance(rec, dict):
        return rec
    return {f: rec[f] for f in rec.dtype.names}


def compare(got, ref, skip=()):
    """Match bands of ``got`` to ``ref``; patterns listed in ``skip`` are left out."""
    got, ref = as_dict(got), as_dict(ref)
    n, nB = ref["valid"].shape
    skip = set(int(s) for s in skip)
    total = matched = 0
    valid_count_equal = 0
    err = {f: 0.0 for f in FLOAT_FIELDS}
    rel = {f: 0.0 for f in ("max", "normmax", "avemax", "width")}
    loc_err = 0.0
    errs = []
    for q in range(n):
        if q in skip:
            continue
        rv = np.nonzero(ref["valid"][q] == 1)[0]
        gv = np.nonzero(got["valid"][q] == 1)[0]
        valid_count_equal += int(len(rv) == len(gv))
        gmap = {tuple(np.round(got["maxloc"][q, j]).astype(int)): j for j in gv}
        for i in rv:
            total += 1
            key = tuple(np.round(ref["maxloc"][q, i]).astype(int))
            j = gmap.get(key)
            if j is None:
                continue
            matched += 1
            e = float(np.abs(got["aveloc"][q, j].astype(np.float64) - ref["aveloc"][q, i].astype(np.float64)).max())
            errs.append(e)
            loc_err = max(loc_err, e)
            for f in FLOAT_FIELDS:
                d = abs(float(got[f][q, j]) - float(ref[f][q, i]))
                err[f] = max(err[f], d)
                if f in rel:
                    rel[f] = max(rel[f], d / max(abs(float(ref[f][q, i])), 1e-6))
    return {
        "bands": total,
        "matched": matched,
        "frac": matched / total if total else 1.0,
        "valid_count_equal": valid_count_equal / max(n, 1),
        "aveloc": loc_err,
        "aveloc_p50": float(np.median(errs)) if errs else 0.0,
        "aveloc_p99": float(np.percentile(errs, 99)) if errs else 0.0,
        "within_1e-3": float(np.mean(np.asarray(errs) <= 1e-3)) if errs else 1.0,
        "abs": err,
        "rel": rel,
    }


def exact_equal_fields(got, ref, fields):
    got, ref = as_dict(got), as_dict(ref)
    return {f: bool(np.array_equal(np.asarray(got[f]), np.asarray(ref[f]))) for f in fields}
