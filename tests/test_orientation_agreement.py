"""Downstream parity: orientations indexed from this repository's GPU band records agree with
the orientations the reference indexes from its own records.

Both record sets go through the reference's own triplet voting (EBSDIndexer.index_pats,
_ebsd_index_single.py:466, with the band-detect plan returning the given records), so any
difference comes from the band records alone.  Fixtures: ``tests/golden/orient_80x80.npz``
(patterns, reference records and orientations; make_orientation_golden.py) and
``tests/golden/orient_80x80_gpu.npz`` (the GPU methods' records on those patterns, produced
on a GPU machine by make_gpu_records.py).  Bar: misorientation <= 0.01 degrees on at least
99% of the patterns the reference indexes (nmatch >= 3, bands present).  Needs the reference
source tree (imported through oracle/refshim.py); skipped without it.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FX = os.path.join(HERE, "golden", "orient_80x80.npz")
GPU = os.path.join(HERE, "golden", "orient_80x80_gpu.npz")
FIELDS = ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")


def cubic_group():
    c = np.sqrt(0.5)
    q = [(1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1)]
    for s in (1, -1):
        q += [(c, s * c, 0, 0), (c, 0, s * c, 0), (c, 0, 0, s * c)]
        q += [(0, c, s * c, 0), (0, c, 0, s * c), (0, 0, c, s * c)]
    for sx in (1, -1):
        for sy in (1, -1):
            for sz in (1, -1):
                q.append((0.5, 0.5 * sx, 0.5 * sy, 0.5 * sz))
    g = np.asarray(q, dtype=np.float64)
    assert g.shape == (24, 4)
    return g


def qmul(a, b):
    w1, x1, y1, z1 = np.moveaxis(a, -1, 0)
    w2, x2, y2, z2 = np.moveaxis(b, -1, 0)
    return np.stack([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2], axis=-1)


def misorientation_deg(q1, q2):
    """Smallest rotation angle between q1 and q2 under cubic symmetry, whichever frame the
    quaternions map from: symmetry-equivalents are q*s or s*q, and the angle of a product is
    invariant under cyclic permutation, so the candidates are conj(q1) q2 s and q2 conj(q1) s."""
    g = cubic_group()
    conj = q1 * np.array([1, -1, -1, -1])
    da = qmul(conj, q2)[:, None, :]
    db = qmul(q2, conj)[:, None, :]
    w = np.maximum(np.abs(qmul(da, g[None])[..., 0]).max(-1), np.abs(qmul(db, g[None])[..., 0]).max(-1))
    return np.degrees(2 * np.arccos(np.clip(w, -1.0, 1.0)))


def test_misorientation_helper():
    g = cubic_group()
    rng = np.random.default_rng(3)
    q = rng.normal(size=(20, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    assert misorientation_deg(q, q).max() < 1e-5
    assert misorientation_deg(q, qmul(q, g[rng.integers(0, 24, 20)])).max() < 1e-5
    r = np.array([np.cos(np.radians(0.5)), np.sin(np.radians(0.5)), 0, 0])  # 1 degree about x
    assert abs(misorientation_deg(q[:1], qmul(q[:1], r[None]))[0] - 1.0) < 1e-6


@pytest.fixture(scope="module")
def reference_indexer():
    from oracle import refshim
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    if not os.path.exists(GPU):
        pytest.skip("GPU record fixture not generated")
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_orientation_golden as mog
    ref = refshim.load()
    return mog, ref, mog.make_indexer(ref)


@pytest.mark.parametrize("method", ["fused", "plain", "plain64"])
def test_gpu_records_index_to_reference_orientations(reference_indexer, method):
    mog, ref, idx = reference_indexer
    fx = np.load(FX)
    gpu = np.load(GPU)
    pats = fx["patterns"]
    recs = np.zeros(fx["ref_max"].shape, dtype=idx.bandDetectPlan.dataType)
    for f in FIELDS:
        recs[f] = gpu[method + "_" + f]
    res = mog.index_records(ref, idx, pats, recs)
    sel = (fx["ref_nmatch"] >= 3) & ~fx["noise_only"]
    assert sel.sum() >= 150
    mis = misorientation_deg(fx["ref_quat"][sel], res["quat"][sel])
    frac = float((mis <= 0.01).mean())
    assert frac >= 0.99, (frac, np.sort(mis)[-5:])
