"""The vectorised record comparison (pyebsdindex_gb300.accuracy) against the per-pattern loop
of tests/bandcmp.py, on a golden case's records with planted differences."""
import numpy as np

from bandcmp import compare
from conftest import load_golden
from gpuhelp import golden_records
from pyebsdindex_gb300.accuracy import compare_records


def test_compare_records_matches_loop():
    ref = golden_records(load_golden("c1_80_u8"))
    rng = np.random.default_rng(5)
    got = {k: v.copy() for k, v in ref.items()}
    got["aveloc"] = got["aveloc"] + rng.normal(0, 1e-4, got["aveloc"].shape).astype(np.float32)
    got["max"] = got["max"] * np.float32(1 + 1e-6)
    # a moved peak, a dropped band, two bands swapped between slots
    got["maxloc"][0, 0] += 3
    got["valid"][1, 2] = 0
    for f in got:
        got[f][2, [0, 1]] = got[f][2, [1, 0]]
    a = compare_records(got, ref)
    b = compare(got, ref)
    assert a["bands"] == b["bands"] and a["matched"] == b["matched"]
    assert a["matched"] == a["bands"] - 2
    assert abs(a["aveloc_max"] - b["aveloc"]) < 1e-12
    assert abs(a["aveloc_p99"] - b["aveloc_p99"]) < 1e-12
    assert abs(a["valid_count_equal"] - b["valid_count_equal"]) < 1e-12
    assert abs(a["max_rel"] - b["rel"]["max"]) < 1e-12


def test_compare_records_identical_and_empty():
    ref = golden_records(load_golden("c0_60_u8"))
    a = compare_records(ref, ref)
    assert a["peak_frac"] == 1.0 and a["aveloc_max"] == 0.0 and a["within_1e-3"] == 1.0
    none = {k: v[:0] for k, v in ref.items()}
    e = compare_records(none, none)
    assert e["bands"] == 0 and e["peak_frac"] == 1.0


def test_cubic_misorientation_and_orientation_agreement():
    from pyebsdindex_gb300.accuracy import _cubic_rotations, _qprod, cubic_misorientation_deg, orientation_agreement
    g = _cubic_rotations()
    assert g.shape == (24, 4) and np.allclose(np.linalg.norm(g, axis=1), 1.0)
    # a group: every product of two elements is an element (up to sign)
    prod = _qprod(g[:, None, :], g[None, :, :]).reshape(-1, 4)
    assert np.abs(np.abs(prod @ g.T).max(axis=1) - 1.0).max() < 1e-12
    rng = np.random.default_rng(4)
    q = rng.normal(size=(50, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    # symmetry-equivalent orientations (either frame) are 0 apart; a 1 degree turn is 1 degree
    assert cubic_misorientation_deg(q, _qprod(q, g[rng.integers(0, 24, 50)])).max() < 1e-5
    assert cubic_misorientation_deg(q, _qprod(g[rng.integers(0, 24, 50)], q)).max() < 1e-5
    turn = np.array([np.cos(np.radians(0.5)), 0.0, np.sin(np.radians(0.5)), 0.0])
    np.testing.assert_allclose(cubic_misorientation_deg(q[:5], _qprod(q[:5], turn[None])), 1.0, atol=1e-6)
    # agreement: only patterns both sides index (>= 3 matched bands) count
    q2 = q.copy()
    q2[0] = _qprod(q[:1], turn[None])[0]
    nm = np.full(50, 5)
    nm_ref = nm.copy()
    nm_ref[1] = 2
    a = orientation_agreement(q2, nm, q, nm_ref, tol_deg=0.01)
    assert a["both_indexed"] == 49 and abs(a["within_tol"] - 48 / 49) < 1e-12
    assert abs(a["mis_max_deg"] - 1.0) < 1e-6 and a["indexed_ref"] == 49 / 50
