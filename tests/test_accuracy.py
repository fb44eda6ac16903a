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
