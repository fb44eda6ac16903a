"""The autotuner's decision cache (pyebsdindex_gb300.tuning): keys, JSON round trip, merging
writers, corrupt files.  Host logic only; tests/test_gpu_graph.py applies a cached decision on
the device."""
import json
import os

import numpy as np

from pyebsdindex_gb300 import tuning


def _key(**over):
    kw = dict(gpu="NVIDIA GB300", sms=152, library="1.0", shape=(80, 80), dtype=1, method="fused",
              nTheta=180, nRho=120, nBands=9, kernel_shape=(5, 5), padding=(11, 11), peakPad=(11, 11),
              lut="0123456789abcdef", background=False)
    kw.update(over)
    return tuning.plan_key(**kw)


def test_keys_separate_what_changes_the_choice():
    base = _key()
    for over in (dict(gpu="other"), dict(sms=148), dict(library="1.1"), dict(shape=(60, 60)), dict(dtype=2),
                 dict(method="fused16"), dict(nRho=90), dict(nBands=8), dict(kernel_shape=(9, 9)),
                 dict(padding=(13, 13)), dict(lut="fedcba9876543210"), dict(background=True)):
        assert _key(**over) != base, over
    assert _key() == base


def test_round_trip_and_merge(tmp_path):
    path = tmp_path / "sub" / "tuning.json"
    a, b = tuning.TuningCache(path), tuning.TuningCache(str(path))
    assert a.get(_key()) is None
    a.put(_key(), {"patterns_per_pass": 8, "timed_patterns": 16384})
    b.put(_key(nRho=90), {"patterns_per_pass": 4, "timed_patterns": 100})
    assert a.get(_key())["patterns_per_pass"] == 8
    assert a.get(_key(nRho=90))["patterns_per_pass"] == 4
    doc = json.loads(path.read_text())
    assert doc["format"] == tuning.FORMAT and len(doc["entries"]) == 2
    assert not [f for f in os.listdir(path.parent) if f.startswith(".tuning.")]


def test_corrupt_file_reads_empty_and_is_rewritten(tmp_path):
    path = tmp_path / "tuning.json"
    path.write_text("{not json")
    c = tuning.TuningCache(path)
    assert c.get(_key()) is None
    c.put(_key(), {"patterns_per_pass": 2})
    assert c.get(_key()) == {"patterns_per_pass": 2}


def test_default_path_follows_the_environment(monkeypatch, tmp_path):
    monkeypatch.setenv(tuning.ENV_PATH, str(tmp_path / "x.json"))
    assert tuning.default_path() == str(tmp_path / "x.json")
    monkeypatch.delenv(tuning.ENV_PATH)
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    assert tuning.default_path() == os.path.join(str(tmp_path), "pyebsdindex_gb300", "tuning.json")


def test_lut_digest_sees_one_entry():
    lut = np.arange(120 * 180 * 4, dtype=np.int64).reshape(120, 180, 4)
    d = tuning.lut_digest(lut)
    lut2 = lut.copy()
    lut2[60, 90, 2] += 1
    assert tuning.lut_digest(lut2) != d and tuning.lut_digest(lut.copy()) == d
