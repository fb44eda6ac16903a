"""The pattern-file readers (pyebsdindex_gb300/ebsd_pattern.py over libebsdgpu) on files the
reference's own writers wrote, against what the reference's own readers returned for them
(tests/golden/patfiles/, made by tests/golden/make_pattern_file_golden.py): header attributes
with their types, every pattern and position, and a slab.  Needs no reference tree."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR

PATDIR = os.path.join(GOLDEN_DIR, "patfiles")
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(PATDIR, "*.npz")))
SLAB = [[1, 1], [2, 2]]


def test_fixtures_present():
    assert {"ebsp_v2_xy", "ebsp_v4_noxy", "tfpat_bg12", "up2_v3"} <= set(CASES)


@pytest.mark.parametrize("name", CASES)
def test_reader_matches_reference_fixture(name, built_lib):
    from pyebsdindex_gb300 import ebsd_pattern as ep
    g = np.load(os.path.join(PATDIR, name + ".npz"))
    path = [p for p in glob.glob(os.path.join(PATDIR, name + ".*")) if not p.endswith(".npz")][0]
    f = ep.get_pattern_file_obj(path)
    for key in g.files:
        if not key.startswith("attr_"):
            continue
        a = key[5:]
        want = g[key]
        got = getattr(f, a)
        if a == "filedatatype":
            assert np.dtype(got).name == str(want), a
            continue
        assert np.all(np.asarray(got) == want), (a, got, want)
        assert np.asarray(got).dtype == want.dtype, (a, np.asarray(got).dtype, want.dtype)
    allp, allxy = f.read_data(patStartCount=[0, -1], returnArrayOnly=True)
    slab, slabxy = f.read_data(patStartCount=SLAB, returnArrayOnly=True)
    for got, key in ((allp, "patterns"), (allxy, "xy"), (slab, "slab"), (slabxy, "slab_xy")):
        assert got.dtype == g[key].dtype and got.shape == g[key].shape, key
        assert got.tobytes() == g[key].tobytes(), key
