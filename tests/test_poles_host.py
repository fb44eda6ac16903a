"""The host restatement of Radon.radon2pole (pyebsdindex_gb300.radon_fast) against the
reference's own radon2pole (radon_fast.py:314-397, imported through oracle/refshim.py) on the
golden band records, for every vendor convention; identical float32 arithmetic, so equal to
the last bit.  Skipped without the reference source tree."""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import radon_fast
from conftest import load_golden

PCS = {"EDAX": [0.46, 0.70, 0.64], "OXFORD": [0.47, 0.69, 0.61], "EMSOFT": [2.5, -3.0, 4100.0, 59.2],
       "KIKUCHIPY": [0.52, 0.28, 0.55], "BRUKER": [0.49, 0.27, 0.58]}


@pytest.fixture(scope="module")
def ref():
    from oracle import refshim
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    return refshim.load()


@pytest.mark.parametrize("vendor", sorted(PCS))
@pytest.mark.parametrize("name", ["c1_80_u8", "f32_rect_48x64"])
def test_host_radon2pole_equals_reference(ref, vendor, name):
    case = load_golden(name)
    H, W = case["patterns"].shape[-2:]
    rec = np.zeros(case["out_theta"].shape, dtype=pg.record_dtype())
    rec["theta"] = case["out_theta"]
    rec["rho"] = case["out_rho"]
    mine = radon_fast.Radon()
    mine.imDim = np.array([H, W])
    theirs = ref.radon_fast.Radon()
    theirs.imDim = np.array([H, W])
    pc = np.array(PCS[vendor], dtype=np.float32)
    a = mine.radon2pole(rec, PC=pc.copy(), vendor=vendor)
    b = theirs.radon2pole(rec, PC=pc.copy(), vendor=vendor)
    assert a.tobytes() == b.tobytes()
