"""Band normals on the device (ebsd_radon2pole) against the host restatement of
Radon.radon2pole (radon_fast.py:314-397; checked against the reference itself in
tests/test_poles_host.py): golden band records, every vendor convention, shared and
per-pattern pattern centres.  Bar: 2e-6 per component (float32; sin/cos are CUDA's, within an
ulp or two of numpy's)."""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import radon_fast
from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

PCS = {"EDAX": [0.46, 0.70, 0.64], "OXFORD": [0.47, 0.69, 0.61], "EMSOFT": [2.5, -3.0, 4100.0, 59.2],
       "KIKUCHIPY": [0.52, 0.28, 0.55], "BRUKER": [0.49, 0.27, 0.58]}


@pytest.mark.parametrize("vendor", sorted(PCS))
@pytest.mark.parametrize("name", ["c1_80_u8", "f32_rect_48x64", "al_sim_20kv"])
def test_device_normals_match_host_restatement(cuda, vendor, name):
    import torch
    case = load_golden(name)
    H, W = case["patterns"].shape[-2:]
    rec = np.zeros(case["out_theta"].shape, dtype=pg.record_dtype())
    rec["theta"] = case["out_theta"]
    rec["rho"] = case["out_rho"]
    rp = radon_fast.Radon()
    rp.imDim = np.array([H, W])
    n = rec.shape[0]
    pcs = np.array(PCS[vendor], dtype=np.float32)
    per = np.tile(pcs, (n, 1)) * (1.0 + 0.01 * np.arange(n, dtype=np.float32))[:, None]
    for pc in (pcs, per):
        want = rp.radon2pole(rec, PC=pc.copy(), vendor=vendor)
        th = torch.from_numpy(np.ascontiguousarray(rec["theta"])).cuda()
        rh = torch.from_numpy(np.ascontiguousarray(rec["rho"])).cuda()
        got = radon_fast.radon2pole_gpu(th, rh, (H, W), PC=pc, vendor=vendor).cpu().numpy()
        np.testing.assert_allclose(got, want, atol=2e-6, rtol=0)


def test_bad_arguments(cuda):
    import torch
    t = torch.zeros((2, 3), device="cuda")
    with pytest.raises(ValueError):
        radon_fast.radon2pole_gpu(t, t, (60, 60), PC=[0.5, 0.5, 0.5], vendor="NOPE")
    with pytest.raises(ValueError):
        radon_fast.radon2pole_gpu(t, t, (60, 60), PC=[0.5, 0.5, 0.5], vendor="EMSOFT")


def test_find_bands_normals_equals_host_path(cuda):
    from pyebsdindex_gb300 import synthetic as syn
    bd = pg.BandDetect(nTheta=180, nRho=90, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=8)
    bd.band_detect_setup(patDim=(60, 60), patternmask=syn.circular_mask(60, 60))
    pats = syn.make_patterns(24, 60, 60, seed=17, noise_frac=0.1)[0]
    recs, normals = bd.find_bands_normals(pats, PC=[0.46, 0.70, 0.64], vendor="EDAX")
    ref = bd.find_bands(pats)
    for f in ("max", "maxloc", "aveloc", "theta", "rho", "valid"):
        assert recs[f].tobytes() == ref[f].tobytes(), f
    want = bd.radonPlan.radon2pole(ref, PC=np.array([0.46, 0.70, 0.64], np.float32), vendor="EDAX")
    np.testing.assert_allclose(normals, want, atol=2e-6, rtol=0)
