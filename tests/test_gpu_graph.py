"""Launch-side features of the device entry point: capture of ebsd_find_bands in a CUDA graph
(replays must equal direct calls on new data in the same buffers) and the autotuner's
patterns-per-pass choice (records must not depend on it)."""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import _lib
from pyebsdindex_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

FIELDS = ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")


def make_bd(h=80, nRho=120, nBands=9):
    bd = pg.BandDetect(nTheta=180, nRho=nRho, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=nBands)
    bd.band_detect_setup(patDim=(h, h), patternmask=syn.circular_mask(h, h))
    return bd


def dev_outputs(torch, n, nB):
    return {f: torch.full((n, nB, 2) if f in ("maxloc", "aveloc") else (n, nB), -7,
                          dtype=torch.int8 if f == "valid" else torch.float32, device="cuda") for f in FIELDS}


@pytest.mark.parametrize("method", ["fused", "plain"])
def test_find_bands_replays_in_a_cuda_graph(cuda, method):
    import torch
    n = 301
    bd = make_bd()
    plan = bd._device_plan()
    a = syn.make_patterns(n, 80, 80, seed=11, noise_frac=0.1)[0]
    b = syn.make_patterns(n, 80, 80, seed=12, noise_frac=0.1)[0]
    d = torch.from_numpy(a).cuda()
    outs = dev_outputs(torch, n, 9)
    ptrs = {f: v.data_ptr() for f, v in outs.items()}
    plan.reserve(method, n)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # warm-up call outside the capture (sets launch attributes)
        plan.find_bands_device(d.data_ptr(), _lib.EBSD_U8, n, ptrs, method, chunk=n, stream=s.cuda_stream)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.find_bands_device(d.data_ptr(), _lib.EBSD_U8, n, ptrs, method, chunk=n, stream=s.cuda_stream)
    for pats in (b, a):
        d.copy_(torch.from_numpy(pats))
        for v in outs.values():
            v.fill_(-7)
        g.replay()
        torch.cuda.synchronize()
        want = bd.find_bands(pats, method=method)
        for f in FIELDS:
            got = outs[f].cpu().numpy()
            assert got.tobytes() == np.ascontiguousarray(want[f]).tobytes(), f


def test_autotune_choice_does_not_change_records(cuda):
    import torch
    bd = make_bd()
    pats = syn.make_patterns(1200, 80, 80, seed=13, noise_frac=0.1)[0]
    before = bd.find_bands(pats, method="fused")
    ppp = bd.autotune(torch.from_numpy(pats), method="fused")
    assert ppp in (1, 2, 4, 8)
    after = bd.find_bands(pats, method="fused")
    plain = bd.find_bands(pats, method="plain")
    for f in FIELDS:
        assert before[f].tobytes() == after[f].tobytes(), f
        if f != "normmax":
            assert plain[f].tobytes() == after[f].tobytes(), f
    np.testing.assert_allclose(plain["normmax"], after["normmax"], rtol=1e-6)


def test_autotune_decision_cache(cuda, tmp_path, monkeypatch):
    """A decision stored by one plan is applied to an equal plan without timing; records match."""
    import torch
    path = tmp_path / "tuning.json"
    pats = syn.make_patterns(1024, 80, 80, seed=16, noise_frac=0.1)[0]
    bd = make_bd()
    ppp = bd.autotune(torch.from_numpy(pats), method="fused", cache=path)
    assert ppp in (1, 2, 4, 8)
    assert len(__import__("json").loads(path.read_text())["entries"]) == 1
    ref = bd.find_bands(pats, method="fused")
    bd2 = make_bd()
    plan2 = bd2._device_plan()

    def timed(*a, **k):
        raise AssertionError("a cached decision must not be timed again")
    monkeypatch.setattr(plan2, "autotune", timed)
    assert bd2.autotune(torch.from_numpy(pats), method="fused", cache=path) == ppp
    got = bd2.find_bands(pats, method="fused")
    for f in FIELDS:
        assert got[f].tobytes() == ref[f].tobytes(), f
    # another geometry is a new key: timed and added beside the first
    bd3 = make_bd(h=60, nRho=90)
    p3 = bd3.autotune(torch.from_numpy(syn.make_patterns(512, 60, 60, seed=17)[0]), method="fused", cache=path)
    assert p3 in (1, 2, 4, 8)
    assert len(__import__("json").loads(path.read_text())["entries"]) == 2


@pytest.mark.parametrize("dtype", [np.uint16, np.float32])
def test_autotune_single_variant_dtypes(cuda, dtype):
    import torch
    bd = make_bd()
    pats = syn.make_patterns(64, 80, 80, seed=14, noise_frac=0.1)[0].astype(dtype)
    assert bd.autotune(torch.from_numpy(pats), method="fused") == 1
    assert bd.autotune(torch.from_numpy(pats), method="plain") == 1


@pytest.mark.parametrize("h,nRho", [(80, 120), (60, 90)])
def test_patterns_per_pass_variants_give_identical_records(cuda, h, nRho):
    bd = make_bd(h=h, nRho=nRho)
    plan = bd._device_plan()
    pats = syn.make_patterns(203, h, h, seed=15, noise_frac=0.1)[0]
    recs = []
    for ppp in (1, 2, 4, 8, 0):
        plan.set_patterns_per_pass(ppp)
        recs.append(bd.find_bands(pats, method="fused"))
    for r in recs[1:]:
        for f in FIELDS:
            assert r[f].tobytes() == recs[0][f].tobytes(), f
    with pytest.raises(RuntimeError, match="invalid argument"):
        plan.set_patterns_per_pass(3)


@pytest.mark.parametrize("h,nRho", [(80, 120), (60, 90)])
def test_fp16_storage_pass_widths_give_identical_records(cuda, h, nRho):
    """FP16 Radon storage with 2, 4 or 8 uint8 patterns per block pass: the ray sums are exact
    integers, the mean the correctly rounded quotient, and each pattern's centre and scale come
    from its own pixels in the one-pattern pass's order -- so every record equals the
    one-pattern pass's bit for bit."""
    bd = make_bd(h=h, nRho=nRho)
    plan = bd._device_plan()
    assert plan.supported("fused16")
    pats = syn.make_patterns(203, h, h, seed=21, noise_frac=0.1)[0]
    pats[5] = 0  # an all-zero pattern inside a packed unit
    recs = []
    for ppp in (1, 2, 4, 8, 0):
        plan.set_patterns_per_pass(ppp)
        recs.append(bd.find_bands(pats, method="fused16"))
    plan.set_patterns_per_pass(0)
    for r in recs[1:]:
        for f in FIELDS:
            assert r[f].tobytes() == recs[0][f].tobytes(), f


def test_non_separable_kernel_uses_2d_taps_in_both_paths(cuda):
    """A plan whose LoG taps are not rank-1 (here: perturbed off-centre taps) convolves with
    the 2-D taps; fused and per-stage records stay identical, and differ from the separable
    plan's only where the kernel does."""
    bd = make_bd(h=60, nRho=90, nBands=8)
    pats = syn.make_patterns(40, 60, 60, seed=16, noise_frac=0.1)[0]
    sep_fused = bd.find_bands(pats, method="fused")
    k = np.array(bd.kernel, dtype=np.float32, copy=True)
    kk = k.reshape(k.shape[-2:])
    kk[0, 1] *= 1.01  # no longer a product of a rho and a theta profile
    bd.kernel = k
    a = bd.find_bands(pats, method="plain")
    b = bd.find_bands(pats, method="fused")
    for f in ("max", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
        assert a[f].tobytes() == b[f].tobytes(), f
    assert not np.array_equal(a["max"], sep_fused["max"])
