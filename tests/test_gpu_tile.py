"""Radon tile shapes: the whole padded Radon image as one on-chip tile (k_fused) or theta slabs
of several widths (k_slab), chosen by the autotuner or pinned with ``set_tile``.

Every shape gives the per-stage FP32 method's records bit for bit on integer patterns (the
same exact ray sums, correctly rounded means, LoG multiply-add order, peak order and fit),
except normmax, whose per-pattern mean the kernels reduce in different orders (last bit).  So
the autotuner's choice never changes a record, and a decision cached for one plan applies to
an equal plan.
"""
import json

import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import synthetic as syn
from pyebsdindex_gb300.band_detect import MixedBandDetect

pytestmark = pytest.mark.gpu

FIELDS = ("max", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")


def plan(h, nrho, nbands=10):
    bd = pg.BandDetect(nTheta=180, nRho=nrho, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=nbands)
    bd.band_detect_setup(patDim=(h, h), patternmask=syn.circular_mask(h, h))
    return bd


def patterns(n, h, seed):
    return syn.make_patterns(n, h, h, seed=seed, dtype=np.uint16, peak=4000.0, noise_frac=0.1)[0]


def as_u16_tensor(pats):
    import torch
    if not hasattr(torch, "uint16"):
        pytest.skip("torch without uint16")
    return torch.from_numpy(np.ascontiguousarray(pats).view(np.int16)).view(torch.uint16)


def same(a, b, with_normmax=False):
    for f in FIELDS:
        assert a[f].tobytes() == b[f].tobytes(), f
    if with_normmax:
        assert a["normmax"].tobytes() == b["normmax"].tobytes()
    else:
        np.testing.assert_allclose(a["normmax"], b["normmax"], rtol=1e-6)


@pytest.mark.parametrize("h", [60, 120])
def test_every_tile_shape_gives_the_per_stage_records(cuda, h):
    bd = plan(h, int(1.5 * h))
    dp = bd._device_plan()
    info = dp.get_tile()
    assert info["slabs"] >= 1 and info["slabs_min"] <= info["slabs_max"]
    assert info["single_fits"] == (1 if h == 60 else 0)
    pats = patterns(150, h, 40 + h)
    ref = bd.find_bands(pats, method="plain")
    shapes = [(2, ns) for ns in range(info["slabs_min"], min(info["slabs_max"], info["slabs_min"] + 3) + 1)]
    if info["single_fits"]:
        shapes.insert(0, (1, 0))
    for tile, ns in shapes:
        dp.set_tile(tile, ns)
        got = dp.get_tile()
        assert got["tile"] == tile, (tile, ns, got)
        if tile == 2:
            assert got["slabs"] == ns and got["slab_columns"] == (180 + ns - 1) // ns
        same(bd.find_bands(pats, method="fused"), ref)
    dp.set_tile(0, 0)
    assert dp.get_tile()["tile"] == (1 if info["single_fits"] else 2)
    assert dp.get_tile()["slabs"] == info["slabs_min"]


def test_set_tile_rejects_shapes_the_plan_cannot_take(cuda):
    bd = plan(120, 180)
    dp = bd._device_plan()
    info = dp.get_tile()
    with pytest.raises(RuntimeError, match="not supported by this method"):
        dp.set_tile(1, 0)  # the single tile does not fit a 120x120 plan
    with pytest.raises(RuntimeError, match="not supported by this method"):
        dp.set_tile(2, info["slabs_max"] + 1)
    with pytest.raises(RuntimeError, match="not supported by this method"):
        dp.set_tile(2, info["slabs_min"] - 1 if info["slabs_min"] > 1 else 181)
    with pytest.raises(RuntimeError, match="invalid argument"):
        dp.set_tile(3, 0)
    assert dp.get_tile() == info  # a refused call leaves the plan as it was


@pytest.mark.parametrize("h", [60, 120])
def test_autotune_picks_a_tile_shape_and_keeps_the_records(cuda, h):
    import torch
    bd = plan(h, int(1.5 * h))
    pats = patterns(600, h, 70 + h)
    ref = bd.find_bands(pats, method="plain")
    ppp = bd.autotune(as_u16_tensor(pats), method="fused")
    assert ppp == 1  # uint16 input: one pattern per pass in either kernel
    t = bd.tuned
    assert t["tile"] in (1, 2) and not t["cached"]
    if t["tile"] == 2:
        assert t["slabs_min"] <= t["slabs"] <= t["slabs_max"]
    print(h, "autotuned tile:", t)
    same(bd.find_bands(pats, method="fused"), ref)


def test_tile_decision_cache_round_trip(cuda, tmp_path, monkeypatch):
    """The cached decision holds the tile shape; an equal plan gets it without timing."""
    import torch
    path = tmp_path / "tuning.json"
    pats = patterns(400, 120, 91)
    bd = plan(120, 180)
    bd.autotune(as_u16_tensor(pats), method="fused", cache=path)
    entry = next(iter(json.loads(path.read_text())["entries"].values()))
    assert entry["tile"] == 2 and entry["slabs"] == bd.tuned["slabs"]
    # store a narrower slab count than the widest and check that an equal plan applies it
    narrower = bd.tuned["slabs_min"] + 1
    key = next(iter(json.loads(path.read_text())["entries"]))
    from pyebsdindex_gb300 import tuning
    tuning.TuningCache(path).put(key, dict(entry, slabs=narrower))
    bd2 = plan(120, 180)
    dp2 = bd2._device_plan()

    def timed(*a, **k):
        raise AssertionError("a cached decision must not be timed again")
    monkeypatch.setattr(dp2, "autotune", timed)
    bd2.autotune(as_u16_tensor(pats), method="fused", cache=path)
    assert dp2.get_tile()["slabs"] == narrower and bd2.tuned["cached"]
    same(bd2.find_bands(pats, method="fused"), bd.find_bands(pats, method="fused"))


def test_mixed_autotune_keeps_the_one_launch_records(cuda):
    import torch
    mb = MixedBandDetect(nBands=10, mask_for=syn.circular_mask)
    dev = torch.device("cuda", 0)
    batches = {(h, h): as_u16_tensor(patterns(n, h, 300 + h)).to(dev)
               for h, n in ((60, 256), (120, 128), (240, 24))}
    before = mb.find_bands_device(batches)
    assert mb.last_mixed
    before = {k: {f: v.cpu().numpy() for f, v in o.items()} for k, o in before.items()}
    chosen = mb.autotune(batches)
    assert set(chosen) == set(batches)
    for key, c in chosen.items():
        info = mb.plan(*key)._device_plan().get_tile()
        assert c["slabs"] == info["slabs"] and info["slabs_min"] <= c["slabs"] <= info["slabs_max"], (key, c, info)
        assert info["tile"] == (1 if info["single_fits"] else 2)  # single-size calls keep the rule
    print("mixed autotune:", chosen)
    after = mb.find_bands_device(batches)
    assert mb.last_mixed
    for k in batches:
        for f in FIELDS:
            assert after[k][f].cpu().numpy().tobytes() == before[k][f].tobytes(), (k, f)
