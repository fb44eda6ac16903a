"""Mixed pattern sizes in one batch (60x60 / 120x120 / 240x240 uint16 at 4000 counts, nRho =
1.5*size, nBands 10): per-size plans, one persistent launch over all sizes, results in input
order, equal to running each size alone; and the precision study on it: FP16 Radon storage vs
FP32 vs the FP64 GPU oracle."""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300.band_detect import MixedBandDetect
from pyebsdindex_gb300 import synthetic as syn
from bandcmp import compare

pytestmark = pytest.mark.gpu


def mixed_batch(n_each=12):
    pats = []
    for k, h in enumerate((60, 120, 240)):
        p = syn.make_patterns(n_each, h, h, seed=700 + 100 * k, dtype=np.uint16, peak=4000.0)[0]
        pats.append([x.astype(np.float32) for x in p])
    # interleave one third each
    out = []
    for a, b, c in zip(*pats):
        out += [a, b, c]
    return out


def test_mixed_sizes_equal_per_size_runs(cuda):
    pats = mixed_batch()
    mb = MixedBandDetect(nBands=10, mask_for=syn.circular_mask)
    rec = mb.find_bands(pats)
    assert rec.shape == (len(pats), 10)
    for h in (60, 120, 240):
        idx = [k for k, p in enumerate(pats) if p.shape[0] == h]
        bd = mb.plan(h, h)
        alone = bd.find_bands(np.stack([pats[k] for k in idx]), method=mb.method_for(h, h, 2))
        for f in ("max", "maxloc", "aveloc", "valid", "theta", "rho"):
            assert np.array_equal(rec[f][idx], alone[f]), (h, f)
        assert (rec["valid"][idx] == 1).mean() > 0.8


@pytest.mark.parametrize("h", [60, 120, 240])
def test_mixed_precision_vs_fp64(cuda, h):
    pats = np.stack([p for p in mixed_batch(16) if p.shape[0] == h])
    mb = MixedBandDetect(nBands=10, mask_for=syn.circular_mask)
    bd = mb.plan(h, h)
    ref = bd.find_bands(pats, method="plain64")
    c32 = compare(bd.find_bands(pats, method="plain"), ref)
    assert c32["frac"] >= 0.999 and c32["aveloc"] <= 1e-3, c32
    if bd._device_plan().supported("fused"):
        cf = compare(bd.find_bands(pats, method="fused"), ref)
        assert cf["frac"] >= 0.999 and cf["aveloc"] <= 1e-3, cf
    if bd._device_plan().supported("fused16"):
        c16 = compare(bd.find_bands(pats, method="fused16"), ref)
        print(h, "fused16 vs fp64", c16)
        assert c16["frac"] >= 0.98 and c16["aveloc_p50"] <= 2e-3, c16


def test_mixed_uint16_one_launch(cuda):
    """uint16 patterns of three sizes in unequal numbers through one launch (ebsd_find_bands_mixed):
    every band field equals the single-size fused call's, normmax to its last bits."""
    import torch
    if getattr(torch, "uint16", None) is None:
        pytest.skip("torch without uint16")
    mb = MixedBandDetect(nBands=10, mask_for=syn.circular_mask)
    batches = {(h, h): syn.make_patterns(n, h, h, seed=40 + h, dtype=np.uint16, peak=4000.0, noise_frac=0.1)[0]
               for h, n in ((60, 301), (120, 77), (240, 19))}
    recs = mb.find_bands_grouped(batches)
    assert mb.last_mixed
    for key, pats in batches.items():
        alone = mb.plan(*key).find_bands(pats, method="fused")
        for f in ("max", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
            assert recs[key][f].tobytes() == alone[f].tobytes(), (key, f)
        np.testing.assert_allclose(recs[key]["normmax"], alone["normmax"], rtol=1e-6)


def test_mixed_one_launch_in_a_cuda_graph(cuda):
    """The mixed-size launch writing a previous call's outputs is captured in a CUDA graph; a
    replay on new patterns in the same input buffers equals a direct call on them."""
    import torch
    if getattr(torch, "uint16", None) is None:
        pytest.skip("torch without uint16")
    dev = torch.device("cuda", 0)
    mb = MixedBandDetect(nBands=10, mask_for=syn.circular_mask)

    def batch(seed):
        return {(h, h): torch.from_numpy(syn.make_patterns(n, h, h, seed=seed + h, dtype=np.uint16, peak=4000.0,
                                                           noise_frac=0.1)[0].view(np.int16)).to(dev).view(torch.uint16)
                for h, n in ((60, 64), (120, 32), (240, 8))}
    bufs = batch(500)
    outs = mb.find_bands_device(bufs)
    torch.cuda.synchronize()
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        mb.find_bands_device(bufs, stream=side, out=outs)
    torch.cuda.synchronize()
    new = batch(900)
    for k in bufs:
        bufs[k].copy_(new[k])
    g.replay()
    torch.cuda.synchronize()
    got = {k: {f: v.cpu().numpy() for f, v in o.items()} for k, o in outs.items()}
    ref = mb.find_bands_device(new)
    torch.cuda.synchronize()
    for k in bufs:
        for f in ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
            assert got[k][f].tobytes() == ref[k][f].cpu().numpy().tobytes(), (k, f)
    with pytest.raises(ValueError):
        mb.find_bands_device({(60, 60): bufs[(60, 60)]}, out=outs)
