"""GPU edge cases: empty and single-pattern input, degenerate patterns, chunk boundaries,
input types, host vs device entry points, determinism and error reporting."""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import synthetic as syn
from bandcmp import compare

pytestmark = pytest.mark.gpu


def make_bd(h=60, w=60, nRho=90, nBands=8, mask=True):
    bd = pg.BandDetect(nTheta=180, nRho=nRho, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=nBands)
    bd.band_detect_setup(patDim=(h, w), patternmask=syn.circular_mask(h, w) if mask else None)
    return bd


@pytest.fixture(scope="module")
def pats60():
    return syn.make_patterns(40, 60, 60, seed=77, noise_frac=0.2)[0]


@pytest.mark.parametrize("method", ["plain", "fused", "fused16"])
def test_empty_input(cuda, method):
    bd = make_bd()
    out = bd.find_bands(np.zeros((0, 60, 60), np.uint8), method=method)
    assert out.shape == (0, 8)


@pytest.mark.parametrize("method", ["plain", "fused"])
def test_single_2d_pattern_equals_batched(cuda, pats60, method):
    bd = make_bd()
    one = bd.find_bands(pats60[5], method=method)
    allp = bd.find_bands(pats60, method=method)
    assert one.shape == (1, 8)
    for f in ("max", "aveloc", "theta", "rho", "valid"):
        assert np.array_equal(one[f][0], allp[f][5]), f


@pytest.mark.parametrize("method", ["plain", "fused", "fused16"])
def test_zero_and_constant_patterns(cuda, method):
    bd = make_bd()
    z = np.zeros((3, 60, 60), np.uint8)
    out = bd.find_bands(z, method=method)
    assert np.all(out["valid"] == 0)
    assert np.all(out["max"] == np.float32(-2.0e6))
    assert np.allclose(out["maxloc"], -11) and np.allclose(out["aveloc"], -11)
    assert np.allclose(out["theta"], np.float32(np.pi))


@pytest.mark.parametrize("method", ["plain", "fused"])
def test_chunk_boundaries(cuda, pats60, method):
    bd = make_bd()
    ref = bd.find_bands(pats60, method=method, chunksize=0)
    for cs in (1, 7, 39, 41):
        out = bd.find_bands(pats60, method=method, chunksize=cs)
        for f in ("max", "aveloc", "valid", "width"):
            assert np.array_equal(out[f], ref[f]), (cs, f)


@pytest.mark.parametrize("method", ["plain", "fused"])
def test_determinism(cuda, pats60, method):
    bd = make_bd()
    a = bd.find_bands(pats60, method=method)
    for _ in range(3):
        b = bd.find_bands(pats60, method=method)
        assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("method", ["plain", "fused"])
def test_torch_device_input_equals_host_input(cuda, pats60, method):
    import torch
    bd = make_bd()
    host = bd.find_bands(pats60, method=method)
    dev = bd.find_bands(torch.from_numpy(pats60).to(cuda), method=method)
    assert host.tobytes() == dev.tobytes()


def test_input_types_agree(cuda, pats60):
    """uint8, uint16 and float32 encodings of the same integer patterns give the same bands."""
    bd = make_bd()
    a = bd.find_bands(pats60, method="plain")
    b = bd.find_bands(pats60.astype(np.uint16), method="plain")
    c = bd.find_bands(pats60.astype(np.float32), method="plain")
    d = bd.find_bands(pats60.astype(np.int32), method="plain")
    assert a.tobytes() == b.tobytes() == c.tobytes() == d.tobytes()


def test_uint16_extremes(cuda):
    bd = make_bd()
    p = syn.make_patterns(6, 60, 60, seed=5, dtype=np.uint16, peak=60000.0)[0]
    p[0] = 65535
    for m in ("plain", "plain64"):
        out = bd.find_bands(p, method=m)
        assert np.isfinite(out["max"]).all()


@pytest.mark.parametrize("nb", [1, 32])
def test_band_count_limits(cuda, pats60, nb):
    bd = make_bd(nBands=nb)
    out = bd.find_bands(pats60[:4], method="plain")
    assert out.shape == (4, nb)


def test_too_many_bands_is_an_error(cuda, pats60):
    bd = make_bd(nBands=33)
    with pytest.raises(RuntimeError, match="invalid argument"):
        bd.find_bands(pats60[:2], method="plain")


def test_unknown_method(cuda, pats60):
    bd = make_bd()
    with pytest.raises(ValueError):
        bd.find_bands(pats60[:2], method="nope")


@pytest.mark.parametrize("n", [2, 3, 5, 6, 7, 9, 15, 41])
def test_packed_passes_partial_units_equal_plain(cuda, n):
    """uint8 patterns without background run eight (or four, two) per pass in the fused kernel;
    counts that are not a multiple leave the last pass partly empty.  Records equal the
    per-stage path's."""
    bd = make_bd()
    pats = syn.make_patterns(n, 60, 60, seed=900 + n, noise_frac=0.2)[0]
    a = bd.find_bands(pats, method="plain")
    b = bd.find_bands(pats, method="fused")
    for f in ("max", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
        assert a[f].tobytes() == b[f].tobytes(), f
    np.testing.assert_allclose(a["normmax"], b["normmax"], rtol=1e-6)
