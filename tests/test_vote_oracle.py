"""The triplet-voting oracle (oracle/vote_oracle.py) against the reference's own bandindex
outputs (tests/golden/vote_*.npz, made by tests/golden/make_vote_golden.py through the
reference source).  Every output and intermediate must be bit-identical, except where the
reference's np.argsort meets equal keys: its order for ties comes from numpy's SIMD sort and
the oracle (like the device) keeps band order instead."""
import os
import platform

import numpy as np
import pytest

from conftest import GOLDEN_DIR, vote_golden_names
from oracle import vote_oracle as vo

OUTS = ("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit")
MIDS = ("accw", "accn", "bandfam", "bandrank", "polevalid")


def differing_rows(a, b):
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    same = (a == b) | ((a != a) & (b != b))
    return set(np.nonzero(~same.all(axis=1))[0].tolist())


@pytest.mark.parametrize("name", vote_golden_names())
def test_oracle_reproduces_reference_bandindex(name):
    lib, params, ins, outs = vo.load_case(os.path.join(GOLDEN_DIR, name + ".npz"))
    res, mid = vo.bandindex(lib, params, ins["norms"], ins["inten"])
    bad = set()
    for k, v in zip(OUTS, res):
        ref = outs["out_" + k]
        assert v.dtype == ref.dtype and v.shape == ref.shape, k
        bad |= differing_rows(v, ref)
    for k in MIDS:
        assert mid[k].tobytes() == outs["mid_" + k].tobytes(), k  # the vote itself has no ties to break
    n = ins["norms"].shape[0]
    assert len(bad) <= max(1, n // 20), sorted(bad)
    if not params["simpleqweights"]:
        assert not bad, sorted(bad)


@pytest.mark.skipif(platform.machine() != "x86_64", reason="numpy's SIMD sort order is platform-specific")
def test_tie_rows_are_the_sort_order(monkeypatch):
    """With numpy's own np.argsort put back for the QUEST weight ranking, the simple-weights case
    (whose band scores tie at 0) matches the reference everywhere."""
    lib, params, ins, outs = vo.load_case(os.path.join(GOLDEN_DIR, "vote_fcc_syn_simpleq.npz"))
    real = np.argsort

    def numpy_default(a, *args, **kw):
        kw.pop("kind", None)
        return real(a, *args, **kw)

    monkeypatch.setattr(vo.np, "argsort", numpy_default)
    res, _ = vo.bandindex(lib, params, ins["norms"], ins["inten"])
    for k, v in zip(OUTS, res):
        assert v.tobytes() == outs["out_" + k].tobytes(), k


def test_band_intensity_matches_indexer():
    lib, params, ins, outs = vo.load_case(os.path.join(GOLDEN_DIR, "vote_fcc_orient.npz"))
    adj, pq, iq = vo.band_intensity(ins["rec_max"], ins["rec_normmax"], ins["rec_theta"], ins["rec_rho"],
                                    ins["rec_valid"], ins["rhomax"])
    assert adj.tobytes() == ins["inten"].tobytes()
    assert pq.tobytes() == ins["ref_pq"].astype(np.float32).tobytes()
    assert iq.tobytes() == ins["ref_iq"].astype(np.float32).tobytes()


def test_vote_library_tables_are_consistent():
    for name in vote_golden_names():
        lib, params, _, _ = vo.load_case(os.path.join(GOLDEN_DIR, name + ".npz"))
        nfam = int(lib["nfam"])
        assert lib["trip_familyid"].max() < nfam and lib["familyid"].max() < nfam
        assert (lib["famIndex"] + lib["nFamily"] <= lib["polesCart"].shape[0]).all()
        assert set(np.unique(lib["lut"])) <= {0, 1, 2}
        assert np.all(np.diff(lib["trip_angles"], axis=1) >= 0)  # rows ascending (_sortlib_id)


@pytest.mark.parametrize("name", vote_golden_names())
def test_c_port_agrees_with_reference(name):
    """oracle/c/votecpu.c (the multi-core CPU baseline of the vote) against the reference's
    outputs: nMatch equal on every pattern; pole match, band pair and acc_correct identical on
    at least 90 % (the rest decide near-ties through libm's arccos, as the device does); on
    those, quaternions within 1e-7."""
    from oracle import votecport
    lib, params, ins, outs = vo.load_case(os.path.join(GOLDEN_DIR, name + ".npz"))
    got = dict(zip(OUTS, votecport.bandindex(lib, params, ins["norms"], ins["inten"], threads=4)))
    assert np.array_equal(got["nmatch"], outs["out_nmatch"])
    n = ins["norms"].shape[0]
    same = np.ones(n, bool)
    for k in ("polematch", "ij", "acc_correct"):
        a, b = got[k].reshape(n, -1), outs["out_" + k].reshape(n, -1)
        same &= np.all(a == b, axis=1)
    assert same.mean() >= 0.9, same.mean()
    if not params["simpleqweights"]:
        np.testing.assert_allclose(got["quat"][same], outs["out_quat"][same], atol=1e-7)
