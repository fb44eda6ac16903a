"""Triplet voting on the device (ebsd_band_index) against the reference's own bandindex outputs
(tests/golden/vote_*.npz; the oracle in oracle/vote_oracle.py reproduces them bit for bit).

The device's arccos is correctly rounded where numpy's float32 arccos is not, and its 3-term
dot products take BLAS's sgemm order everywhere, so float32 values can differ in the last bit.
That matters where the reference itself is deciding a near-tie: between symmetry-equivalent
TRIAD solutions (the candidates of one pole family score the same up to rounding) and between
band pairs that reach the same solution.  So each pattern must be one of:
  * identical: pole match, nMatch, band pair, acc_correct, polevalid, voted family and vote
    counts all equal; quaternion within 1e-7, fit and per-band fit within 1e-5 deg, cm and the
    weighted votes within 1e-5 relative, band ranks in the same order and within 1e-2 relative;
  * equivalent: nMatch, acc_correct, polevalid, voted family and vote counts equal, the matched
    poles of the same families, and the two orientations related by a rotation that maps the
    library's pole set onto itself (a crystal symmetry), fits within 1e-4 deg;
and at most 2 % of a case's patterns may be neither (a vote or a tolerance test on the
other side of its edge).  Patterns whose QUEST band selection meets a tie in its scores keep
the integer bar only (see quest_tie_rows).  The band-weight kernel must be bit-identical."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, vote_golden_names
from oracle import vote_oracle as vo

pytestmark = pytest.mark.gpu

INTS = ("polematch", "nmatch", "ij", "acc_correct")
MID_INTS = ("accn", "bandfam", "polevalid")


def load(name):
    return vo.load_case(os.path.join(GOLDEN_DIR, name + ".npz"))


def indexer(lib, params):
    from pyebsdindex_gb300 import tripletvote as tv
    return tv.BandIndexer(lib=lib, angTol=params["angTol"], nband_earlyexit=params["nband_earlyexit"],
                          simpleqweights=params["simpleqweights"], high_fidelity=True)


def run(bi, norms, inten, intermediates=True):
    import torch
    d_n = torch.from_numpy(np.ascontiguousarray(norms)).cuda()
    d_i = torch.from_numpy(np.ascontiguousarray(inten)).cuda() if inten is not None else None
    out = bi.bandindex_device(d_n, d_i, intermediates=intermediates)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def rows_equal(a, b):
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    return np.all((a == b) | ((a != a) & (b != b)), axis=1)


def rot_matrix(q):
    """Matrix of the reference's passive quaternion rotation (rotlib.quat_vectorL1N)."""
    return vo.quat_vector_l1n(np.asarray(q, np.float64), np.eye(3)).T


def symmetry_related(q1, q2, poles, tol=1e-5):
    """True when the rotation taking orientation q1's frame to q2's maps the pole set onto
    itself (every rotated pole lands on a library pole)."""
    M = rot_matrix(q2) @ rot_matrix(q1).T
    mp = poles @ M.T
    return bool(np.all(np.max(mp @ poles.T, axis=1) > 1.0 - tol))


def classify(got, want, lib):
    """Per pattern: 0 identical integers, 1 symmetry-equivalent solution, 2 neither."""
    n = got["nmatch"].shape[0]
    same = np.ones(n, bool)
    for k in INTS:
        same &= rows_equal(got[k], want["out_" + k])
    for k in MID_INTS:
        same &= rows_equal(got[k], want["mid_" + k])
    core = rows_equal(got["nmatch"], want["out_nmatch"]) & rows_equal(got["acc_correct"], want["out_acc_correct"])
    for k in MID_INTS:
        core &= rows_equal(got[k], want["mid_" + k])
    fam = np.asarray(lib["familyid"])
    pg, pw = got["polematch"], want["out_polematch"]
    core &= rows_equal(np.where(pg >= 0, fam[pg.clip(0)], -1), np.where(pw >= 0, fam[pw.clip(0)], -1))
    poles = np.asarray(lib["polesCart"], np.float64)
    cls = np.full(n, 2)
    cls[same] = 0
    for p in np.nonzero(core & ~same)[0]:
        if (symmetry_related(want["out_quat"][p], got["quat"][p], poles)
                and abs(got["fit"][p] - want["out_fit"][p]) < 1e-4):
            cls[p] = 1
    return cls


def quest_tie_rows(lib, params, inten, want):
    """Patterns whose QUEST band selection (the top six scores, tripletvote.py:885-891) meets
    equal scores at its edge: the reference orders those through numpy's SIMD argsort, the
    device keeps band order, so the fitted weights -- and the quaternion -- may differ."""
    fam = np.asarray(lib["familyid"])
    pm, pv = want["out_polematch"], want["mid_polevalid"]
    accw, accn = want["mid_accw"], want["mid_accn"]
    n, nb = pm.shape
    tie = np.zeros(n, bool)
    for p in range(n):
        good = np.nonzero(pv[p] > 0)[0]
        if good.size < 3:
            continue
        score = np.full(nb, -1.0, np.float32)
        for q, g in enumerate(good):
            if params["simpleqweights"]:
                score[g] = inten[p, q]
            else:
                a = fam[pm[p, g]]
                score[g] = accw[p, a, g] / (accn[p, a, g] if accn[p, a, g] > 0 else np.float32(1e-12))
        srt = np.sort(score)[::-1]
        nfit = min(6, good.size)
        tie[p] = nfit < nb and srt[nfit - 1] == srt[nfit]
    return tie


def compare(got, want, lib, tie=None, max_other=0.02):
    cls = classify(got, want, lib)
    n = cls.size
    assert (cls == 2).mean() <= max_other, ((cls == 2).mean(), np.nonzero(cls == 2)[0][:20])
    if tie is not None:
        assert tie.mean() <= 0.2
        cls[(cls == 0) & tie] = 3  # integers identical, QUEST weights chosen through a tie
    a = cls == 0
    np.testing.assert_allclose(got["quat"][a], want["out_quat"][a], atol=1e-7, rtol=0)
    np.testing.assert_allclose(got["fit"][a], want["out_fit"][a], atol=1e-5, rtol=0)
    np.testing.assert_allclose(got["bandfit"][a], want["out_bandfit"][a], atol=1e-5, rtol=0)
    np.testing.assert_allclose(got["cm"][a], want["out_cm"][a], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(got["accw"][a], want["mid_accw"][a], rtol=1e-5, atol=1e-5)
    # rank = (top vote - runner-up) / int(vote sum) * int(top vote): a vote sum an ulp either side
    # of an integer moves the rank by a percent; the order of the ranks is what the search uses
    np.testing.assert_allclose(got["bandrank"][a], want["mid_bandrank"][a], rtol=1e-2, atol=5e-5)
    assert np.array_equal(np.argsort(got["bandrank"][a], axis=1, kind="stable"),
                          np.argsort(want["mid_bandrank"][a], axis=1, kind="stable"))
    e = cls == 1
    np.testing.assert_allclose(got["bandfit"][e], want["out_bandfit"][e], atol=1e-4, rtol=0)
    return cls


@pytest.mark.parametrize("name", vote_golden_names())
def test_device_bandindex_matches_reference(cuda, name):
    lib, params, ins, outs = load(name)
    got = run(indexer(lib, params), ins["norms"], ins["inten"])
    compare(got, outs, lib, tie=quest_tie_rows(lib, params, ins["inten"], outs))


def test_host_api_returns_reference_tuple(cuda):
    lib, params, ins, outs = load("vote_fcc_syn")
    res = indexer(lib, params).bandindex(ins["norms"], band_intensity=ins["inten"], band_widths=None)
    assert len(res) == 8
    for v, k in zip(res, ("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit")):
        ref = outs["out_" + k]
        assert v.dtype == ref.dtype and v.shape == ref.shape, k
    single = indexer(lib, params).bandindex(ins["norms"][3], band_intensity=ins["inten"][3])
    assert single[4].shape == (1,) and single[4][0] == res[4][3]


def test_no_intensity_means_ones(cuda):
    lib, params, ins, _ = load("vote_fcc_syn")
    ones = np.ones_like(ins["inten"])
    a = run(indexer(lib, params), ins["norms"][:60], None)
    b = run(indexer(lib, params), ins["norms"][:60], ones[:60])
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k


def test_band_intensity_kernel_is_bit_exact(cuda):
    import torch
    from pyebsdindex_gb300 import tripletvote as tv
    _, _, ins, _ = load("vote_fcc_orient")
    t = {k: torch.from_numpy(np.ascontiguousarray(ins["rec_" + k])).cuda()
         for k in ("max", "normmax", "theta", "rho", "valid")}
    adj, pq, iq = tv.band_intensity_gpu(t["max"], t["normmax"], t["theta"], t["rho"], t["valid"], ins["rhomax"])
    assert adj.cpu().numpy().tobytes() == ins["inten"].tobytes()
    assert pq.cpu().numpy().tobytes() == ins["ref_pq"].astype(np.float32).tobytes()
    assert iq.cpu().numpy().tobytes() == ins["ref_iq"].astype(np.float32).tobytes()


def test_records_to_orientations_on_the_device(cuda):
    """find_bands -> ebsd_radon2pole -> ebsd_band_intensity -> ebsd_band_index without leaving
    the device, against the oracle fed the same device normals and weights."""
    import torch
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import radon_fast, tripletvote as tv
    from pyebsdindex_gb300 import synthetic as syn
    lib, params, _, _ = load("vote_fcc_syn")
    bd = pg.BandDetect(nTheta=180, nRho=120, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=9)
    bd.band_detect_setup(patDim=(80, 80), patternmask=syn.circular_mask(80, 80))
    pats = syn.make_patterns(120, 80, 80, seed=31, noise_frac=0.1)[0]
    plan = bd._device_plan()
    dev = bd._find_bands_dev(plan, torch.from_numpy(pats).cuda(), bd._pick_method(plan, "fused"), 0)
    normals = radon_fast.radon2pole_gpu(dev["theta"], dev["rho"], (80, 80), PC=[0.46, 0.70, 0.64], vendor="EDAX")
    adj, pq, iq = tv.band_intensity_gpu(dev["max"], dev["normmax"], dev["theta"], dev["rho"], dev["valid"], bd.rhoMax)
    got = {k: v.cpu().numpy() for k, v in indexer(lib, params).bandindex_device(normals, adj).items()}
    res, _ = vo.bandindex(lib, params, normals.cpu().numpy(), adj.cpu().numpy())
    agree = np.ones(len(pats), bool)
    for k, v in zip(("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit"), res):
        if k in INTS:
            agree &= rows_equal(got[k], v)
    assert agree.mean() >= 0.98
    np.testing.assert_allclose(got["quat"][agree], res[0][agree], atol=1e-7)
    assert (got["nmatch"] >= 3).mean() > 0.8  # most synthetic patterns index


def test_band_index_replays_in_a_cuda_graph(cuda):
    import torch
    lib, params, ins, outs = load("vote_bcc_syn")
    bi = indexer(lib, params)
    d_n = torch.from_numpy(ins["norms"]).cuda()
    d_i = torch.from_numpy(ins["inten"]).cuda()
    out = bi.bandindex_device(d_n, d_i)  # plan creation and launch attributes outside the capture
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        bi.bandindex_device(d_n, d_i, out=out, stream=s.cuda_stream)
    want = {k: v.clone() for k, v in out.items()}
    for v in out.values():
        v.zero_()
    g.replay()
    torch.cuda.synchronize()
    for k in out:
        assert torch.equal(out[k], want[k]), k


def test_bad_arguments(cuda):
    import torch
    from pyebsdindex_gb300 import tripletvote as tv
    lib, params, ins, _ = load("vote_fcc_syn4")
    bi = indexer(lib, params)
    with pytest.raises(RuntimeError, match="invalid argument"):
        bi.bandindex_device(torch.zeros((2, 33, 3), device="cuda"))
    bad = dict(lib)
    bad["nfam"] = 1
    with pytest.raises(RuntimeError, match="invalid argument"):
        tv.BandIndexer(lib=bad).plan()
    with pytest.raises(NotImplementedError):
        tv.BandIndexer(lib=lib, high_fidelity=False).plan()


def test_many_matches_per_triplet_take_the_ordered_fallback(cuda):
    """A library whose triplet rows repeat 40 times gives band triplets more matches than the
    kernel's 96-entry list: those take the one-at-a-time path, still in library order.  The
    oracle runs the same duplicated library."""
    lib, params, ins, _ = load("vote_fcc_syn")
    dup = dict(lib)
    dup["trip_angles"] = np.tile(lib["trip_angles"], (40, 1))
    dup["trip_familyid"] = np.tile(lib["trip_familyid"], (40, 1))
    n = 40
    got = run(indexer(dup, params), ins["norms"][:n], ins["inten"][:n])
    want, mid = vo.bandindex(dup, params, ins["norms"][:n], ins["inten"][:n])
    assert (mid["accn"].max(axis=(1, 2)) > 96).any()  # some band triplet overflowed the list
    same = np.ones(n, bool)
    for k, v in zip(("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit"), want):
        if k in INTS:
            same &= rows_equal(got[k], v)
    same &= rows_equal(got["accn"], mid["accn"])
    assert same.mean() >= 0.9
    np.testing.assert_allclose(got["accw"][same], mid["accw"][same], rtol=1e-5, atol=1e-4)


def test_many_bands_against_the_c_port(cuda):
    """24 bands per pattern (the kernel's per-warp tables grow with nBands): seeded FCC normals
    under random rotations with 0.3 deg of noise, against the C/OpenMP restatement of bandindex
    (oracle/c/votecpu.c, libm arccos): nMatch equal on every pattern, pole match and band pair
    on at least 98 %, quaternions within 1e-7 there."""
    from oracle import votecport
    lib, params, _, _ = load("vote_fcc_syn")
    rng = np.random.default_rng(77)
    poles = np.asarray(lib["polesCart"])
    n, nb = 120, 24
    norms = np.zeros((n, nb, 3), np.float32)
    for p in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        pick = rng.choice(poles.shape[0], size=nb, replace=False)
        v = (R @ poles[pick].T).T + rng.normal(scale=np.deg2rad(0.3), size=(nb, 3))
        norms[p] = v / np.linalg.norm(v, axis=1, keepdims=True)
    inten = np.sort(rng.uniform(0.3, 1.0, (n, nb)).astype(np.float32), axis=1)[:, ::-1].copy()
    got = run(indexer(lib, params), norms, inten)
    want = dict(zip(("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit"),
                    votecport.bandindex(lib, params, norms, inten)))
    assert np.array_equal(got["nmatch"], want["nmatch"])
    same = rows_equal(got["polematch"], want["polematch"]) & rows_equal(got["ij"], want["ij"])
    assert same.mean() >= 0.98, same.mean()
    np.testing.assert_allclose(got["quat"][same], want["quat"][same], atol=1e-7)
