"""NLPAR with each unordered pair's distance summed once (ebsd_nlpar_pairs_out) against the
per-slot kernels (ebsd_nlpar_sigma + ebsd_nlpar_out), through the C ABI.  The pair path's
weighted average is the register-blocked kernel (patterns of a multiple of 4 pixels), the
per-slot path's the tiled kernel, so the comparison also pins the one against the other.

A pair's squared difference is symmetric bit for bit, so the two paths must agree exactly:
sigma, and the averaged patterns (float32, uint8 or uint16), for search radii 1-3, with and
without saturation protection, a distance threshold, diff_offset's centre additions, and scans
narrow enough that the windows shifted inward at the edges reach past +-sr (the slots the pair
kernel sums directly).  The sigma of the combined call comes from the same pass over the
patterns; with compute_sigma = 0 a given sigma is used."""

import numpy as np
import pytest

from pyebsdindex_gb300 import _lib
from pyebsdindex_gb300 import nlpar as nlp
from pyebsdindex_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

CASES = [  # nrows, ncols, sr, saturation_protect, dthresh, centre offset, output type[, pattern side]
    (9, 40, 3, True, 0.0, False, "f32"),
    (12, 70, 2, False, 0.5, False, "u8"),
    (7, 33, 1, True, 0.0, True, "f32"),
    (13, 36, 3, True, 0.3, True, "u16"),
    (8, 7, 3, True, 0.0, False, "f32"),
    (10, 45, 3, True, 0.0, False, "u8", 31),  # 961 pixels: not a multiple of 4 (the tiled average)
    (9, 61, 3, True, 0.0, False, "u8", 80),   # the bench's pattern size, interior and edge tiles
    (7, 150, 3, True, 0.2, True, "f32"),      # wider scans: several blocks per row
    (5, 270, 2, True, 0.0, False, "u8"),
    (8, 140, 1, False, 0.0, False, "f32"),
    (7, 160, 3, True, 0.0, False, "u8", 32, 2e-6),  # saturation at a single value
]


def _scan(nr, nc, seed, side=32, satfrac=0.002):
    pats, _ = syn.voronoi_scan(nr, nc, ngrains=6, h=side, w=side, seed=seed, peak_range=(40.0, 220.0))
    pats = pats.astype(np.float32)
    rng = np.random.default_rng(seed)
    sat = rng.random(pats.shape) < satfrac  # a few saturated pixels
    if not sat.any():
        sat.flat[rng.integers(sat.size)] = True
    pats[sat] = pats.max()
    return pats.reshape(nr * nc, -1)


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}x{c[1]}_sr{c[2]}_{c[6]}" + ("_sat1" if len(c) > 8 else "")
                                             for c in CASES])
def test_pair_sums_equal_per_slot_kernels(cuda, case):
    import torch
    nr, nc, sr, sat, dth, use_off, odt = case[:7]
    side = case[7] if len(case) > 7 else 32
    satfrac = case[8] if len(case) > 8 else 0.002
    lib = nlp._bind()
    x = torch.from_numpy(_scan(nr, nc, seed=nr * 100 + nc, side=side, satfrac=satfrac)).to(cuda).contiguous()
    npix, npx = x.shape
    ind = torch.from_numpy(np.nonzero(syn.circular_mask(side, side).ravel())[0].astype(np.int32)).to(cuda)
    dmax = float(x.max().item())
    code, tdt = {"f32": (_lib.EBSD_F32, torch.float32), "u8": (_lib.EBSD_U8, torch.uint8),
                 "u16": (_lib.EBSD_U16, torch.int16)}[odt]
    coff = (torch.from_numpy(np.random.default_rng(3).uniform(0, 0.5, npix).astype(np.float32)).to(cuda)
            if use_off else None)
    cp = None if coff is None else coff.data_ptr()
    st = torch.cuda.current_stream().cuda_stream
    winsz = (2 * sr + 1) ** 2
    nf = sr * (2 * sr + 1) + sr
    # per-slot kernels
    sig_a = torch.empty(npix, dtype=torch.float32, device=cuda)
    _lib.check(lib.ebsd_nlpar_sigma(x.data_ptr(), nr, nc, npx, ind.data_ptr(), ind.numel(), dmax, int(sat),
                                    sig_a.data_ptr(), st))
    out_a = torch.empty((npix, npx), dtype=tdt, device=cuda)
    work_a = torch.empty(npix * winsz, dtype=torch.float32, device=cuda)
    _lib.check(lib.ebsd_nlpar_out(x.data_ptr(), nr, nc, npx, ind.data_ptr(), ind.numel(), dmax, 0.7, sr, dth,
                                  sig_a.data_ptr(), int(sat), work_a.data_ptr(), code, out_a.data_ptr(), cp, st))
    # pair sums, sigma from the same pass
    sig_b = torch.full((npix,), -1.0, dtype=torch.float32, device=cuda)
    out_b = torch.empty((npix, npx), dtype=tdt, device=cuda)
    nedge = 2 * sr * (nr + nc - 2 * sr)
    work_b = torch.empty(npix * (winsz + 2 * nf + 8) + 2 * nedge * winsz + 1, dtype=torch.float32, device=cuda)
    _lib.check(lib.ebsd_nlpar_pairs_out(x.data_ptr(), nr, nc, npx, ind.data_ptr(), ind.numel(), dmax, 0.7, sr, dth,
                                        sig_b.data_ptr(), 1, int(sat), work_b.data_ptr(), code, out_b.data_ptr(), cp,
                                        st))
    torch.cuda.synchronize()
    assert torch.equal(sig_a, sig_b), (sig_a - sig_b).abs().max()
    assert out_a.cpu().numpy().tobytes() == out_b.cpu().numpy().tobytes()
    assert torch.equal(work_a, work_b[:npix * winsz]), "normalised weights differ"
    # a given sigma (compute_sigma = 0) is read, not written
    sig_c = sig_a.clone()
    out_c = torch.empty_like(out_b)
    _lib.check(lib.ebsd_nlpar_pairs_out(x.data_ptr(), nr, nc, npx, ind.data_ptr(), ind.numel(), dmax, 0.7, sr, dth,
                                        sig_c.data_ptr(), 0, int(sat), work_b.data_ptr(), code, out_c.data_ptr(), cp,
                                        st))
    torch.cuda.synchronize()
    assert torch.equal(sig_c, sig_a)
    assert out_c.cpu().numpy().tobytes() == out_a.cpu().numpy().tobytes()


def test_pair_entry_rejects_what_it_does_not_serve(cuda):
    import torch
    lib = nlp._bind()
    x = torch.zeros((49, 64), dtype=torch.float32, device=cuda)
    ind = torch.arange(64, dtype=torch.int32, device=cuda)
    sig = torch.zeros(49, dtype=torch.float32, device=cuda)
    out = torch.empty_like(x)
    work = torch.empty(49 * 200, dtype=torch.float32, device=cuda)
    args = lambda sr: (x.data_ptr(), 7, 7, 64, ind.data_ptr(), 64, 1.0, 0.7, sr, 0.0, sig.data_ptr(), 1, 1,
                       work.data_ptr(), _lib.EBSD_F32, out.data_ptr(), None, 0)
    assert lib.ebsd_nlpar_pairs_out(*args(0)) == -1  # EBSD_E_ARG: radius 0 has no pairs
    assert lib.ebsd_nlpar_pairs_out(*args(4)) == -1  # EBSD_E_ARG: window wider than the 7 x 7 scan
