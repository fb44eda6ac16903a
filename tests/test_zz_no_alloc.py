"""ebsd_find_bands_static: band detection for callers that may not allocate device memory.

Applications whose device memory belongs to a framework pool, or streaming loops that must
keep a fixed device footprint, cannot let the library cudaMalloc a per-plan workspace.  The
static entry point runs the same per-stage FP32 kernels with their scratch in the library's
64 MiB file-scope device array.  These tests call it through the C ABI and check it against
the allocating entry point (ebsd_find_bands, EBSD_PLAIN_F32) on two consecutive calls of
different sizes (the second call must not see the first call's scratch), and that a request
larger than the array is refused.  This file is collected last so that a failure here leaves
every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import _lib
from pyebsdindex_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

EBSD_E_SCRATCH = -8
MAX_PER_CALL_80 = 183  # 64 MiB / 365,816 B per 80x80 pattern (nRho 120, nTheta 180, padding 11)


def _bind():
    lib = _lib.load()
    f = lib.ebsd_find_bands_static
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.POINTER(_lib.Bands), C.c_void_p]
    f.restype = C.c_int
    return lib


def _outputs(torch, n, nB, dev):
    return {
        "max": torch.empty((n, nB), dtype=torch.float32, device=dev),
        "normmax": torch.empty((n, nB), dtype=torch.float32, device=dev),
        "maxloc": torch.empty((n, nB, 2), dtype=torch.float32, device=dev),
        "avemax": torch.empty((n, nB), dtype=torch.float32, device=dev),
        "aveloc": torch.empty((n, nB, 2), dtype=torch.float32, device=dev),
        "width": torch.empty((n, nB), dtype=torch.float32, device=dev),
        "theta": torch.empty((n, nB), dtype=torch.float32, device=dev),
        "rho": torch.empty((n, nB), dtype=torch.float32, device=dev),
        "valid": torch.empty((n, nB), dtype=torch.int8, device=dev),
    }


def _plan():
    bd = pg.BandDetect(nTheta=180, nRho=120, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=9)
    bd.band_detect_setup(patDim=(80, 80), patternmask=syn.circular_mask(80, 80))
    return bd._device_plan()


def test_static_scratch_matches_allocating_entry(cuda):
    import torch
    lib = _bind()
    plan = _plan()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    for n, seed in ((150, 501), (97, 502)):
        pats = syn.make_patterns(n, 80, 80, seed=seed, noise_frac=0.1)[0]
        d = torch.from_numpy(pats).to(cuda)
        got = _outputs(torch, n, 9, cuda)
        want = _outputs(torch, n, 9, cuda)
        b = _lib.Bands(**{k: C.c_void_p(v.data_ptr()) for k, v in got.items()})
        rc = lib.ebsd_find_bands_static(plan.handle, _lib.EBSD_U8, C.c_void_p(d.data_ptr()), n,
                                        C.byref(b), C.c_void_p(stream))
        assert rc == 0, lib.ebsd_strerror(rc)
        plan.find_bands_device(d.data_ptr(), _lib.EBSD_U8, n, {k: v.data_ptr() for k, v in want.items()},
                               "plain", stream=stream)
        torch.cuda.synchronize()
        for k in got:
            np.testing.assert_array_equal(got[k].cpu().numpy(), want[k].cpu().numpy(), err_msg=k)
        assert int(got["valid"].sum()) > 0


def test_static_scratch_refuses_oversize_request(cuda):
    import torch
    lib = _bind()
    plan = _plan()
    n = MAX_PER_CALL_80 + 1
    d = torch.zeros((n, 80, 80), dtype=torch.uint8, device=cuda)
    out = _outputs(torch, n, 9, cuda)
    b = _lib.Bands(**{k: C.c_void_p(v.data_ptr()) for k, v in out.items()})
    stream = torch.cuda.current_stream(cuda).cuda_stream
    rc = lib.ebsd_find_bands_static(plan.handle, _lib.EBSD_U8, C.c_void_p(d.data_ptr()), n, C.byref(b),
                                    C.c_void_p(stream))
    assert rc == EBSD_E_SCRATCH
    assert b"static device array" in lib.ebsd_strerror(rc)
    # the largest admissible request still runs
    rc = lib.ebsd_find_bands_static(plan.handle, _lib.EBSD_U8, C.c_void_p(d.data_ptr()), n - 1, C.byref(b),
                                    C.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(out["valid"][: n - 1].sum()) == 0  # all-zero patterns have no valid band
