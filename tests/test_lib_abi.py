"""The C-ABI library builds, loads and exports every symbol its header declares."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def header_functions():
    src = open(os.path.join(ROOT, "include", "ebsdgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ebsd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = header_functions()
    for n in ("ebsd_plan_create", "ebsd_plan_destroy", "ebsd_find_bands", "ebsd_find_bands_host",
              "ebsd_strerror"):
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_strerror_texts(built_lib):
    from pyebsdindex_gb300 import _lib
    lib = _lib.load()
    assert lib.ebsd_strerror(0).decode() == "success"
    for code in range(-7, 0):
        assert lib.ebsd_strerror(code).decode() != "unknown error"
    assert lib.ebsd_strerror(-99).decode() == "unknown error"
    assert b"sm_103a" in lib.ebsd_version()


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_plan_create_without_device_raises(built_lib):
    import pyebsdindex_gb300 as pg
    bd = pg.BandDetect(patDim=(20, 20), nRho=30, nTheta=60, tSigma=1.0, rSigma=1.0)
    with pytest.raises(RuntimeError, match="CUDA device"):
        bd.find_bands(np.zeros((2, 20, 20), np.uint8))


def test_plan_create_rejects_bad_descriptors(built_lib):
    from pyebsdindex_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ebsd_plan_create(None, 0, ctypes.byref(h)) == -1
    d = _lib.PlanDesc()
    d.H = 0
    assert lib.ebsd_plan_create(ctypes.byref(d), 0, ctypes.byref(h)) == -1


def test_tile_entries_reject_null_arguments(built_lib):
    from pyebsdindex_gb300 import _lib
    lib = _lib.load()
    info = _lib.TileInfo()
    assert lib.ebsd_plan_get_tile(None, ctypes.byref(info)) == -1
    assert lib.ebsd_plan_set_tile(None, 1, 0) == -1
    assert lib.ebsd_plan_set_patterns_per_pass(None, 1) == -1
