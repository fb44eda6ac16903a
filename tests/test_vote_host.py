"""Host side of the device band indexer: the wrapper around a phase library object forwards
attribute reads and writes to it (so an EBSDIndexer keeps working with wrapped phases), reads
the library tables the way the reference's BandIndexer stores them, and raises -- never falls
back to a CPU path -- when there is no CUDA device."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import GOLDEN_DIR, gpu_available
from oracle import vote_oracle as vo


def fake_phase():
    lib, params, _, _ = vo.load_case(os.path.join(GOLDEN_DIR, "vote_fcc_syn4.npz"))
    return SimpleNamespace(
        phasename="Al", angTol=params["angTol"], nband_earlyexit=params["nband_earlyexit"],
        simpleqweights=params["simpleqweights"], high_fidelity=True,
        polefamilies=np.zeros((int(lib["nfam"]), 3)), lut=lib["lut"],
        angtriplets={"angles": lib["trip_angles"], "familyid": lib["trip_familyid"]},
        completelib={k: lib[k] for k in ("polesCart", "familyid", "angTable", "nFamily", "famIndex")}), lib


def test_wrapper_forwards_attributes():
    from pyebsdindex_gb300 import tripletvote as tv
    phase, lib = fake_phase()
    bi = tv.BandIndexer(phase)
    assert bi.phasename == "Al" and bi.angTol == phase.angTol
    bi.nband_earlyexit = 5
    assert bi.nband_earlyexit == 5
    bi.phasename = "Ni"
    assert phase.phasename == "Ni"
    got = tv.phase_library(phase)
    for k in ("trip_angles", "trip_familyid", "lut", "polesCart", "angTable", "famIndex", "nFamily"):
        assert np.array_equal(got[k], lib[k]), k
    assert got["nfam"] == int(lib["nfam"])


def test_defaults_without_a_phase_object():
    from pyebsdindex_gb300 import tripletvote as tv
    _, lib = fake_phase()
    bi = tv.BandIndexer(lib=lib)
    assert (bi.angTol, bi.nband_earlyexit, bi.simpleqweights, bi.high_fidelity) == (2.0, 8, False, True)
    with pytest.raises(AttributeError):
        bi.not_an_attribute
    with pytest.raises(ValueError):
        tv.BandIndexer()


def test_descriptor_layout_matches_header():
    """The ctypes mirrors have one field per member of the C structs."""
    import re
    from conftest import ROOT
    from pyebsdindex_gb300 import tripletvote as tv
    src = open(os.path.join(ROOT, "include", "ebsdgpu.h")).read()
    for cname, py in (("ebsd_triplib_desc", tv.TripLibDesc), ("ebsd_index_out", tv.IndexOut)):
        body = re.search(r"typedef struct \{([^}]*)\}\s*" + cname + ";", src).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        names = re.findall(r"\b(\w+)\s*;", body)
        assert names == [f[0] for f in py._fields_], cname


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_plan_without_device_raises(built_lib):
    from pyebsdindex_gb300 import tripletvote as tv
    phase, _ = fake_phase()
    with pytest.raises(RuntimeError, match="CUDA device"):
        tv.BandIndexer(phase).plan()
