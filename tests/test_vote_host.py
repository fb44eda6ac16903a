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


def test_wrapped_phases_drive_the_reference_indexer(monkeypatch):
    """The reference's own EBSDIndexer._indexbandsphase (_ebsd_index_single.py:720-830) runs
    with its phases wrapped; the wrapper's device call is stood in for by the oracle (no GPU
    here), so the indexer's outputs must equal the unwrapped run's."""
    import json
    import warnings
    from oracle import refshim
    if not refshim.reference_available():
        pytest.skip("reference source tree not available")
    from pyebsdindex_gb300 import tripletvote as tv
    from pyebsdindex_gb300 import synthetic as syn
    ref = refshim.load()
    d = np.load(os.path.join(GOLDEN_DIR, "orient_80x80.npz"))
    params = json.loads(str(d["params"]))
    pc = tuple(float(x) for x in d["pc"])

    def make():
        idx = ref.ebsd_index_single.EBSDIndexer(PC=pc, patDim=(80, 80), **params)
        idx.bandDetectPlan.band_detect_setup(patDim=(80, 80), patternmask=syn.circular_mask(80, 80))
        return idx

    n = 24
    idx = make()
    recs = np.zeros((n, 9), dtype=idx.bandDetectPlan.dataType)
    for f in ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid"):
        recs[f] = d["ref_" + f][:n]
    norms = idx.bandDetectPlan.radonPlan.radon2pole(recs, PC=np.asarray(pc), vendor="EDAX")
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        want, _ = idx._indexbandsphase(recs, norms)

    def oracle_bandindex(self, band_norms, band_intensity=None, band_widths=None, verbose=0):
        p = {"angTol": self.angTol, "nband_earlyexit": self.nband_earlyexit, "simpleqweights": self.simpleqweights}
        return vo.bandindex(tv.phase_library(self._phase), p, np.asarray(band_norms, np.float32),
                            np.asarray(band_intensity, np.float32))[0]

    monkeypatch.setattr(tv.BandIndexer, "bandindex", oracle_bandindex)
    idx2 = make()
    idx2.phaseLib = [tv.BandIndexer(ph) for ph in idx2.phaseLib]
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        got, _ = idx2._indexbandsphase(recs, norms)
    for f in ("quat", "fit", "cm", "nmatch", "phase", "pq", "iq"):
        assert np.array_equal(got[f], want[f]), f


def test_record_offsets_check_the_field_types():
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import _lib
    dt = pg.record_dtype()
    offs = _lib.record_offsets(dt)
    assert [offs[i] for i in range(9)] == [dt.fields[f][1] for f in _lib.BAND_FIELDS]
    bad = np.dtype([("max", np.float64), ("normmax", np.float32), ("maxloc", np.float32, (2,)),
                    ("avemax", np.float32), ("aveloc", np.float32, (2,)), ("width", np.float32),
                    ("theta", np.float32), ("rho", np.float32), ("valid", np.int8)])
    with pytest.raises(TypeError, match="max"):
        _lib.record_offsets(bad)
