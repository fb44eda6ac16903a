"""Band indexing by triplet voting on the device: a drop-in ``bandindex`` for the reference's
``tripletvote.BandIndexer`` (tripletvote.py:172-633), and the indexer's band weights
(_ebsd_index_single.py:751-763).

``BandIndexer(phase)`` wraps a phase library object -- the reference's own ``BandIndexer`` as
``tripletvote.addphase`` builds it, or anything with its ``angtriplets``, ``lut``,
``completelib``, ``polefamilies``, ``angTol``, ``nband_earlyexit``, ``simpleqweights`` and
``high_fidelity`` attributes -- and replaces its ``bandindex`` with ``ebsd_band_index`` of
libebsdgpu.so; every other attribute read falls through to the wrapped object, so an
``EBSDIndexer`` whose ``phaseLib`` entries are wrapped indexes on the GPU unchanged.  The
library tables can also be given directly as arrays (``lib=``), as the tests do.

Outputs follow the reference: ``(avequat, fit, cm, polematch, nMatch, ij, acc_correct,
bandfit)`` with its dtypes.  Band intensities are taken as float32 (what the indexer passes).
There is no CPU path: without the CUDA library or a device every call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

LIB_KEYS = ("polesCart", "familyid", "angTable", "nFamily", "famIndex")
OUT_NAMES = ("quat", "fit", "cm", "polematch", "nmatch", "ij", "acc_correct", "bandfit")
MID_NAMES = ("accw", "accn", "bandfam", "bandrank", "polevalid")


class TripLibDesc(C.Structure):
    _fields_ = [
        ("nfam", C.c_int32), ("ntrip", C.c_int32), ("trip_angles", C.c_void_p), ("trip_family", C.c_void_p),
        ("lut", C.c_void_p), ("npoles", C.c_int32), ("poles_cart", C.c_void_p), ("pole_family", C.c_void_p),
        ("ang_table", C.c_void_p), ("fam_count", C.c_void_p), ("fam_index", C.c_void_p),
        ("ang_tol", C.c_double), ("nband_earlyexit", C.c_int32), ("simple_qweights", C.c_int32),
    ]


class IndexOut(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in OUT_NAMES + MID_NAMES]


def _bind():
    lib = _lib.load()
    if not hasattr(lib, "_vote_bound"):
        P = C.c_void_p
        lib.ebsd_vote_plan_create.argtypes = [C.POINTER(TripLibDesc), C.c_int, C.POINTER(P)]
        lib.ebsd_vote_plan_create.restype = C.c_int
        lib.ebsd_vote_plan_destroy.argtypes = [P]
        lib.ebsd_vote_plan_destroy.restype = C.c_int
        lib.ebsd_band_index.argtypes = [P, P, P, C.c_int64, C.c_int32, C.POINTER(IndexOut), P]
        lib.ebsd_band_index.restype = C.c_int
        lib.ebsd_band_intensity.argtypes = [P, P, P, P, P, C.c_int64, C.c_int32, C.c_float, P, P, P, P]
        lib.ebsd_band_intensity.restype = C.c_int
        lib._vote_bound = True
    return lib


def phase_library(phase):
    """The library arrays of a reference ``BandIndexer`` (tripletvote.py:320-490)."""
    lib = {k: np.asarray(phase.completelib[k]) for k in LIB_KEYS}
    lib["trip_angles"] = np.asarray(phase.angtriplets["angles"])
    lib["trip_familyid"] = np.asarray(phase.angtriplets["familyid"])
    lib["lut"] = np.asarray(phase.lut)
    lib["nfam"] = int(np.asarray(phase.polefamilies).shape[0])
    return lib


class VotePlan:
    """Owns one ``ebsd_vote_plan_t`` (the phase library on the device)."""

    def __init__(self, lib, angTol, nband_earlyexit, simpleqweights, device=0):
        self._lib = _bind()
        self._keep = {
            "trip_angles": np.ascontiguousarray(lib["trip_angles"], np.float64),
            "trip_family": np.ascontiguousarray(lib["trip_familyid"], np.int64),
            "lut": np.ascontiguousarray(lib["lut"], np.int64),
            "poles": np.ascontiguousarray(lib["polesCart"], np.float64),
            "pfam": np.ascontiguousarray(lib["familyid"], np.int32),
            "angtab": np.ascontiguousarray(lib["angTable"], np.float64),
            "famcnt": np.ascontiguousarray(lib["nFamily"], np.int32),
            "famidx": np.ascontiguousarray(lib["famIndex"], np.int64),
        }
        k = self._keep
        if k["lut"].size != 81:
            raise ValueError("the triplet LUT must have 3x3x3x3 entries")
        d = TripLibDesc()
        d.nfam = int(lib["nfam"])
        d.ntrip = int(k["trip_angles"].shape[0])
        d.trip_angles, d.trip_family, d.lut = (k[n].ctypes.data for n in ("trip_angles", "trip_family", "lut"))
        d.npoles = int(k["poles"].shape[0])
        d.poles_cart, d.pole_family, d.ang_table = (k[n].ctypes.data for n in ("poles", "pfam", "angtab"))
        d.fam_count, d.fam_index = k["famcnt"].ctypes.data, k["famidx"].ctypes.data
        d.ang_tol = float(angTol)
        d.nband_earlyexit = int(nband_earlyexit)
        d.simple_qweights = 1 if simpleqweights else 0
        h = C.c_void_p()
        _lib.check(self._lib.ebsd_vote_plan_create(C.byref(d), int(device), C.byref(h)), "ebsd_vote_plan_create")
        self.handle = h
        self.nfam = d.nfam
        self.device = int(device)

    def index_device(self, norms_ptr, inten_ptr, n, nBands, out_ptrs, stream=0):
        o = IndexOut(**{k: C.c_void_p(int(out_ptrs[k]) if out_ptrs.get(k) else None) for k in OUT_NAMES + MID_NAMES})
        _lib.check(self._lib.ebsd_band_index(self.handle, C.c_void_p(int(norms_ptr)),
                                             C.c_void_p(int(inten_ptr) if inten_ptr else None), int(n),
                                             int(nBands), C.byref(o), C.c_void_p(int(stream))), "ebsd_band_index")

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self._lib.ebsd_vote_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def alloc_outputs(torch, n, nb, nfam, device, intermediates=False):
    f64, f32, i64 = torch.float64, torch.float32, torch.int64
    out = {
        "quat": torch.empty((n, 4), dtype=f64, device=device), "fit": torch.empty(n, dtype=f64, device=device),
        "cm": torch.empty(n, dtype=f32, device=device), "polematch": torch.empty((n, nb), dtype=i64, device=device),
        "nmatch": torch.empty(n, dtype=i64, device=device), "ij": torch.empty((n, 4), dtype=i64, device=device),
        "acc_correct": torch.empty(n, dtype=torch.int32, device=device),
        "bandfit": torch.empty((n, nb), dtype=f64, device=device),
    }
    if intermediates:
        out.update({
            "accw": torch.empty((n, nfam, nb), dtype=f32, device=device),
            "accn": torch.empty((n, nfam, nb), dtype=f32, device=device),
            "bandfam": torch.empty((n, nb), dtype=torch.int32, device=device),
            "bandrank": torch.empty((n, nb), dtype=f32, device=device),
            "polevalid": torch.empty((n, nb), dtype=torch.uint8, device=device),
        })
    return out


class BandIndexer:
    """GPU ``bandindex`` for one phase; see the module docstring."""

    def __init__(self, phase=None, *, lib=None, angTol=None, nband_earlyexit=None, simpleqweights=None,
                 high_fidelity=None, device=0):
        if phase is None and lib is None:
            raise ValueError("give a phase library object or its arrays (lib=)")
        object.__setattr__(self, "_phase", phase)
        object.__setattr__(self, "_lib_arrays", lib)
        object.__setattr__(self, "_over", {k: v for k, v in dict(
            angTol=angTol, nband_earlyexit=nband_earlyexit, simpleqweights=simpleqweights,
            high_fidelity=high_fidelity).items() if v is not None})
        object.__setattr__(self, "device", int(device))
        object.__setattr__(self, "_plan_cache", (None, None))

    # attribute reads fall through to the wrapped phase (phasename, polefamilies, ...)
    def __getattr__(self, name):
        over = object.__getattribute__(self, "_over")
        if name in over:
            return over[name]
        phase = object.__getattribute__(self, "_phase")
        if phase is not None:
            return getattr(phase, name)
        defaults = {"angTol": 2.0, "nband_earlyexit": 8, "simpleqweights": False, "high_fidelity": True}
        if name in defaults:
            return defaults[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in ("angTol", "nband_earlyexit", "simpleqweights", "high_fidelity"):
            self._over[name] = value
        elif self._phase is not None and not name.startswith("_"):
            setattr(self._phase, name, value)
        else:
            object.__setattr__(self, name, value)

    def _library(self):
        return self._lib_arrays if self._lib_arrays is not None else phase_library(self._phase)

    def plan(self):
        lib = self._library()
        key = (id(lib["trip_angles"]), id(lib["polesCart"]), float(self.angTol), int(self.nband_earlyexit),
               bool(self.simpleqweights), self.device)
        cached_key, plan = self._plan_cache
        if plan is None or cached_key != key:
            if not bool(self.high_fidelity):
                raise NotImplementedError("the device indexer implements the QUEST (high_fidelity) refinement")
            plan = VotePlan(lib, self.angTol, self.nband_earlyexit, self.simpleqweights, device=self.device)
            object.__setattr__(self, "_plan_cache", (key, plan))
        return plan

    def bandindex_device(self, norms, intensity=None, out=None, intermediates=False, stream=None):
        """Device tensors in ([n, nBands, 3] float32 normals, [n, nBands] float32 weights or
        None) -> dict of device tensors (``OUT_NAMES``, plus ``MID_NAMES`` when asked)."""
        import torch
        plan = self.plan()
        norms = norms.to(torch.float32).contiguous()
        n, nb = int(norms.shape[0]), int(norms.shape[1])
        if intensity is not None:
            intensity = intensity.to(torch.float32).contiguous()
            if tuple(intensity.shape) != (n, nb):
                raise ValueError("band_intensity must be [nPats, nBands]")
        if out is None:
            out = alloc_outputs(torch, n, nb, plan.nfam, norms.device, intermediates)
        st = stream if stream is not None else torch.cuda.current_stream(norms.device).cuda_stream
        plan.index_device(norms.data_ptr(), intensity.data_ptr() if intensity is not None else 0, n, nb,
                          {k: v.data_ptr() for k, v in out.items()}, stream=st)
        return out

    def bandindex(self, band_norms, band_intensity=None, band_widths=None, verbose=0):
        """tripletvote.py:492-633 on the device; host arrays in, host arrays out."""
        import torch
        bn = np.asarray(band_norms)
        if bn.ndim == 2:
            bn = bn[np.newaxis, ...]
        n, nb = bn.shape[0], bn.shape[1]
        inten = None
        if band_intensity is not None:
            inten = np.asarray(band_intensity)
            if inten.ndim == 1:
                inten = inten[np.newaxis, ...]
        dev = torch.device("cuda", self.device)
        d_norms = torch.from_numpy(np.ascontiguousarray(bn, np.float32)).to(dev)
        d_int = torch.from_numpy(np.ascontiguousarray(inten, np.float32)).to(dev) if inten is not None else None
        out = self.bandindex_device(d_norms, d_int)
        torch.cuda.current_stream(dev).synchronize()
        h = {k: v.cpu().numpy() for k, v in out.items()}
        return (h["quat"], h["fit"], h["cm"], h["polematch"], h["nmatch"], h["ij"], h["acc_correct"],
                h["bandfit"])


def band_intensity_gpu(mx, normmax, theta, rho, valid, rhomax, stream=None):
    """Band weights for the vote and pq / iq per pattern (_ebsd_index_single.py:751-763) from
    device band fields ([n, nBands] float32; valid int8) -> (adj, pq, iq) device tensors."""
    import torch
    lib = _bind()
    mx, normmax, theta, rho = (t.to(torch.float32).contiguous() for t in (mx, normmax, theta, rho))
    valid = valid.to(torch.int8).contiguous()
    n, nb = int(mx.shape[0]), int(mx.shape[1])
    adj = torch.empty((n, nb), dtype=torch.float32, device=mx.device)
    pq = torch.empty(n, dtype=torch.float32, device=mx.device)
    iq = torch.empty(n, dtype=torch.float32, device=mx.device)
    st = stream if stream is not None else torch.cuda.current_stream(mx.device).cuda_stream
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _lib.check(lib.ebsd_band_intensity(ptr(mx), ptr(normmax), ptr(theta), ptr(rho), ptr(valid), n, nb,
                                       float(np.float32(rhomax)), ptr(adj), ptr(pq), ptr(iq), C.c_void_p(int(st))),
               "ebsd_band_intensity")
    return adj, pq, iq
