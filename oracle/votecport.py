"""ctypes wrapper of oracle/c/votecpu.c, the C/OpenMP restatement of the reference's triplet
voting (BandIndexer.bandindex, tripletvote.py:492-633).

TEST / BENCHMARK INFRASTRUCTURE ONLY: used by tests/ (as a second oracle) and by bench.py's
indexing CPU-baseline leg (the timed multi-core CPU port).  Built in-tree into
``oracle/c/libvotecpu.so`` with gcc.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c", "votecpu.c")
LIB = os.path.join(HERE, "c", "libvotecpu.so")

_lib = None


class _Lib(C.Structure):
    _fields_ = [("nfam", C.c_int), ("ntrip", C.c_int), ("npoles", C.c_int), ("early", C.c_int),
                ("simpleq", C.c_int), ("tol", C.c_double)] + [
        (n, C.c_void_p) for n in ("trip_angles", "trip_family", "lut", "poles", "pfam", "angtab", "famcnt",
                                  "famidx")]


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB + ".tmp", SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed: " + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.votecpu_bandindex.argtypes = [C.POINTER(_Lib), C.c_void_p, C.c_void_p, C.c_int64, C.c_int] + \
            [C.c_void_p] * 8 + [C.c_int]
        _lib.votecpu_bandindex.restype = C.c_int
        _lib.votecpu_threads.restype = C.c_int
    return _lib


def threads():
    return int(load().votecpu_threads())


def bandindex(lib, params, norms, inten=None, threads=0):
    """(quat, fit, cm, polematch, nmatch, ij, acc_correct, bandfit) for a library dict and
    parameters as oracle.vote_oracle.load_case returns them."""
    L = load()
    keep = {
        "ta": np.ascontiguousarray(lib["trip_angles"], np.float64),
        "tf": np.ascontiguousarray(lib["trip_familyid"], np.int64),
        "lut": np.ascontiguousarray(lib["lut"], np.int64).ravel(),
        "po": np.ascontiguousarray(lib["polesCart"], np.float64),
        "pf": np.ascontiguousarray(lib["familyid"], np.int32),
        "at": np.ascontiguousarray(lib["angTable"], np.float64),
        "fc": np.ascontiguousarray(lib["nFamily"], np.int32),
        "fi": np.ascontiguousarray(lib["famIndex"], np.int64),
    }
    d = _Lib(int(lib["nfam"]), keep["ta"].shape[0], keep["po"].shape[0], int(params["nband_earlyexit"]),
             int(bool(params["simpleqweights"])), float(params["angTol"]),
             *(keep[k].ctypes.data for k in ("ta", "tf", "lut", "po", "pf", "at", "fc", "fi")))
    nrm = np.ascontiguousarray(norms, np.float32)
    if nrm.ndim == 2:
        nrm = nrm[None]
    n, nb = nrm.shape[:2]
    w = None if inten is None else np.ascontiguousarray(inten, np.float32).reshape(n, nb)
    out = (np.empty((n, 4)), np.empty(n), np.empty(n, np.float32), np.empty((n, nb), np.int64),
           np.empty(n, np.int64), np.empty((n, 4), np.int64), np.empty(n, np.int32), np.empty((n, nb)))
    rc = L.votecpu_bandindex(C.byref(d), nrm.ctypes.data, None if w is None else w.ctypes.data, n, nb,
                             *(o.ctypes.data for o in out), int(threads))
    if rc != 0:
        raise RuntimeError(f"votecpu_bandindex failed ({rc})")
    return out
