"""ctypes wrapper of oracle/c/bandcpu.c, the C/OpenMP restatement of the reference find_bands.

TEST / BENCHMARK INFRASTRUCTURE ONLY: used by tests/ (as a second oracle) and by bench.py's
CPU-baseline leg (the timed CPU port).  Built in-tree into ``oracle/c/libbandcpu.so`` with gcc.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c", "bandcpu.c")
LIB = os.path.join(HERE, "c", "libbandcpu.so")

_lib = None


class _Plan(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("H", "W", "nTheta", "nRho", "nB", "p0", "p1", "pk0", "pk1", "k0", "k1", "L")] + [
        ("kernel", C.c_void_p), ("lut", C.c_void_p), ("rdnmask", C.c_void_p), ("theta", C.c_void_p),
        ("rho", C.c_void_p), ("bg", C.c_void_p)]


class _Out(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho",
                                          "valid")]


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
        _lib.bandcpu_find_bands.argtypes = [C.POINTER(_Plan), C.c_void_p, C.c_int, C.c_int64, C.POINTER(_Out), C.c_int]
        _lib.bandcpu_find_bands.restype = C.c_int
    return _lib


def find_bands(plan, pats, threads=0):
    """Run the C restatement with an ``oracle.band_oracle.Plan``; returns a dict of band fields."""
    lib = load()
    if pats.ndim == 2:
        pats = pats[None]
    pats = np.ascontiguousarray(pats)
    dt = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.float32): 2}.get(pats.dtype)
    if dt is None:
        pats = pats.astype(np.float32)
        dt = 2
    n = pats.shape[0]
    nB = plan.nBands
    lut = np.ascontiguousarray(np.where(plan.lut < plan.nPx, plan.lut, -1).astype(np.int32))
    kern = np.ascontiguousarray(plan.kernel, dtype=np.float32)
    rmask = np.ascontiguousarray(plan.rdnmask.astype(np.uint8))
    th = np.ascontiguousarray(plan.theta.astype(np.float64))
    rh = np.ascontiguousarray(plan.rho.astype(np.float64))
    bg = None if plan.background is None else np.ascontiguousarray(np.asarray(plan.background, dtype=np.float64))
    P = _Plan(int(plan.patDim[0]), int(plan.patDim[1]), plan.nTheta, plan.nRho, nB, int(plan.padding[0]),
              int(plan.padding[1]), int(plan.peakPad[0]), int(plan.peakPad[1]), kern.shape[0], kern.shape[1],
              lut.shape[-1], kern.ctypes.data, lut.ctypes.data, rmask.ctypes.data, th.ctypes.data, rh.ctypes.data,
              None if bg is None else bg.ctypes.data)
    out = {"max": np.empty((n, nB), np.float32), "normmax": np.empty((n, nB), np.float32),
           "maxloc": np.empty((n, nB, 2), np.float32), "avemax": np.empty((n, nB), np.float32),
           "aveloc": np.empty((n, nB, 2), np.float32), "width": np.empty((n, nB), np.float32),
           "theta": np.empty((n, nB), np.float32), "rho": np.empty((n, nB), np.float32),
           "valid": np.empty((n, nB), np.int8)}
    o = _Out(**{k: v.ctypes.data for k, v in out.items()})
    rc = lib.bandcpu_find_bands(C.byref(P), pats.ctypes.data, dt, n, C.byref(o), int(threads))
    if rc != 0:
        raise RuntimeError(f"bandcpu_find_bands failed ({rc})")
    return out
