"""ctypes binding of libebsdgpu.so (the C ABI declared in include/ebsdgpu.h).

The shared library is built in-tree (``pyebsdindex_gb300/libebsdgpu.so``) by
``pyebsdindex_gb300/_build.py``.  There is no CPU fallback: if the library or a CUDA device is
missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libebsdgpu.so")

EBSD_U8, EBSD_U16, EBSD_F32 = 0, 1, 2
EBSD_PLAIN_F32, EBSD_PLAIN_F64, EBSD_FUSED_F32, EBSD_FUSED_F16 = 0, 1, 2, 3
EBSD_E_UNSUPPORTED = -5  # include/ebsdgpu.h

METHODS = {
    "plain": EBSD_PLAIN_F32, "plain32": EBSD_PLAIN_F32, "plain_f32": EBSD_PLAIN_F32,
    "plain64": EBSD_PLAIN_F64, "fp64": EBSD_PLAIN_F64, "plain_f64": EBSD_PLAIN_F64,
    "fused": EBSD_FUSED_F32, "fused32": EBSD_FUSED_F32, "fused_f32": EBSD_FUSED_F32,
    "fused16": EBSD_FUSED_F16, "fused_f16": EBSD_FUSED_F16,
}

DTYPES = {np.dtype(np.uint8): EBSD_U8, np.dtype(np.uint16): EBSD_U16, np.dtype(np.float32): EBSD_F32}


class PlanDesc(C.Structure):
    _fields_ = [
        ("H", C.c_int32), ("W", C.c_int32), ("nTheta", C.c_int32), ("nRho", C.c_int32),
        ("nBands", C.c_int32), ("pad_rho", C.c_int32), ("pad_theta", C.c_int32),
        ("peak_rho", C.c_int32), ("peak_theta", C.c_int32), ("ksz_rho", C.c_int32),
        ("ksz_theta", C.c_int32), ("kernel", C.POINTER(C.c_float)), ("lut_len", C.c_int32),
        ("lut", C.POINTER(C.c_int64)), ("rdnmask", C.POINTER(C.c_uint8)),
        ("theta", C.POINTER(C.c_float)), ("rho", C.POINTER(C.c_float)),
        ("background", C.POINTER(C.c_double)), ("background_f32", C.c_int32),
    ]


class TileInfo(C.Structure):
    _fields_ = [("tile", C.c_int), ("patterns_per_pass", C.c_int), ("slabs", C.c_int),
                ("slab_columns", C.c_int), ("slabs_min", C.c_int), ("slabs_max", C.c_int),
                ("single_fits", C.c_int), ("slabs_fp16", C.c_int)]


class Bands(C.Structure):
    _fields_ = [
        ("max", C.c_void_p), ("normmax", C.c_void_p), ("maxloc", C.c_void_p), ("avemax", C.c_void_p),
        ("aveloc", C.c_void_p), ("width", C.c_void_p), ("theta", C.c_void_p), ("rho", C.c_void_p),
        ("valid", C.c_void_p),
    ]


BAND_FIELDS = ("max", "normmax", "maxloc", "avemax", "aveloc", "width", "theta", "rho", "valid")

_lib = None
_lock = threading.Lock()


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libebsdgpu.so not found at {LIB_PATH}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` or "
                "`python pyebsdindex_gb300/_build.py`")
        lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        lib.ebsd_plan_create.argtypes = [C.POINTER(PlanDesc), C.c_int, C.POINTER(P)]
        lib.ebsd_plan_create.restype = C.c_int
        lib.ebsd_plan_destroy.argtypes = [P]
        lib.ebsd_plan_destroy.restype = C.c_int
        lib.ebsd_method_supported.argtypes = [P, C.c_int]
        lib.ebsd_method_supported.restype = C.c_int
        lib.ebsd_method_supported_for.argtypes = [P, C.c_int, C.c_int]
        lib.ebsd_method_supported_for.restype = C.c_int
        lib.ebsd_plan_reserve.argtypes = [P, C.c_int, C.c_int64]
        lib.ebsd_plan_reserve.restype = C.c_int
        lib.ebsd_find_bands.argtypes = [P, C.c_int, C.c_int, P, C.c_int64, C.POINTER(Bands), C.c_int64, P]
        lib.ebsd_find_bands.restype = C.c_int
        lib.ebsd_find_bands_mixed.argtypes = [C.POINTER(P), C.c_int, C.c_int, C.POINTER(P), C.POINTER(C.c_int64),
                                              C.POINTER(Bands), P]
        lib.ebsd_find_bands_mixed.restype = C.c_int
        lib.ebsd_find_bands_host.argtypes = [P, C.c_int, C.c_int, P, C.c_int64, C.POINTER(Bands), C.c_int64]
        lib.ebsd_find_bands_host.restype = C.c_int
        lib.ebsd_find_bands_host_records.argtypes = [P, C.c_int, C.c_int, P, C.c_int64, P, C.c_int32,
                                                     C.POINTER(C.c_int32), C.c_int64]
        lib.ebsd_find_bands_host_records.restype = C.c_int
        lib.ebsd_find_bands_file_records.argtypes = [P, C.c_int, C.c_char_p, C.c_int, C.c_int64, C.c_int64, P,
                                                     C.c_int32, C.POINTER(C.c_int32), C.c_int64]
        lib.ebsd_find_bands_file_records.restype = C.c_int
        lib.ebsd_last_launch_count.argtypes = [P]
        lib.ebsd_last_launch_count.restype = C.c_int64
        lib.ebsd_plan_autotune.argtypes = [P, C.c_int, C.c_int, P, C.c_int64, P, C.POINTER(C.c_int)]
        lib.ebsd_plan_autotune.restype = C.c_int
        lib.ebsd_plan_set_host_input.argtypes = [P, C.c_int]
        lib.ebsd_plan_set_host_input.restype = C.c_int
        lib.ebsd_plan_host_input_in_place.argtypes = [P]
        lib.ebsd_plan_host_input_in_place.restype = C.c_int
        lib.ebsd_plan_set_patterns_per_pass.argtypes = [P, C.c_int]
        lib.ebsd_plan_set_patterns_per_pass.restype = C.c_int
        lib.ebsd_plan_get_tile.argtypes = [P, C.POINTER(TileInfo)]
        lib.ebsd_plan_get_tile.restype = C.c_int
        lib.ebsd_plan_set_tile.argtypes = [P, C.c_int, C.c_int]
        lib.ebsd_plan_set_tile.restype = C.c_int
        lib.ebsd_strerror.argtypes = [C.c_int]
        lib.ebsd_strerror.restype = C.c_char_p
        lib.ebsd_version.argtypes = []
        lib.ebsd_version.restype = C.c_char_p
        _lib = lib
        return lib


def version() -> str:
    """The library's version string (ebsd_version)."""
    return load().ebsd_version().decode()


def check(code: int, what: str = "ebsdgpu"):
    if code != 0:
        msg = load().ebsd_strerror(code).decode()
        raise RuntimeError(f"{what} failed: {msg} (code {code})")
    return code


def method_id(method) -> int:
    if isinstance(method, int):
        return method
    try:
        return METHODS[str(method).lower()]
    except KeyError:
        raise ValueError(f"unknown method {method!r}; choose from {sorted(METHODS)}") from None


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class DevicePlan:
    """Owns one ``ebsd_plan_t`` built from a band-detect plan's host arrays."""

    def __init__(self, *, H, W, nTheta, nRho, nBands, padding, peakPad, kernel, lut, rdnmask, theta,
                 rho, background=None, device=0):
        lib = load()
        self._lib = lib
        kernel = np.ascontiguousarray(kernel, dtype=np.float32)
        lut = np.ascontiguousarray(lut, dtype=np.int64)
        rdnmask = np.ascontiguousarray(rdnmask, dtype=np.uint8)
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        rho = np.ascontiguousarray(rho, dtype=np.float32)
        bg_f32 = 0
        if background is not None:
            bg_f32 = 1 if np.asarray(background).dtype == np.float32 else 0
            background = np.ascontiguousarray(np.broadcast_to(np.asarray(background, dtype=np.float64),
                                                              (H, W)))
        d = PlanDesc()
        d.H, d.W, d.nTheta, d.nRho, d.nBands = int(H), int(W), int(nTheta), int(nRho), int(nBands)
        d.pad_rho, d.pad_theta = int(padding[0]), int(padding[1])
        d.peak_rho, d.peak_theta = int(peakPad[0]), int(peakPad[1])
        d.ksz_rho, d.ksz_theta = int(kernel.shape[-2]), int(kernel.shape[-1])
        d.kernel = _fptr(kernel)
        d.lut_len = int(lut.shape[-1])
        d.lut = lut.ctypes.data_as(C.POINTER(C.c_int64))
        d.rdnmask = rdnmask.ctypes.data_as(C.POINTER(C.c_uint8))
        d.theta = _fptr(theta)
        d.rho = _fptr(rho)
        d.background = background.ctypes.data_as(C.POINTER(C.c_double)) if background is not None else None
        d.background_f32 = bg_f32
        h = C.c_void_p()
        check(lib.ebsd_plan_create(C.byref(d), int(device), C.byref(h)), "ebsd_plan_create")
        self.handle = h
        self.H, self.W, self.nBands = int(H), int(W), int(nBands)
        self.device = int(device)

    def supported(self, method, dtype=None) -> bool:
        """Whether ``method`` can run this plan (for input of ``dtype``, an EBSD_* code, if given)."""
        if dtype is None:
            return self._lib.ebsd_method_supported(self.handle, method_id(method)) == 1
        return self._lib.ebsd_method_supported_for(self.handle, method_id(method), int(dtype)) == 1

    def reserve(self, method, max_chunk):
        check(self._lib.ebsd_plan_reserve(self.handle, method_id(method), int(max_chunk)), "ebsd_plan_reserve")

    def last_launches(self) -> int:
        return int(self._lib.ebsd_last_launch_count(self.handle))

    def set_patterns_per_pass(self, ppp: int):
        """Pin the fused kernel's patterns per block pass (1, 2, 4, 8; 0 = rule)."""
        check(self._lib.ebsd_plan_set_patterns_per_pass(self.handle, int(ppp)), "ebsd_plan_set_patterns_per_pass")

    def get_tile(self) -> dict:
        """The Radon tile shape FP32 fused calls take (``ebsd_plan_get_tile``): ``tile`` 1 one
        tile, 2 theta slabs, 0 neither; ``patterns_per_pass`` (0 = rule), ``slabs`` (the slab
        tables' count), ``slab_columns``, ``slabs_min`` / ``slabs_max``, ``single_fits``."""
        t = TileInfo()
        check(self._lib.ebsd_plan_get_tile(self.handle, C.byref(t)), "ebsd_plan_get_tile")
        return {f: int(getattr(t, f)) for f, _ in TileInfo._fields_}

    def set_tile(self, tile: int, slabs: int = 0):
        """Pin the Radon tile shape: ``tile`` 1 one tile, 2 theta slabs, 0 the rule; ``slabs``
        the slab count (0 = the widest that fit).  A new slab count rebuilds the slab tables
        (the device is synchronised and the old tables freed): capture CUDA graphs after it."""
        check(self._lib.ebsd_plan_set_tile(self.handle, int(tile), int(slabs)), "ebsd_plan_set_tile")

    def set_host_input(self, mode: int):
        """Pinned host input: -1 read in place on coherent CPU-GPU links (default), 0 copy, 1 in place."""
        check(self._lib.ebsd_plan_set_host_input(self.handle, int(mode)), "ebsd_plan_set_host_input")

    def host_input_in_place(self) -> bool:
        r = self._lib.ebsd_plan_host_input_in_place(self.handle)
        if r < 0:
            check(r, "ebsd_plan_host_input_in_place")
        return r == 1

    def autotune(self, pats_ptr: int, dtype: int, n: int, method, stream=0) -> int:
        """Time the record-identical kernel variants (Radon tile shapes: one tile with 1, 2, 4
        or 8 patterns per block pass, theta slabs of several widths) on a device-resident sample
        and keep the fastest in the plan; returns the chosen patterns per block pass (1, 2, 4 or
        8; 1 for slabs).  ``get_tile()`` reads the chosen shape."""
        ppp = C.c_int(0)
        check(self._lib.ebsd_plan_autotune(self.handle, method_id(method), int(dtype), C.c_void_p(int(pats_ptr)),
                                           int(n), C.c_void_p(int(stream)), C.byref(ppp)), "ebsd_plan_autotune")
        return int(ppp.value)

    def find_bands_host(self, pats: np.ndarray, method, chunk=0):
        """Host patterns [n,H,W] -> dict of host SoA band arrays (C ABI with host buffers)."""
        dt = DTYPES.get(pats.dtype)
        if dt is None:
            raise TypeError(f"unsupported pattern dtype {pats.dtype}")
        pats = np.ascontiguousarray(pats)
        n = pats.shape[0]
        out = alloc_host_bands(n, self.nBands)
        b = bands_struct(out)
        check(self._lib.ebsd_find_bands_host(self.handle, method_id(method), dt, C.c_void_p(pats.ctypes.data),
                                             n, C.byref(b), int(chunk)), "ebsd_find_bands_host")
        return out

    def find_bands_host_records(self, pats: np.ndarray, method, rec_dtype, chunk=0):
        """Host patterns [n,H,W] -> (n, nBands) record array of ``rec_dtype`` (the reference's
        BandDetect.dataType): the records are packed by the library while the GPU runs."""
        dt = DTYPES.get(pats.dtype)
        if dt is None:
            raise TypeError(f"unsupported pattern dtype {pats.dtype}")
        pats = np.ascontiguousarray(pats)
        n = pats.shape[0]
        rec = np.empty((n, self.nBands), dtype=rec_dtype)
        offs = record_offsets(rec_dtype)
        check(self._lib.ebsd_find_bands_host_records(self.handle, method_id(method), dt, C.c_void_p(pats.ctypes.data),
                                                     n, C.c_void_p(rec.ctypes.data), rec_dtype.itemsize, offs,
                                                     int(chunk)), "ebsd_find_bands_host_records")
        return rec

    def find_bands_file_records(self, path: str, pat_start: int, n: int, method, rec_dtype, chunk=0):
        """Patterns [pat_start, pat_start + n) of a UP1 / UP2, .ebsp or .pat file -> record array."""
        rec = np.empty((n, self.nBands), dtype=rec_dtype)
        offs = record_offsets(rec_dtype)
        check(self._lib.ebsd_find_bands_file_records(self.handle, method_id(method), str(path).encode(), 0,
                                                     int(pat_start), int(n), C.c_void_p(rec.ctypes.data),
                                                     rec_dtype.itemsize, offs, int(chunk)),
              "ebsd_find_bands_file_records")
        return rec

    def find_bands_device(self, pats_ptr: int, dtype: int, n: int, out_ptrs: dict, method, chunk=0, stream=0):
        """Device patterns -> device SoA outputs (raw pointers), asynchronous on `stream`."""
        b = Bands(**{k: C.c_void_p(int(out_ptrs[k])) for k in BAND_FIELDS})
        check(self._lib.ebsd_find_bands(self.handle, method_id(method), int(dtype), C.c_void_p(int(pats_ptr)),
                                        int(n), C.byref(b), int(chunk), C.c_void_p(int(stream))),
              "ebsd_find_bands")

    @staticmethod
    def find_bands_mixed(plans, dtype: int, pats_ptrs, counts, out_ptrs, stream=0):
        """One persistent launch over several plans' device patterns (mixed pattern sizes):
        plans[k] detects counts[k] patterns at pats_ptrs[k] into the device arrays out_ptrs[k]
        (dicts of raw pointers), the FP32 fused method in theta slabs.  Asynchronous."""
        lib = load()
        k = len(plans)
        hp = (C.c_void_p * k)(*[p.handle.value for p in plans])
        pp = (C.c_void_p * k)(*[int(x) for x in pats_ptrs])
        nn = (C.c_int64 * k)(*[int(x) for x in counts])
        bb = (Bands * k)(*[Bands(**{f: C.c_void_p(int(o[f])) for f in BAND_FIELDS}) for o in out_ptrs])
        check(lib.ebsd_find_bands_mixed(hp, k, int(dtype), pp, nn, bb, C.c_void_p(int(stream))),
              "ebsd_find_bands_mixed")

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self._lib.ebsd_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def record_offsets(rec_dtype):
    """Byte offsets of the nine band fields in a record dtype, in BAND_FIELDS order (checked
    to be float32, pairs of float32 for maxloc / aveloc, int8 for valid)."""
    want = {"maxloc": (np.float32, (2,)), "aveloc": (np.float32, (2,)), "valid": (np.int8, ())}
    offs = (C.c_int32 * 9)()
    for i, f in enumerate(BAND_FIELDS):
        ft, off = rec_dtype.fields[f][:2]
        base, shape = want.get(f, (np.float32, ()))
        if ft.base != np.dtype(base) or ft.shape != shape:
            raise TypeError(f"record field {f!r} has type {ft}, expected {np.dtype(base)}{shape}")
        offs[i] = off
    return offs


def alloc_host_bands(n, nB):
    return {
        "max": np.empty((n, nB), np.float32), "normmax": np.empty((n, nB), np.float32),
        "maxloc": np.empty((n, nB, 2), np.float32), "avemax": np.empty((n, nB), np.float32),
        "aveloc": np.empty((n, nB, 2), np.float32), "width": np.empty((n, nB), np.float32),
        "theta": np.empty((n, nB), np.float32), "rho": np.empty((n, nB), np.float32),
        "valid": np.empty((n, nB), np.int8),
    }


def bands_struct(arrs):
    return Bands(**{k: C.c_void_p(arrs[k].ctypes.data) for k in BAND_FIELDS})
