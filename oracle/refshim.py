"""Import the reference PyEBSDIndex package (pure Python) with stub numba / matplotlib / h5py.

TEST INFRASTRUCTURE ONLY.  This module is used by ``tests/golden/make_golden.py`` (which
generates the committed golden vectors) and by CPU tests that skip when the reference
source tree is absent.  It is never imported by the product package, by ``bench.py`` or by
the GPU tests.

The reference modules on the band-detection path (``band_detect.py``, ``radon_fast.py``,
``nlpar_cpu.py``, ``tripletvote.py``, ``rotlib.py``) decorate their loops with ``numba.jit``
and ``numba.prange``; numba is not installed here, so a stub package makes ``jit`` return
the plain Python function and ``prange`` the builtin ``range``.  The numeric results are
then those of the reference's own Python source (float32 arrays, float32 accumulators where
the source declares them), only slower.  matplotlib and h5py are only touched by debug
plotting and HDF5 persistence, so empty stand-ins suffice.
"""
from __future__ import annotations

import os
import sys
import types
import warnings

import numpy as np

# the reference source tree is named by the environment only; without it the callers skip
REFERENCE_ROOT = os.environ.get("PYEBSDINDEX_REFERENCE", "")

_loaded = None


def reference_available() -> bool:
    return bool(REFERENCE_ROOT) and os.path.isfile(os.path.join(REFERENCE_ROOT, "pyebsdindex", "band_detect.py"))


def _make_numba_stub() -> types.ModuleType:
    numba = types.ModuleType("numba")

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]

        def deco(f):
            return f

        return deco

    numba.jit = jit
    numba.njit = jit
    numba.prange = range
    for name in ("float32", "float64", "int32", "int64", "uint64", "complex128"):
        setattr(numba, name, getattr(np, name))
    numba.boolean = np.bool_
    numba.get_num_threads = lambda: 1
    numba.set_num_threads = lambda n: None

    typed = types.ModuleType("numba.typed")

    class _Dict:
        @staticmethod
        def empty(key_type=None, value_type=None):
            return {}

    typed.Dict = _Dict
    numba.typed = typed

    core = types.ModuleType("numba.core")
    ctypes_ = types.ModuleType("numba.core.types")
    ctypes_.float32 = np.float32
    ctypes_.uint64 = np.uint64
    core.types = ctypes_
    numba.core = core
    return numba


def _make_mpl_stub() -> tuple[types.ModuleType, types.ModuleType]:
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")

    def _unavailable(*a, **k):
        raise RuntimeError("matplotlib is not available in this environment")

    plt.figure = _unavailable
    plt.imshow = _unavailable
    plt.imread = _unavailable
    mpl.pyplot = plt
    return mpl, plt


def _make_h5py_stub() -> types.ModuleType:
    h5py = types.ModuleType("h5py")

    class Dataset:  # isinstance() target only
        pass

    class Group:
        pass

    class File:
        def __init__(self, *a, **k):
            raise RuntimeError("h5py is not available in this environment")

    h5py.Dataset = Dataset
    h5py.Group = Group
    h5py.File = File
    return h5py


def load():
    """Return a namespace with the reference modules needed by the golden generator."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not reference_available():
        raise RuntimeError(f"reference source not found under {REFERENCE_ROOT}")

    numba = _make_numba_stub()
    sys.modules.setdefault("numba", numba)
    sys.modules.setdefault("numba.typed", numba.typed)
    sys.modules.setdefault("numba.core", numba.core)
    sys.modules.setdefault("numba.core.types", numba.core.types)
    try:
        import matplotlib  # noqa: F401
    except ImportError:
        mpl, plt = _make_mpl_stub()
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = plt
    try:
        import h5py  # noqa: F401
    except ImportError:
        sys.modules["h5py"] = _make_h5py_stub()

    # band_detect.py / radon_fast.py create ~/.pyebsdindex/numbacache at import time.
    # Point HOME at a git-ignored scratch directory for the duration of the import.
    here = os.path.dirname(os.path.abspath(__file__))
    scratch_home = os.path.join(here, "_ref", "home")
    os.makedirs(scratch_home, exist_ok=True)
    old_home = os.environ.get("HOME")
    os.environ["HOME"] = scratch_home
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    try:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            from pyebsdindex import band_detect, radon_fast, nlpar_cpu  # type: ignore
            from pyebsdindex import _ebsd_index_single, rotlib, tripletvote  # type: ignore
    finally:
        if old_home is None:
            os.environ.pop("HOME", None)
        else:
            os.environ["HOME"] = old_home

    ns = types.SimpleNamespace(
        band_detect=band_detect,
        radon_fast=radon_fast,
        nlpar_cpu=nlpar_cpu,
        ebsd_index_single=_ebsd_index_single,
        rotlib=rotlib,
        tripletvote=tripletvote,
    )
    _loaded = ns
    return ns


def find_bands(bd, pats, **kw):
    """Run the reference CPU ``find_bands`` with numpy overflow warnings silenced.

    ``_grey_dilation`` (band_detect.py:811-843) mixes uint64 window half-widths with Python
    ints; without numba this wraps inside the outermost ``k`` rows/columns of the padded
    Radon, which lie in the padding that ``rdn_local_max`` masks out (band_detect.py:661-663).
    """
    with warnings.catch_warnings(), np.errstate(all="ignore"):
        warnings.simplefilter("ignore")
        return bd.find_bands(pats, **kw)


class _ScalarSlotArray(np.ndarray):
    """An ndarray that accepts a one-element array where one element goes, as numpy < 2.x did
    (numpy 2.5 raises "setting an array element with a sequence")."""

    def __setitem__(self, key, value):
        if isinstance(value, np.ndarray) and value.size == 1 and np.ndim(np.asarray(self)[key]) == 0:
            value = value.reshape(())[()]
        super().__setitem__(key, value)


class _LegacyNumpy(types.ModuleType):
    """numpy as seen by a reference module whose arrays take one-element arrays into scalar
    slots: ``zeros`` returns _ScalarSlotArray views, everything else is numpy's own."""

    def __init__(self):
        super().__init__("numpy")

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def zeros(*a, **k):
        return np.zeros(*a, **k).view(_ScalarSlotArray)


def pattern_module():
    """The reference's ebsd_pattern module (ebsd_pattern.py) with the numpy shim above:
    EBSPFile.read_header stores the one-element arrays np.fromfile returns into scalar slots
    (ebsd_pattern.py:884-887), which numpy 2.5 refuses."""
    import importlib
    load()
    mod = importlib.import_module("pyebsdindex.ebsd_pattern")
    if not isinstance(mod.np, _LegacyNumpy):
        mod.np = _LegacyNumpy()
    return mod
